"""GPU parity of the Re-sensitivity tangent forcings (c_tangent_forcing and
the batched inhomo values 2 / 3) against the oracle
(oracle/chan_port.c: cport_tangent_forcing), and the exact forcing against
central finite differences of the GPU primal in Re.

Kind 2 reconnects the reference's forcing (channel/tangent_forcing.c,
tangent_forcing0.c, increproject.c:61-104); kind 3 is the exact derivative
of the discrete step, checked here at the finite-difference floor.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 6)
TOL_TAN = 1e-11
# The pure forced response (zero initial tangent) is re^2 times fourth-order
# operators of the primal, which weigh the primal's rounding at high Legendre
# modes: the oracle built with and without FMA contraction differs by
# 1.8e-10 (kind 2) and 2.2e-10 (kind 3) here, against 3.8e-12 with an O(1)
# initial tangent.
TOL_FORCED = 5e-10


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


@pytest.mark.parametrize("kind", [2, 3])
@pytest.mark.parametrize("zero_ic", [True, False])
def test_single_api_matches_oracle(cc, kind, zero_ic):
    n = ARGS[-1]
    port = O.PortChannel(*ARGS)
    C0 = O.synthetic_state(*ARGS[:3], seed=0)
    port.primal(0, C0.copy())
    assert cc.c_init(*ARGS) == 0
    cc.c_primal(0, C0.copy())
    IC0 = np.zeros(port.coef_shape, complex) if zero_ic else O.synthetic_state(*ARGS[:3], seed=3, laminar=False)
    a, b = IC0.copy(), IC0.copy()
    cc.c_tangent_forcing(1, n, a, kind)
    port.tangent_forcing(1, n, b, kind)
    tol = TOL_FORCED if zero_ic else TOL_TAN
    assert rel(a, b) <= tol
    for i in range(2, n + 1):
        assert rel(cc.c_getincresoln(i), port.getincresoln(i)) <= tol, i


def test_batch_mixed_forcings(cc):
    """One batch with tangents forced by Re (exact), Re (reference) and the
    mean flux; fused forward sweep and tangent-only sweep."""
    n = 4
    args = ARGS[:-1] + (n,)
    nseg, inhomo = 2, [3, 2, 1]
    C = np.stack([O.synthetic_state(*args[:3], seed=s) for s in range(nseg)])
    IC = np.stack([np.stack([O.synthetic_state(*args[:3], seed=40 + 3 * s + j, laminar=False)
                             for j in range(3)]) for s in range(nseg)])
    assert cc.c_init(*args) == 0
    lib = cc.lib
    inh = (ctypes.c_int * 3)(*inhomo)
    for fused in (True, False):
        assert lib.c_batch_init(nseg, 3, 2) == 0
        try:
            hC, hIC = C.copy(), IC.copy()
            if fused:
                assert lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, inh) == 0
            else:
                assert lib.c_batch_primal(0, hC.ctypes.data) == 0
                assert lib.c_batch_tangent(0, n, hIC.ctypes.data, inh) == 0
            for s in range(nseg):
                port = O.PortChannel(*args)
                port.primal(0, C[s].copy())
                for j in range(3):
                    t = IC[s, j].copy()
                    port.tangent_forcing(0, n, t, inhomo[j])
                    assert rel(hIC[s, j], t) <= TOL_TAN, (fused, s, j)
        finally:
            lib.c_batch_destroy()


def test_exact_re_forcing_matches_central_differences(cc):
    """d C_n / d Re from the kind-3 tangent against (C_n(Re+h) - C_n(Re-h)) / 2h
    of the GPU primal (h = 0.4 at Re = 2000, where truncation and rounding
    both sit near 1e-8 relative)."""
    n = 3
    args = ARGS[:-1] + (n,)
    C0 = O.synthetic_state(*args[:3], seed=2, amp=5e-2)
    h = 0.4

    def final(Re):
        a = list(args)
        a[5] = Re
        assert cc.c_init(*a) == 0
        C = C0.copy()
        cc.c_primal(0, C)
        return C

    fd = (final(args[5] + h) - final(args[5] - h)) / (2 * h)
    assert cc.c_init(*args) == 0
    cc.c_primal(0, C0.copy())
    tan = np.zeros_like(C0)
    cc.c_tangent_forcing(0, n, tan, 3)
    assert np.linalg.norm(fd) > 0
    assert rel(tan, fd) <= 1e-6
