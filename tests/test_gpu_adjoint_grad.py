"""Parameter gradients from one exact-adjoint sweep (c_adjoint_exact_grad)
against the forced tangent sweeps they transpose.

For J = <AC, C_n> + sum_{m=0}^{n-1} <src, C_m> (Euclidean inner product of
the real and imaginary parts) and a parameter p whose tangent v_m = dC_m/dp
starts from zero and is driven by the forcing of c_tangent_forcing kind 1
(the mean flux of the reference's inhomogeneous tangent,
channel/increproject0.c:209-214: p = meanU) or kind 3 (the exact Re
derivative of the discrete step: p = Re),
    dJ/dp = <AC, v_n> + sum_m <src, v_m>.
The adjoint sweep gets both from the cotangents of the forcing terms at
every substage.  In exact arithmetic the two sides are equal; in FP64 they
agree to the rounding of the two evaluation orders.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

CASES = [(16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 6), (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 5)]
TOL = 1e-9


def dot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _tangent_sides(cc, n, AC, src, kind):
    v = np.zeros_like(AC)
    cc.c_tangent_forcing(0, n, v, kind)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    return dot(AC, v) + sum(dot(src, cc.c_getincresoln(m)) for m in range(n))


@pytest.mark.parametrize("args", CASES)
def test_grad_matches_forced_tangents(cc, args):
    n = args[-1]
    assert cc.c_init(*args) == 0, cc.c_last_error_message()
    C0 = O.synthetic_state(*args[:3], seed=0)
    cc.c_primal(0, C0.copy())
    AC = O.synthetic_state(*args[:3], seed=11, laminar=False)
    src = O.synthetic_state(*args[:3], seed=12, laminar=False)
    lam = AC.copy()
    gU, gRe = cc.c_adjoint_exact_grad(n, 0, lam, src.copy())
    tU = _tangent_sides(cc, n, AC, src, 1)
    tRe = _tangent_sides(cc, n, AC, src, 3)
    print(f"\n{args[:3]}: dJ/dmeanU adjoint {gU:.15e} tangent {tU:.15e}; dJ/dRe adjoint {gRe:.15e} tangent {tRe:.15e}")
    assert abs(gU - tU) <= TOL * abs(tU), (gU, tU)
    assert abs(gRe - tRe) <= TOL * abs(tRe), (gRe, tRe)
    # the state gradient is the one c_adjoint_exact_source gives, bit for bit
    lam2 = AC.copy()
    cc.c_adjoint_exact_source(n, 0, lam2, src.copy())
    assert np.array_equal(lam, lam2)
    # without a source: J = <AC, C_n>
    lam3 = AC.copy()
    gU0, gRe0 = cc.c_adjoint_exact_grad(n, 0, lam3, None)
    v = np.zeros_like(AC)
    cc.c_tangent_forcing(0, n, v, 3)
    assert abs(gRe0 - dot(AC, v)) <= TOL * abs(dot(AC, v))
    cc.c_destroy()


def test_batched_grad_matches_single(cc):
    torch = pytest.importorskip("torch")
    args = CASES[0]
    n, nseg = args[-1], 3
    Nx, Ny, Nz = args[:3]
    C = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=s) for s in range(nseg)])
    AC = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=20 + s, laminar=False) for s in range(nseg)])
    src = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=40 + s, laminar=False) for s in range(nseg)])
    single = []
    for s in range(nseg):
        assert cc.c_init(*args) == 0
        cc.c_primal(0, C[s].copy())
        single.append(cc.c_adjoint_exact_grad(n, 0, AC[s].copy(), src[s].copy()))
        cc.c_destroy()
    assert cc.c_init(*args) == 0
    lib = cc.lib
    assert lib.c_batch_init(nseg, 0, 0) == 0, cc.c_last_error_message()
    try:
        dev = torch.device("cuda:0")
        dC = torch.from_numpy(C.view(np.float64)).to(dev)
        dAC = torch.from_numpy(AC.view(np.float64)).to(dev)
        dsrc = torch.from_numpy(src.view(np.float64)).to(dev)
        torch.cuda.synchronize()
        assert lib.c_batch_primal_dev(0, dC.data_ptr()) == 0, cc.c_last_error_message()
        grad = np.zeros((nseg, 2))
        rc = lib.c_batch_adjoint_exact_grad_dev(n, 0, dAC.data_ptr(), dsrc.data_ptr(), grad.ctypes.data)
        assert rc == 0, cc.c_last_error_message()
        for s in range(nseg):
            assert abs(grad[s, 0] - single[s][0]) <= 1e-12 * abs(single[s][0]), s
            assert abs(grad[s, 1] - single[s][1]) <= 1e-12 * abs(single[s][1]), s
    finally:
        lib.c_batch_destroy()
        cc.c_destroy()
