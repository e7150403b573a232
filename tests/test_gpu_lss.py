"""GPU parity of the device LSS operator (channel/lss.py, c_lss_*) against the
reference's LSS driver layer restated on the oracle (oracle/lss_oracle.py:
drivers/wrapper.py's Wrapper.matvec and drivers/pariter.py's par_minres over
one stored primal trajectory split into time segments).

Tolerances: the matvec chains ddt_project (whose V - r dC/dt cancellation
has a floor near 3.5e-11), tangents (1e-11) and coupled adjoints (3e-11);
the KKT residual is held to 1e-9 relative, zeta to 1e-9, MINRES iterates to
1e-7 (the Lanczos recurrences amplify the operator's differences).
"""
import numpy as np
import pytest

import oracle as O
from conftest import has_gpu
from lss_oracle import Wrapper, par_minres

pytestmark = pytest.mark.gpu

NSEG, L = 3, 2
ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, NSEG * L)


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


@pytest.fixture(scope="module")
def setup():
    if not has_gpu():
        pytest.skip("no CUDA device")
    pytest.importorskip("torch")
    from channel import c_channel as cc
    from channel.lss import KKT
    port = O.PortChannel(*ARGS)
    C0 = O.synthetic_state(*ARGS[:3], seed=0)
    port.primal(0, C0.copy())
    nb = [L * i for i in range(NSEG + 1)]
    starts = np.stack([port.getsoln(nb[i]).copy() for i in range(NSEG)])
    assert cc.c_init(*ARGS) == 0, cc.c_last_error_message()
    kkt = KKT(starts, L)
    wr = Wrapper(port, nb)
    yield kkt, wr
    kkt.close()


def _vector(wr, seed):
    parts = [O.synthetic_state(*ARGS[:3], seed=seed + j, laminar=False, amp=1e-3) for j in range(2 * NSEG - 1)]
    return np.concatenate([p.ravel() for p in parts]).view(np.float64).copy()


@pytest.mark.parametrize("inhomo", [0, 1])
def test_kkt_matvec(setup, inhomo):
    kkt, wr = setup
    x = _vector(wr, 100)
    y_gpu = kkt.matvec(x, inhomo)
    z_gpu = kkt.zeta.copy()
    y_ref = wr.matvec(x, inhomo)
    assert rel(y_gpu, y_ref) <= 1e-9
    assert np.allclose(z_gpu, wr.zeta, rtol=1e-9, atol=1e-12 * np.abs(wr.zeta).max())


def test_kkt_rhs_and_dot(setup):
    kkt, wr = setup
    b_gpu = kkt.rhs()
    zero = np.zeros(kkt.size)
    b_ref = -wr.matvec(zero, 1) - wr.matvec(zero, 0)
    assert rel(b_gpu, b_ref) <= 1e-9
    assert abs(kkt.dot(b_gpu, b_gpu) - float(np.dot(b_ref, b_ref))) <= 1e-8 * float(np.dot(b_ref, b_ref))


def test_minres_iterates(setup):
    kkt, wr = setup
    b = -wr.matvec(np.zeros(kkt.size), 1) - wr.matvec(np.zeros(kkt.size), 0)
    x_ref, (info_r, it_r) = par_minres(lambda v: wr.matvec(v, 0), b, np.zeros_like(b), np.dot, tol=1e-30,
                                       maxiter=3)
    x_gpu, (info_g, it_g) = kkt.minres(b, tol=1e-30, maxiter=3)
    assert (info_g, it_g) == (info_r, it_r) == (1, 3)
    assert rel(x_gpu, x_ref) <= 1e-7
