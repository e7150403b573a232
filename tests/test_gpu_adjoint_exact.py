"""The exact discrete adjoint on the GPU (c_adjoint_exact, c_batch_adjoint_exact,
c_multi_adjoint_exact): the transpose of the homogeneous tangent step.

- Dot-product identity on the GPU alone: <lambda, T v> = <T^T lambda, v> with
  T v from c_tangent(inhomo 0) and T^T lambda from c_adjoint_exact, over
  several steps: 1e-10 relative on a correlated pair lambda = T v + noise,
  and 1e-12 of |lambda| |T v| for an independent lambda (both sides are FP64
  evaluations of one bilinear form; the oracle's own sweeps agree to
  4e-16 .. 3e-13 of the norm product).
- Parity with the oracle's transpose (oracle/chan_port.c,
  cport_adjoint_exact) on the same inputs, held to the tangent tolerance of
  test_gpu_parity.py (1e-11).
- A laminar start without run-up, where the tangent linearises about a
  re-advanced primal rather than the stored one.
- The batched, device-array and uneven-batch entry points.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

TOL_DOT = 1e-10
TOL_PAR = 1e-11


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


def dot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def nrm(a):
    return float(np.linalg.norm(a.ravel()))


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _dot_checks(cc, n, v, lam):
    Tv = v.copy()
    cc.c_tangent(0, n, Tv, 0)
    Tl = lam.copy()
    cc.c_adjoint_exact(n, 0, Tl)
    assert cc.c_last_error() == 0, cc.c_last_error_message()
    lhs, rhs = dot(lam, Tv), dot(Tl, v)
    assert abs(lhs - rhs) <= 1e-12 * nrm(lam) * nrm(Tv), (lhs, rhs)
    lam2 = Tv + 0.1 * lam * (nrm(Tv) / nrm(lam))
    Tl2 = lam2.copy()
    cc.c_adjoint_exact(n, 0, Tl2)
    lhs2, rhs2 = dot(lam2, Tv), dot(Tl2, v)
    assert abs(lhs2 - rhs2) <= TOL_DOT * abs(lhs2), (lhs2, rhs2)
    return Tl


@pytest.mark.parametrize("args", [
    (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 4),
    (12, 17, 24, 2 * np.pi, np.pi, 1000.0, 2.0, 0.01, 3),
])
def test_dot_product_identity_and_oracle(cc, args):
    n = args[-1]
    C0 = O.synthetic_state(*args[:3], seed=0)
    v = O.synthetic_state(*args[:3], seed=5, laminar=False)
    lam = O.synthetic_state(*args[:3], seed=6, laminar=False)
    assert cc.c_init(*args) == 0, cc.c_last_error_message()
    cc.c_primal(0, C0.copy())
    Tl = _dot_checks(cc, n, v, lam)
    port = O.PortChannel(*args)
    port.primal(0, C0.copy())
    ref = lam.copy()
    assert port.adjoint_exact(n, 0, ref) == 0
    assert rel(Tl, ref) <= TOL_PAR
    # a partial range on the same stored trajectory
    Tl2 = lam.copy()
    cc.c_adjoint_exact(n - 1, 1, Tl2)
    ref2 = lam.copy()
    assert port.adjoint_exact(n - 1, 1, ref2) == 0
    assert rel(Tl2, ref2) <= TOL_PAR


def test_laminar_start_without_run_up(cc):
    """The tangent rebuilds MC[0] and re-advances the primal from it
    (channel/channel.c:496-514); the transpose re-advances it too."""
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 3)
    n = args[-1]
    assert cc.c_init(*args) == 0
    O.libc_srand(2)
    cc.c_primal(0, np.zeros((0, 0, 0, 0), complex))
    v = O.synthetic_state(*args[:3], seed=3, laminar=False)
    lam = O.synthetic_state(*args[:3], seed=4, laminar=False)
    Tl = _dot_checks(cc, n, v, lam)
    port = O.PortChannel(*args)
    O.libc_srand(2)
    port.primal(0, None)
    ref = lam.copy()
    assert port.adjoint_exact(n, 0, ref) == 0
    assert rel(Tl, ref) <= TOL_PAR


def test_batch_and_device_api(cc):
    torch = pytest.importorskip("torch")
    args = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 3)
    n, nseg = args[-1], 3
    Nx, Ny, Nz = args[:3]
    C = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=s) for s in range(nseg)])
    AC = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=30 + s, laminar=False) for s in range(nseg)])
    assert cc.c_init(*args) == 0
    lib = cc.lib
    assert lib.c_batch_init(nseg, 1, 0) == 0, cc.c_last_error_message()
    try:
        hC, hAC = C.copy(), AC.copy()
        assert lib.c_batch_primal(0, hC.ctypes.data) == 0
        assert lib.c_batch_adjoint_exact(n, 0, hAC.ctypes.data) == 0, cc.c_last_error_message()
        for s in range(nseg):
            port = O.PortChannel(*args)
            port.primal(0, C[s].copy())
            ref = AC[s].copy()
            assert port.adjoint_exact(n, 0, ref) == 0
            assert rel(hAC[s], ref) <= TOL_PAR, s
        dAC = torch.from_numpy(AC.view(np.float64).copy()).to("cuda:0")
        torch.cuda.synchronize()
        assert lib.c_batch_adjoint_exact_dev(n, 0, dAC.data_ptr()) == 0
        assert lib.c_synchronize() == 0
        assert np.array_equal(dAC.cpu().numpy().view(np.complex128), hAC)
        assert lib.c_batch_adjoint_exact(0, 0, hAC.ctypes.data) == -4
    finally:
        lib.c_batch_destroy()


def test_uneven_batch(cc):
    """c_multi_adjoint_exact on two grids equals the single-grid call on each."""
    grids = [(16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01), (12, 17, 24, 2 * np.pi, np.pi, 1000.0, 2.0, 0.008)]
    n = 2
    lib = cc.lib
    I = lambda v: (ctypes.c_int * 2)(*v)
    D = lambda v: (ctypes.c_double * 2)(*v)
    col = lambda j: [g[j] for g in grids]
    states = [O.synthetic_state(*g[:3], seed=i) for i, g in enumerate(grids)]
    lams = [O.synthetic_state(*g[:3], seed=10 + i, laminar=False) for i, g in enumerate(grids)]
    singles = []
    for g, c0, l0 in zip(grids, states, lams):
        assert cc.c_init(*g, n) == 0
        cc.c_primal(0, c0.copy())
        l = l0.copy()
        cc.c_adjoint_exact(n, 0, l)
        singles.append(l)
    assert lib.c_multi_init(2, I(col(0)), I(col(1)), I(col(2)), D(col(3)), D(col(4)), D(col(5)), D(col(6)),
                            D(col(7)), n, 1, 0) == 0, cc.c_last_error_message()
    try:
        flatC = np.concatenate([c.ravel() for c in states])
        assert lib.c_multi_primal(0, flatC.ctypes.data) == 0
        flatL = np.concatenate([l.ravel() for l in lams])
        assert lib.c_multi_adjoint_exact(n, 0, flatL.ctypes.data) == 0, cc.c_last_error_message()
        off = 0
        for l, ref in zip(lams, singles):
            got = flatL[off:off + l.size].reshape(l.shape)
            off += l.size
            assert rel(got, ref) <= 1e-13
    finally:
        lib.c_multi_destroy()
