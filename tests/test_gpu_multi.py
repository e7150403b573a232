"""Uneven batches (c_multi_*): instances with different grids, Re and dt in
the same launches, each against the oracle run on its own; and a batch of
equal instances against the single-grid batch path, bit for bit."""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

# (Nx, Ny, Nz, Re, dt)
INSTANCES = [(16, 33, 16, 2000.0, 0.01), (32, 65, 32, 3300.0, 0.005), (16, 33, 16, 3000.0, 0.008),
             (48, 97, 48, 2500.0, 0.004)]
NSTEPS = 3
# tolerance per grid for 3 steps (primal, tangent, adjoint): a few times the
# per-step FP64 noise floor of the oracle itself at that size
TOL = {16: (2e-11, 2e-11, 6e-11), 32: (6e-11, 3e-11, 1e-10), 48: (2e-10, 1e-9, 5e-10)}


def rel(a, b):
    return np.linalg.norm(np.ravel(a - b)) / max(np.linalg.norm(np.ravel(b)), 1e-300)


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _arr(vals, t):
    return (t * len(vals))(*vals)


def _init(cc, inst, ntan, couple):
    n = len(inst)
    rc = cc.lib.c_multi_init(n, _arr([i[0] for i in inst], ctypes.c_int), _arr([i[1] for i in inst], ctypes.c_int),
                             _arr([i[2] for i in inst], ctypes.c_int), _arr([2 * np.pi] * n, ctypes.c_double),
                             _arr([np.pi] * n, ctypes.c_double), _arr([i[3] for i in inst], ctypes.c_double),
                             _arr([2.0] * n, ctypes.c_double), _arr([i[4] for i in inst], ctypes.c_double),
                             NSTEPS, ntan, couple)
    assert rc == 0, cc.c_last_error_message()


def test_uneven_batch_matches_oracle(cc):
    n = len(INSTANCES)
    Cs = [O.synthetic_state(a[0], a[1], a[2], seed=i) for i, a in enumerate(INSTANCES)]
    ICs = [O.synthetic_state(a[0], a[1], a[2], seed=10 + i, laminar=False) for i, a in enumerate(INSTANCES)]
    ACs = [O.synthetic_state(a[0], a[1], a[2], seed=20 + i, laminar=False) for i, a in enumerate(INSTANCES)]
    pack = lambda xs: np.concatenate([x.ravel() for x in xs]).copy()
    C, IC, AC = pack(Cs), pack(ICs), pack(ACs)
    _init(cc, INSTANCES, 1, 0)
    try:
        for i, a in enumerate(INSTANCES):
            assert cc.lib.c_multi_coef_elems(i) == Cs[i].size
        inh = _arr([1], ctypes.c_int)
        assert cc.lib.c_multi_forward(0, NSTEPS, C.ctypes.data, IC.ctypes.data, inh) == 0, cc.c_last_error_message()
        assert cc.lib.c_multi_adjoint(NSTEPS, 0, AC.ctypes.data, 0.5) == 0, cc.c_last_error_message()
        off = 0
        for i, (Nx, Ny, Nz, Re, dt) in enumerate(INSTANCES):
            args = (Nx, Ny, Nz, 2 * np.pi, np.pi, Re, 2.0, dt, NSTEPS)
            port = O.PortChannel(*args)
            c, ic, ac = Cs[i].copy(), ICs[i].copy(), ACs[i].copy()
            port.primal(0, c)
            port.tangent(0, NSTEPS, ic, 1)
            port.adjoint(NSTEPS, 0, ac, 0, 0.5)
            sz = Cs[i].size
            tp, tt, ta = TOL[Nx]
            assert rel(C[off:off + sz].reshape(c.shape), c) <= tp, i
            assert rel(IC[off:off + sz].reshape(c.shape), ic) <= tt, i
            assert rel(AC[off:off + sz].reshape(c.shape), ac) <= ta, i
            out = np.zeros_like(c)
            for k in range(NSTEPS + 1):
                assert cc.lib.c_multi_getsoln(i, k, out.ctypes.data) == 0
                assert rel(out, port.getsoln(k)) <= tp, (i, k)
            off += sz
    finally:
        cc.lib.c_multi_destroy()


def test_equal_instances_match_single_grid_batch_bitwise(cc):
    args = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, NSTEPS)
    nseg = 3
    C = np.stack([O.synthetic_state(*args[:3], seed=s) for s in range(nseg)])
    IC = np.stack([O.synthetic_state(*args[:3], seed=30 + s, laminar=False) for s in range(nseg)])[:, None]
    AC = np.stack([O.synthetic_state(*args[:3], seed=40 + s, laminar=False) for s in range(nseg)])
    inh = _arr([1], ctypes.c_int)
    assert cc.c_init(*args) == 0
    lib = cc.lib
    assert lib.c_batch_init(nseg, 1, 0) == 0
    b = [C.copy(), np.ascontiguousarray(IC.copy()), AC.copy()]
    assert lib.c_batch_forward(0, NSTEPS, b[0].ctypes.data, b[1].ctypes.data, inh) == 0
    assert lib.c_batch_adjoint(NSTEPS, 0, b[2].ctypes.data, 0.7) == 0
    lib.c_batch_destroy()
    _init(cc, [(16, 33, 16, 2000.0, 0.01)] * nseg, 1, 0)
    try:
        m = [C.copy(), np.ascontiguousarray(IC.copy()), AC.copy()]
        assert lib.c_multi_forward(0, NSTEPS, m[0].ctypes.data, m[1].ctypes.data, inh) == 0
        assert lib.c_multi_adjoint(NSTEPS, 0, m[2].ctypes.data, 0.7) == 0
    finally:
        lib.c_multi_destroy()
    for x, y in zip(m, b):
        assert np.array_equal(x, y)
