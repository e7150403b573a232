"""GPU parity of the batched segment API (c_batch_*), the path the benchmark
times, against the oracle run segment by segment through the reference's
single-trajectory API.

A batch of nseg segments with ntan tangents each is the reference's
sequence primal -> tangent (each tangent, the coupled one last, so MIC is
its trajectory) -> adjoint with ddt coupling (channel/channel.c:399-780),
run independently per segment.  Tolerances are those of test_gpu_parity.py.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

TOL_STEP = 5e-12
TOL_TAN = 1e-11
TOL_ADJ = 3e-11

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 4)
NSEG, NTAN, COUPLE = 3, 3, 2
INHOMO = [0, 0, 1]


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _inputs():
    Nx, Ny, Nz = ARGS[:3]
    C = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=s) for s in range(NSEG)])
    IC = np.stack([np.stack([O.synthetic_state(Nx, Ny, Nz, seed=10 + 3 * s + j, laminar=False)
                             for j in range(NTAN)]) for s in range(NSEG)])
    AC = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=30 + s, laminar=False) for s in range(NSEG)])
    return C, IC, AC


def _reference(C, IC, AC, start, end, strength):
    """Per segment: primal over [0, nsteps], tangents over [start, end] with the
    coupled one last, adjoint from end back to start."""
    outs = []
    order = [j for j in range(NTAN) if j != COUPLE] + [COUPLE]
    for s in range(NSEG):
        ref = O.PortChannel(*ARGS)
        c = C[s].copy()
        ref.primal(0, c)
        ic = IC[s].copy()
        for j in order:
            t = ic[j].copy()
            ref.tangent(start, end, t, INHOMO[j])
            ic[j] = t
        ac = AC[s].copy()
        ref.adjoint(end, start, ac, 0, strength)
        outs.append(dict(ref=ref, IC=ic, AC=ac))
    return outs


def _inh():
    return (ctypes.c_int * NTAN)(*INHOMO)


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("strength", [0.0, 1.0])
def test_batch_host_api(cc, fused, strength):
    n = ARGS[-1]
    C, IC, AC = _inputs()
    assert cc.c_init(*ARGS) == 0, cc.c_last_error_message()
    lib = cc.lib
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0, cc.c_last_error_message()
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        if fused:
            assert lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, _inh()) == 0
        else:
            assert lib.c_batch_primal(0, hC.ctypes.data) == 0
            assert lib.c_batch_tangent(0, n, hIC.ctypes.data, _inh()) == 0
        assert lib.c_batch_adjoint(n, 0, hAC.ctypes.data, strength) == 0
        refs = _reference(C, IC, AC, 0, n, strength)
        out = np.zeros_like(C[0])
        for s in range(NSEG):
            for i in range(n + 1):
                assert lib.c_batch_getsoln(s, i, out.ctypes.data) == 0
                assert rel(out, refs[s]["ref"].getsoln(i)) <= TOL_STEP * max(i, 1), (s, i)
                assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
                assert rel(out, refs[s]["ref"].getincresoln(i)) <= TOL_TAN, (s, i)
            for j in range(NTAN):
                assert rel(hIC[s, j], refs[s]["IC"][j]) <= TOL_TAN, (s, j)
            assert rel(hAC[s], refs[s]["AC"]) <= TOL_ADJ, s
    finally:
        lib.c_batch_destroy()


def test_batch_partial_ranges(cc):
    """Tangent over [1, n-1] on a stored primal and the coupled adjoint back
    over the same range: the coupling reads MIC only where the sweep wrote it."""
    n = ARGS[-1]
    C, IC, AC = _inputs()
    assert cc.c_init(*ARGS) == 0
    lib = cc.lib
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        assert lib.c_batch_primal(0, hC.ctypes.data) == 0
        assert lib.c_batch_tangent(1, n - 1, hIC.ctypes.data, _inh()) == 0
        assert lib.c_batch_adjoint(n - 1, 1, hAC.ctypes.data, 0.7) == 0
        refs = _reference(C, IC, AC, 1, n - 1, 0.7)
        for s in range(NSEG):
            for j in range(NTAN):
                assert rel(hIC[s, j], refs[s]["IC"][j]) <= TOL_TAN, (s, j)
            assert rel(hAC[s], refs[s]["AC"]) <= TOL_ADJ, s
    finally:
        lib.c_batch_destroy()


def test_batch_device_api(cc):
    """c_batch_*_dev on torch CUDA tensors equals the host-array calls."""
    torch = pytest.importorskip("torch")
    n = ARGS[-1]
    C, IC, AC = _inputs()
    assert cc.c_init(*ARGS) == 0
    lib = cc.lib
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        assert lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, _inh()) == 0
        assert lib.c_batch_adjoint(n, 0, hAC.ctypes.data, 1.0) == 0
        dev = torch.device("cuda:0")
        dC = torch.from_numpy(C.view(np.float64)).to(dev)
        dIC = torch.from_numpy(IC.view(np.float64)).to(dev)
        dAC = torch.from_numpy(AC.view(np.float64)).to(dev)
        torch.cuda.synchronize()
        assert lib.c_batch_forward_dev(0, n, dC.data_ptr(), dIC.data_ptr(), _inh()) == 0
        assert lib.c_batch_adjoint_dev(n, 0, dAC.data_ptr(), 1.0) == 0
        assert lib.c_synchronize() == 0
        gIC = dIC.cpu().numpy().view(np.complex128)
        gAC = dAC.cpu().numpy().view(np.complex128)
        assert np.array_equal(gIC, hIC)
        assert np.array_equal(gAC, hAC)
    finally:
        lib.c_batch_destroy()


def test_laminar_start_tangent_and_coupled_adjoint(cc):
    """Laminar start without run-up: the first primal substage runs on the raw
    samples while the tangent and adjoint rebuild MC[0]
    (channel/channel.c:409-422, 496-514)."""
    args = (8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01, 4)
    n = args[-1]
    ref = O.PortChannel(*args)
    O.libc_srand(2)
    ref.primal(0, None)
    assert cc.c_init(*args) == 0
    O.libc_srand(2)
    cc.c_primal(0, np.zeros((0, 0, 0, 0), complex))
    IC0 = O.synthetic_state(*args[:3], seed=3, laminar=False)
    ICg, ICr = IC0.copy(), IC0.copy()
    cc.c_tangent(0, n, ICg, 1)
    ref.tangent(0, n, ICr, 1)
    assert rel(ICg, ICr) <= TOL_TAN
    AC0 = O.synthetic_state(*args[:3], seed=4, laminar=False)
    ACg, ACr = AC0.copy(), AC0.copy()
    cc.c_adjoint(n, 0, ACg, 0, 0.9)
    ref.adjoint(n, 0, ACr, 0, 0.9)
    assert rel(ACg, ACr) <= TOL_ADJ
