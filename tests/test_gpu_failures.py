"""Failure detection in the batched path, with failures made on the host.

The reference's only runtime fault is the CFL stop (channel/pass1.c:116-138:
pass1 returns ERROR and primal/tangent silently leave the time loop,
channel/channel.c:448-452, 538-542).  The GPU keeps a status word per
segment: bit 0 = CFL stop (that segment's kernels return from then on, its
state stays as the reference leaves it), bit 1 = a non-finite value seen in
a physical field (diagnostic).  c_last_error() returns the OR over the
segments of the last call.

Both tests seed the failure into ONE segment's input on the host and check
that it is reported and that every other segment's results are bit for bit
those of a batch without the failure (segments never mix).  No kernel is
made to fault, trap or hang.
"""
import ctypes

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

ARGS = (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 4)
NSEG, NTAN, COUPLE = 3, 3, 2
INHOMO = [0, 0, 1]
BAD = 1


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


def _run(cc, C, IC, AC, strength=1.0):
    """forward + coupled adjoint of the batch; returns the end states, the
    stored trajectories and the status of each call"""
    n = ARGS[-1]
    lib = cc.lib
    assert cc.c_init(*ARGS) == 0, cc.c_last_error_message()
    assert lib.c_batch_init(NSEG, NTAN, COUPLE) == 0, cc.c_last_error_message()
    try:
        hC, hIC, hAC = C.copy(), IC.copy(), AC.copy()
        inh = (ctypes.c_int * NTAN)(*INHOMO)
        rc = lib.c_batch_forward(0, n, hC.ctypes.data, hIC.ctypes.data, inh)
        st_fwd, cfl_fwd = cc.c_last_error(), cc.c_last_cfl()
        assert rc == st_fwd and rc >= 0, (rc, cc.c_last_error_message())   # the call returns its status
        rc = lib.c_batch_adjoint(n, 0, hAC.ctypes.data, strength)
        st_adj = cc.c_last_error()
        assert rc == st_adj and rc >= 0, (rc, cc.c_last_error_message())
        out = np.zeros(C[0].shape, np.complex128)
        MC, MIC = [], []
        for s in range(NSEG):
            mc, mic = [], []
            for i in range(n + 1):
                assert lib.c_batch_getsoln(s, i, out.ctypes.data) == 0
                mc.append(out.copy())
                assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
                mic.append(out.copy())
            MC.append(np.stack(mc))
            MIC.append(np.stack(mic))
        return dict(C=hC, IC=hIC, AC=hAC, MC=MC, MIC=MIC, st_fwd=st_fwd, st_adj=st_adj, cfl_fwd=cfl_fwd)
    finally:
        lib.c_batch_destroy()
        cc.c_destroy()


def _others_unchanged(got, clean):
    for s in range(NSEG):
        if s == BAD:
            continue
        assert np.array_equal(got["C"][s], clean["C"][s]), s
        assert np.array_equal(got["IC"][s], clean["IC"][s]), s
        assert np.array_equal(got["AC"][s], clean["AC"][s]), s
        assert np.array_equal(got["MC"][s], clean["MC"][s]), s
        assert np.array_equal(got["MIC"][s], clean["MIC"][s]), s


def test_nan_in_one_segment_is_flagged_and_contained(cc):
    C, IC, AC = _inputs()
    clean = _run(cc, C, IC, AC)
    assert clean["st_fwd"] == 0 and clean["st_adj"] == 0
    Cbad = C.copy()
    Cbad[BAD, 1, 0, 2, 1] = complex(np.nan, 0.0)  # one coefficient of one segment's state
    got = _run(cc, Cbad, IC, AC)
    assert got["st_fwd"] & 2, got["st_fwd"]
    assert not got["st_fwd"] & 1   # a NaN never reads as a CFL stop
    assert not np.isfinite(got["C"][BAD]).all()
    _others_unchanged(got, clean)
    # the status is per call: a clean batch afterwards reports nothing
    again = _run(cc, C, IC, AC)
    assert again["st_fwd"] == 0 and again["st_adj"] == 0
    assert np.array_equal(again["AC"], clean["AC"])


def test_cfl_stop_in_one_segment(cc):
    """One segment whose velocity is large enough for CFL >= 2.8 at the first
    substage stops there, as the reference's primal does for that segment
    alone; the others run to the end unchanged."""
    C, IC, AC = _inputs()
    clean = _run(cc, C, IC, AC, strength=0.0)
    Cbad = C.copy()
    Cbad[BAD] *= 40.0
    got = _run(cc, Cbad, IC, AC, strength=0.0)
    assert got["st_fwd"] & 1, got["st_fwd"]
    assert got["cfl_fwd"] >= 2.8
    _others_unchanged(got, clean)
    ref = O.PortChannel(*ARGS)
    Cr = Cbad[BAD].copy()
    assert ref.primal(0, Cr) == -1
    rel = lambda a, b: np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)
    assert rel(got["C"][BAD], Cr) <= 1e-12
    for i in range(ARGS[-1] + 1):
        assert rel(got["MC"][BAD][i], ref.getsoln(i)) <= 1e-12, i
    ref.close()
