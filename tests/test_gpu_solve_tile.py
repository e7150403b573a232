"""The implicit solve's block tile (kx columns per block: 16 or 8), which
the autotuner picks per batch, changes which columns share a block but no
column's arithmetic: the batched sweeps give the same bits with either
tile.  CHN_SOLVE_TILE fixes the tile at c_init / c_batch_init.  Grids:
32x65x32 (16 kx columns: one tile of 16 or two of 8) and 48x97x48 (24
columns: 16 + 8 or three of 8).
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

GRIDS = [(32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 3), (48, 97, 48, 2 * np.pi, np.pi, 3300.0, 2.0, 0.004, 2)]
NSEG, NTAN = 2, 3


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _sweeps(cc, args, tile):
    old = os.environ.get("CHN_SOLVE_TILE")
    if tile is None:
        os.environ.pop("CHN_SOLVE_TILE", None)
    else:
        os.environ["CHN_SOLVE_TILE"] = str(tile)
    try:
        n = args[-1]
        Nx, Ny, Nz = args[:3]
        C = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=s) for s in range(NSEG)])
        IC = np.stack([np.stack([O.synthetic_state(Nx, Ny, Nz, seed=10 + 3 * s + j, laminar=False)
                                 for j in range(NTAN)]) for s in range(NSEG)])
        AC = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=30 + s, laminar=False) for s in range(NSEG)])
        assert cc.c_init(*args) == 0, cc.c_last_error_message()
        lib = cc.lib
        assert lib.c_batch_init(NSEG, NTAN, NTAN - 1) == 0, cc.c_last_error_message()
        report = json.loads(lib.c_autotune_report().decode() or "{}")
        try:
            inh = (ctypes.c_int * NTAN)(0, 0, 1)
            assert lib.c_batch_forward(0, n, C.ctypes.data, IC.ctypes.data, inh) == 0, cc.c_last_error_message()
            assert lib.c_batch_adjoint(n, 0, AC.ctypes.data, 1.0) == 0, cc.c_last_error_message()
            out = np.zeros(C[0].shape, np.complex128)
            traj = []
            for s in range(NSEG):
                for i in range(n + 1):
                    assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
                    traj.append(out.copy())
        finally:
            lib.c_batch_destroy()
        single = O.synthetic_state(Nx, Ny, Nz, seed=99)
        cc.c_primal(0, single)   # the single-trajectory engine takes the tile of c_init
        cc.c_destroy()
        return [C, IC, AC, np.stack(traj), single], report
    finally:
        if old is None:
            os.environ.pop("CHN_SOLVE_TILE", None)
        else:
            os.environ["CHN_SOLVE_TILE"] = old


@pytest.mark.parametrize("gi", [0, 1])
def test_solve_tiles_give_the_same_bits(cc, gi):
    a, _ = _sweeps(cc, GRIDS[gi], 16)
    b, _ = _sweeps(cc, GRIDS[gi], 8)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.float64), y.view(np.float64))


def test_autotuner_reports_the_solve_tile(cc):
    res, report = _sweeps(cc, GRIDS[0], None)
    if "solve_chosen" not in report:
        pytest.skip("autotuner off (CHN_AUTOTUNE=0)")
    assert report["solve_chosen"] in ("tile16", "tile8")
    assert report["solve_tile16"] > 0 and report["solve_tile8"] > 0
    ref, _ = _sweeps(cc, GRIDS[0], 16)
    for x, y in zip(res, ref):
        assert np.array_equal(x.view(np.float64), y.view(np.float64))
