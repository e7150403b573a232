"""Kernel variants the autotuner chooses among give the same bits.

The implicit solve's block tile (kx columns per block: 16 or 8, and 8 in
128-thread blocks; CHN_SOLVE_TILE=16, 8, 8/128) changes which columns share
a block, not any column's arithmetic.  The builds of the tensor-core inverse transform
(CHN_INVERSE_BUILD: 2 = two fields per pass in 256-thread blocks at two
blocks per SM, 3 = the same at three, 4 / 5 = one field per pass in
128-thread blocks at four / five, 6 / 7 = builds 4 / 2 compiled for the
sizes of 32x65x32 and 16x33x16, 8 / 9 = one field per pass in 192-thread
blocks at three, run-time / compiled sizes, 10 / 11 / 12 = one field per
pass compiled for the sizes in 128 / 192 / 256-thread blocks at five / four
/ three) change how the columns of a plane are
grouped, not the digit sums or their rounding; nor do the builds of the
products, reconstruction and solve kernels (and the exact adjoint's
transposed solve) compiled for those sizes (CHN_FIXED_SIZES=1), nor the adjoint products' planes per pass (1 or 3,
CHN_ADJ_PRODUCTS_PER_PASS; the reference adjoint and the exact one), nor
the reconstruction's build (CHN_RECON_BUILD: 0 = 16 columns in 256-thread
blocks at two per SM, 1 = 8 columns in 128-thread blocks at four, 2 = 16
columns at three without the table prefetch), nor the products' build
(CHN_PRODUCTS_BUILD: 1 = two product planes per pass at three blocks per
SM), nor the concurrent branches of a substage (CHN_CONCURRENT_CHAINS: the
primal and tangent chains of a forward substage and the adjoint's two
product passes on two streams, or one).  Each variant runs the
batched forward (primal + 3 tangents, one forced), the coupled adjoint
and the exact adjoint, and the single-trajectory primal, and must reproduce the default's outputs
bit for bit.  Grids: 32x65x32 (the benchmarked one), 16x33x16 (both with
compiled-size builds) and 48x97x48 (run-time sizes; 24 kx columns: 16 + 8
or three tiles of 8 in the solve).
"""
import ctypes
import json
import os

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

GRIDS = [(32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005, 3), (48, 97, 48, 2 * np.pi, np.pi, 3300.0, 2.0, 0.004, 2),
         (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01, 3)]
NSEG, NTAN = 2, 3
KNOBS = ("CHN_SOLVE_TILE", "CHN_INVERSE_BUILD", "CHN_FIXED_SIZES", "CHN_ADJ_PRODUCTS_PER_PASS", "CHN_RECON_BUILD",
         "CHN_PRODUCTS_BUILD", "CHN_AUTOTUNE", "CHN_CONCURRENT_CHAINS", "CHN_NO_FIELD_CACHE")


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


def _sweeps(cc, args, env):
    old = {k: os.environ.get(k) for k in KNOBS}
    for k in KNOBS:
        os.environ.pop(k, None)
    os.environ.update(env)
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
            AX = AC.copy()
            assert lib.c_batch_adjoint(n, 0, AC.ctypes.data, 1.0) == 0, cc.c_last_error_message()
            assert lib.c_batch_adjoint_exact(n, 0, AX.ctypes.data) == 0, cc.c_last_error_message()
            out = np.zeros(C[0].shape, np.complex128)
            traj = []
            for s in range(NSEG):
                for i in range(n + 1):
                    assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
                    traj.append(out.copy())
        finally:
            lib.c_batch_destroy()
        single = O.synthetic_state(Nx, Ny, Nz, seed=99)
        cc.c_primal(0, single)   # the single-trajectory engine takes the variants of c_init
        cc.c_destroy()
        return [C, IC, AC, AX, np.stack(traj), single], report
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _same(a, b):
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.float64), y.view(np.float64))


@pytest.mark.parametrize("gi,tile", [(0, "8"), (0, "8/128"), (1, "8"), (1, "8/128"), (2, "8/128")])
def test_solve_tiles_give_the_same_bits(cc, gi, tile):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_SOLVE_TILE": "16"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_SOLVE_TILE": tile})
    _same(a, b)


@pytest.mark.parametrize("gi,build", [(0, "3"), (0, "4"), (0, "5"), (0, "6"), (0, "7"), (0, "8"), (0, "9"),
                                      (0, "10"), (0, "11"), (0, "12"), (2, "4"), (2, "6"), (2, "7"), (2, "9"),
                                      (2, "12"), (1, "4"), (1, "8")])
def test_inverse_builds_give_the_same_bits(cc, gi, build):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_INVERSE_BUILD": "2", "CHN_AUTOTUNE": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_INVERSE_BUILD": build, "CHN_AUTOTUNE": "0"})
    _same(a, b)


@pytest.mark.parametrize("gi", [0, 2])
def test_fixed_size_builds_give_the_same_bits(cc, gi):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_FIXED_SIZES": "0", "CHN_AUTOTUNE": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_FIXED_SIZES": "1", "CHN_AUTOTUNE": "0"})
    _same(a, b)


@pytest.mark.parametrize("gi", [0, 2])
def test_adjoint_products_per_pass_give_the_same_bits(cc, gi):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_ADJ_PRODUCTS_PER_PASS": "1", "CHN_AUTOTUNE": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_ADJ_PRODUCTS_PER_PASS": "3", "CHN_AUTOTUNE": "0"})
    _same(a, b)


@pytest.mark.parametrize("gi,build,fixed", [(0, "1", "1"), (0, "1", "0"), (2, "1", "1"), (0, "2", "1"), (0, "2", "0"),
                                            (2, "2", "1"), (1, "1", "0"), (1, "2", "0")])
def test_recon_builds_give_the_same_bits(cc, gi, build, fixed):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_RECON_BUILD": "0", "CHN_AUTOTUNE": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_RECON_BUILD": build, "CHN_FIXED_SIZES": fixed, "CHN_AUTOTUNE": "0"})
    _same(a, b)


@pytest.mark.parametrize("gi,fixed", [(0, "1"), (0, "0"), (2, "1"), (1, "0")])
def test_products_builds_give_the_same_bits(cc, gi, fixed):
    a, _ = _sweeps(cc, GRIDS[gi], {"CHN_PRODUCTS_BUILD": "0", "CHN_AUTOTUNE": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {"CHN_PRODUCTS_BUILD": "1", "CHN_FIXED_SIZES": fixed, "CHN_AUTOTUNE": "0"})
    _same(a, b)


@pytest.mark.parametrize("gi,cache", [(0, "1"), (1, "1"), (2, "1"), (0, "0"), (2, "0")])
def test_concurrent_chains_give_the_same_bits(cc, gi, cache):
    """with and without the primal field cache (without it the primal's
    fields share one buffer across substages, read by both branches)"""
    env = {"CHN_AUTOTUNE": "0", "CHN_NO_FIELD_CACHE": "1" if cache == "0" else "0"}
    a, _ = _sweeps(cc, GRIDS[gi], {**env, "CHN_CONCURRENT_CHAINS": "0"})
    b, _ = _sweeps(cc, GRIDS[gi], {**env, "CHN_CONCURRENT_CHAINS": "1"})
    _same(a, b)


def test_autotuner_reports_its_choices(cc):
    res, report = _sweeps(cc, GRIDS[0], {})
    if "solve_chosen" not in report:
        pytest.skip("autotuner off (CHN_AUTOTUNE=0)")
    assert report["solve_chosen"] in ("tile16", "tile8", "tile8_t128")
    assert report["solve_tile16"] > 0 and report["solve_tile8"] > 0
    assert report["chosen"].startswith("tc_inverse_")
    for b in ("f2_b2", "f2_b3", "f1_b4", "f1_b5", "f1_b4_fixed", "f2_b2_fixed", "f1_t192_b3", "f1_t192_b3_fixed"):
        assert report["tc_inverse_" + b] > 0
    for part in ("products", "recon", "solve"):
        assert report[part + "_sizes"] in ("runtime", "fixed") and report[part + "_fixed_sizes"] > 0
    assert report["adjoint_products_per_pass"] in (1, 3)
    assert report["recon_build"] in (0, 1, 2)
    assert report["products_build"] in (0, 1)
    ref, _ = _sweeps(cc, GRIDS[0], {"CHN_SOLVE_TILE": "16", "CHN_INVERSE_BUILD": "2", "CHN_AUTOTUNE": "0"})
    _same(res, ref)
