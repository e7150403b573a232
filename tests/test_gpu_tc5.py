"""The inverse transforms on tcgen05 (k_phys_inverse_tc5) against the
mma.sync kernel (k_phys_inverse_tc).

Both compute each output as the once-rounded exact sum of the same 56-bit
digit products (the same tables, row exponents and column scaling), so the
outputs must agree bit for bit whatever the order in which the tensor cores
add the products.  CHN_INVERSE_TC5=0 at c_init selects the mma.sync kernel.
Covered: the three-field path (spec2phys), the six-field path of the
batched forward sweep (primal and tangents, every stored step), a column
holding a NaN (NaN out of that column only), and the grids the kernel
serves (16x33x16, 32x65x32; 8x9x8 with its small tables).
"""
import ctypes
import os

import numpy as np
import pytest

import oracle as O
from conftest import has_gpu

pytestmark = pytest.mark.gpu

GRIDS = [(8, 9, 8, 2 * np.pi, np.pi, 500.0, 2.0, 0.01), (16, 33, 16, 2 * np.pi, np.pi, 2000.0, 2.0, 0.01),
         (32, 65, 32, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005)]


@pytest.fixture(scope="module")
def cc():
    if not has_gpu():
        pytest.skip("no CUDA device")
    from channel import c_channel
    return c_channel


class _kernel:
    """CHN_INVERSE_TC5 set for the next c_init"""

    def __init__(self, on):
        self.on = on

    def __enter__(self):
        self.old = os.environ.get("CHN_INVERSE_TC5")
        os.environ["CHN_INVERSE_TC5"] = "1" if self.on else "0"

    def __exit__(self, *exc):
        if self.old is None:
            os.environ.pop("CHN_INVERSE_TC5", None)
        else:
            os.environ["CHN_INVERSE_TC5"] = self.old


def _spec2phys(cc, grid, on, states):
    with _kernel(on):
        assert cc.c_init(*grid, 1) == 0, cc.c_last_error_message()
    Nx, Ny, Nz = grid[:3]
    out = []
    for C in states:
        f = np.zeros((3, 3 * Nx // 2, 3 * Ny // 2, 3 * Nz // 2))
        cc.c_spec2phys(np.ascontiguousarray(C), f)
        out.append(f)
    err = cc.c_last_error()
    cc.c_destroy()
    return out, err


@pytest.mark.parametrize("gi", range(len(GRIDS)))
def test_spec2phys_bit_identical(cc, gi):
    grid = GRIDS[gi]
    states = [O.synthetic_state(*grid[:3], seed=s) for s in (1, 2)]
    a, ea = _spec2phys(cc, grid, True, states)
    b, eb = _spec2phys(cc, grid, False, states)
    assert ea == 0 and eb == 0
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.int64), y.view(np.int64))


def test_nan_column_stays_in_its_column(cc):
    grid = GRIDS[1]
    C = O.synthetic_state(*grid[:3], seed=3)
    C[2, 1, 4, 3] = complex(np.nan, 0.0)    # kz = 2, beta, n = 4, kx = 3
    a, _ = _spec2phys(cc, grid, True, [C])
    b, _ = _spec2phys(cc, grid, False, [C])
    assert np.isnan(a[0]).any()
    assert np.array_equal(np.isnan(a[0]), np.isnan(b[0]))
    fin = ~np.isnan(b[0])
    assert np.array_equal(a[0][fin].view(np.int64), b[0][fin].view(np.int64))


def _batch(cc, grid, on, nseg=3, ntan=3, n=4):
    Nx, Ny, Nz = grid[:3]
    C = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=s) for s in range(nseg)])
    IC = np.stack([np.stack([O.synthetic_state(Nx, Ny, Nz, seed=10 + 3 * s + j, laminar=False)
                             for j in range(ntan)]) for s in range(nseg)])
    AC = np.stack([O.synthetic_state(Nx, Ny, Nz, seed=30 + s, laminar=False) for s in range(nseg)])
    with _kernel(on):
        assert cc.c_init(*grid, n) == 0, cc.c_last_error_message()
    lib = cc.lib
    assert lib.c_batch_init(nseg, ntan, ntan - 1) == 0, cc.c_last_error_message()
    try:
        inh = (ctypes.c_int * ntan)(*([0] * (ntan - 1) + [1]))
        assert lib.c_batch_forward(0, n, C.ctypes.data, IC.ctypes.data, inh) == 0, cc.c_last_error_message()
        assert lib.c_batch_adjoint(n, 0, AC.ctypes.data, 1.0) == 0, cc.c_last_error_message()
        out = np.zeros(C[0].shape, np.complex128)
        traj = []
        for s in range(nseg):
            for i in range(n + 1):
                assert lib.c_batch_getsoln(s, i, out.ctypes.data) == 0
                traj.append(out.copy())
                assert lib.c_batch_getincresoln(s, i, out.ctypes.data) == 0
                traj.append(out.copy())
        return C, IC, AC, np.stack(traj)
    finally:
        lib.c_batch_destroy()
        cc.c_destroy()


@pytest.mark.parametrize("gi", [1, 2])
def test_batched_sweeps_bit_identical(cc, gi):
    a = _batch(cc, GRIDS[gi], True)
    b = _batch(cc, GRIDS[gi], False)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.int64), y.view(np.int64))


def test_tc5_kernel_is_the_one_timed(cc):
    """at 32x65x32 the six-field inverse of the batch runs on tcgen05 (its
    per-launch time differs from the mma.sync kernel's), and the error word of
    its bounded waits stays clear"""
    grid = GRIDS[2]
    times = {}
    for on in (True, False):
        with _kernel(on):
            assert cc.c_init(*grid, 2) == 0
        assert cc.lib.c_batch_init(8, 3, 2) == 0
        times[on] = cc.lib.c_batch_kernel_ms(1, 3)
        cc.lib.c_batch_destroy()
        cc.c_destroy()
    print(f"\nphys_inverse per 24-instance launch: tcgen05 {times[True]:.3f} ms, mma.sync {times[False]:.3f} ms")
    assert times[True] > 0 and times[False] > 0
    assert cc.c_last_error() == 0
