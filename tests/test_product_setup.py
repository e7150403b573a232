"""The product's host-side setup tables equal the reference's bit for bit.

Quadrature nodes and weights, basis values, weighted transposes and banded
Gram matrices (channel/LegendreSetup.c:25-527, channel/RsQs.c:55-174) are
built by the product library on the host (no GPU needed) and compared with
the oracle port, which is itself pinned bit-exact to the reference.
"""
import ctypes
from pathlib import Path

import numpy as np
import pytest

import oracle as O

LIB = Path(__file__).resolve().parent.parent / "shadow-channel_gb300" / "libc_channel.so"


@pytest.fixture(scope="module")
def lib():
    if not LIB.exists():
        import build
        build.build()
    L = ctypes.CDLL(str(LIB))
    L.c_setup_table.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5 + [ctypes.c_int, ctypes.c_void_p,
                                                                             ctypes.c_int]
    L.c_setup_table.restype = ctypes.c_int
    return L


def table(lib, args, which):
    n = lib.c_setup_table(*args, which, None, 0)
    assert n > 0
    out = np.zeros(n)
    assert lib.c_setup_table(*args, which, out.ctypes.data, n) == n
    return out


@pytest.mark.parametrize("grid", [(8, 9, 8), (16, 33, 16), (32, 65, 32), (48, 97, 48)])
def test_tables_bitwise(lib, grid):
    args = (*grid, 2 * np.pi, np.pi, 3300.0, 2.0, 0.005)
    port = O.PortChannel(*args, 1)
    y, w = port.quad()
    assert np.array_equal(table(lib, args, 15), y)
    assert np.array_equal(table(lib, args, 16), w)
    for which in range(15):
        ref = port.table(which).ravel()
        got = table(lib, args, which)
        assert np.array_equal(got, ref), which


def test_rejects_reference_invalid_sizes(lib):
    assert lib.c_setup_table(10, 9, 8, 1.0, 1.0, 100.0, 2.0, 0.01, 0, None, 0) == -1
    assert lib.c_setup_table(8, 9, 7, 1.0, 1.0, 100.0, 2.0, 0.01, 0, None, 0) == -1
