"""The digit tables of the tensor-core contractions, decoded on the host.

Each fixed matrix is stored as seven balanced base-256 digits per entry
(the top digit in [-256, 256], the others in [-128, 127]) of its rows scaled
to 56-bit integers, in mma.sync m16n8k16 A-fragment order
[row tiles][k-tiles][digit][32 lanes][4 words], with one exponent per row.
The test decodes the fragments back into matrices and compares them with
the matrices themselves: the reconstruction bases from c_setup_table, and
the DFT matrices of the radix-2 inverse transform and of the forward
transforms rebuilt here from their definitions.  No GPU is needed (the
library's table builders are host code).
"""
import ctypes
import math
from pathlib import Path

import numpy as np
import pytest

LIB = Path(__file__).resolve().parent.parent / "shadow-channel_gb300" / "libc_channel.so"
GRID = (16, 33, 16, 2 * math.pi, math.pi, 2000.0, 2.0, 0.01)


@pytest.fixture(scope="module")
def lib():
    if not LIB.exists():
        import build
        build.build()
    L = ctypes.CDLL(str(LIB))
    L.c_setup_tc_table.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5 + [
        ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p]
    L.c_setup_tc_table.restype = ctypes.c_int
    L.c_setup_table.argtypes = [ctypes.c_int] * 3 + [ctypes.c_double] * 5 + [ctypes.c_int, ctypes.c_void_p,
                                                                             ctypes.c_int]
    L.c_setup_table.restype = ctypes.c_int
    return L


def tc_table(lib, which):
    sizes = (ctypes.c_longlong * 2)()
    assert lib.c_setup_tc_table(*GRID, which, None, 0, None, 0, sizes) == 0
    frag = np.zeros(sizes[0], np.uint32)
    ex = np.zeros(sizes[1], np.int32)
    assert lib.c_setup_tc_table(*GRID, which, frag.ctypes.data, sizes[0], ex.ctypes.data, sizes[1], sizes) == 0
    return frag, ex


def decode(frag, ex, ntab, MT, KT):
    """Matrices [ntab][MT*16][KT*16] from A-fragment digit tables."""
    w = frag.reshape(ntab, MT, KT, 7, 32, 4)
    lo = (w & 0xFFFF).astype(np.uint32) << 16
    hi = w & 0xFFFF0000
    dlo = lo.view(np.float32).astype(np.int64)  # bf16 bits in the upper half of a float
    dhi = hi.view(np.float32).astype(np.int64)
    val = np.zeros((ntab, MT * 16, KT * 16), np.int64)
    lane = np.arange(32)
    g, t = lane >> 2, lane & 3
    for i in range(7):
        scale = 256 ** (6 - i)
        for mt in range(MT):
            for kt in range(KT):
                r0, k0 = mt * 16 + g, kt * 16 + 2 * t
                for word, (dr, dk) in enumerate(((0, 0), (8, 0), (0, 8), (8, 8))):
                    val[:, r0 + dr, k0 + dk] += dlo[:, mt, kt, i, :, word] * scale
                    val[:, r0 + dr, k0 + dk + 1] += dhi[:, mt, kt, i, :, word] * scale
    rows = ex.size // ntab
    e = ex.reshape(ntab, rows).astype(np.float64)
    return val[:, :rows, :].astype(np.float64) * np.exp2(e - 56.0)[:, :, None]


def setup(lib, which, shape):
    n = lib.c_setup_table(*GRID, which, None, 0)
    out = np.zeros(n)
    assert lib.c_setup_table(*GRID, which, out.ctypes.data, n) == n
    return out.reshape(shape)


def close(dec, ref):
    # 56-bit rows: each entry within 2^-56 of its row's scale
    scale = np.abs(ref).max(axis=-1, keepdims=True)
    return np.all(np.abs(dec - ref) <= np.exp2(-55.0) * np.maximum(scale, 1e-300))


def test_reconstruction_bases(lib):
    Nx, Ny, Nz = GRID[:3]
    Q, R, D = 3 * Ny // 2, Ny - 2, Ny - 4
    frag, ex = tc_table(lib, 0)
    MT, KT = (Q + 15) // 16, (R + 15) // 16
    dec = decode(frag, ex, 5, MT, KT)
    for b, (which, cols) in enumerate(((0, D), (1, D), (2, D), (3, R), (4, R))):
        ref = setup(lib, which, (Q, cols))
        assert close(dec[b][:, :cols], ref), b
        assert np.all(dec[b][:, cols:] == 0)


def test_inverse_dft_tables(lib):
    """The radix-2 z stage: rows Re, Im of Z[m < pz/2], K words: the kept kz
    modes of even padded index zp, then the odd ones (cos, -sin of the angle
    2 pi m zp / pz for the real part of each word)."""
    Nx, Ny, Nz = GRID[:3]
    pz, X = 3 * Nz // 2, Nx // 2
    pzh = pz // 2
    zp = [kk if kk < Nz // 2 else kk + 1 + Nz // 2 for kk in range(Nz - 1)]
    modes = [kk for kk in range(Nz - 1) if zp[kk] % 2 == 0] + [kk for kk in range(Nz - 1) if zp[kk] % 2 == 1]
    nE = sum(1 for kk in range(Nz - 1) if zp[kk] % 2 == 0)
    KTE, KTO = (2 * nE + 15) // 16, (2 * (Nz - 1 - nE) + 15) // 16
    frag, ex = tc_table(lib, 2)
    dec = decode(frag, ex, 1, (2 * pzh + 15) // 16, KTE + KTO)[0]
    ref = np.zeros_like(dec)
    for c, lst in enumerate((modes[:nE], modes[nE:])):
        w0 = KTE * 8 if c else 0
        for e, kk in enumerate(lst):
            for m in range(pzh):
                a = 2 * math.pi * ((m * zp[kk]) % pz) / pz
                ref[m, 2 * (w0 + e)], ref[m, 2 * (w0 + e) + 1] = math.cos(a), -math.sin(a)
                ref[pzh + m, 2 * (w0 + e)], ref[pzh + m, 2 * (w0 + e) + 1] = math.sin(a), math.cos(a)
    # the library's twiddles (long double cosl, rounded) against Python's
    # cos within a few ulps; a misplaced entry would be off by O(1)
    assert np.abs(dec - ref).max() <= 4e-15


def test_forward_dft_tables(lib):
    """The forward x stage: rows Re, Im of kx (-sin for Im) times 1/(px pz);
    the z stage: rows Re, Im of the kept modes, K = Re, Im of Y[zp]."""
    Nx, Ny, Nz = GRID[:3]
    px, pz, X = 3 * Nx // 2, 3 * Nz // 2, Nx // 2
    norm = 1.0 / (px * pz)
    frag, ex = tc_table(lib, 4)
    dec = decode(frag, ex, 1, (2 * X + 15) // 16, (px + 15) // 16)[0]
    ref = np.zeros_like(dec)
    for kx in range(X):
        for xp in range(px):
            a = 2 * math.pi * ((kx * xp) % px) / px
            ref[2 * kx, xp], ref[2 * kx + 1, xp] = math.cos(a) * norm, -math.sin(a) * norm
    assert np.abs(dec - ref).max() <= 4e-15 * norm
    frag, ex = tc_table(lib, 6)  # the unscaled copy
    dec_u = decode(frag, ex, 1, (2 * X + 15) // 16, (px + 15) // 16)[0]
    assert np.abs(dec_u * norm - ref).max() <= 4e-15 * norm
    frag, ex = tc_table(lib, 5)
    Kk = Nz - 1
    dec = decode(frag, ex, 1, (2 * Kk + 15) // 16, (2 * pz + 15) // 16)[0]
    ref = np.zeros_like(dec)
    for kk in range(Kk):
        zo = kk if kk < Nz // 2 else kk + 1 + Nz // 2
        for z in range(pz):
            a = 2 * math.pi * ((zo * z) % pz) / pz
            c, ms = math.cos(a), -math.sin(a)
            ref[2 * kk, 2 * z], ref[2 * kk, 2 * z + 1] = c, -ms
            ref[2 * kk + 1, 2 * z], ref[2 * kk + 1, 2 * z + 1] = ms, c
    assert np.abs(dec - ref).max() <= 4e-15


def test_adjoint_tables(lib):
    """Recon^T's bases transposed (rows padded to R) and Quad^T's weighted
    transposes plane-major (columns padded to R)."""
    Nx, Ny, Nz = GRID[:3]
    Q, R, D = 3 * Ny // 2, Ny - 2, Ny - 4
    MTw, KTq = (R + 15) // 16, (Q + 15) // 16
    frag, ex = tc_table(lib, 7)
    dec = decode(frag, ex, 5, MTw, KTq)
    for b, (which, cols) in enumerate(((0, D), (1, D), (2, D), (3, R), (4, R))):
        ref = np.zeros((R, Q))
        ref[:cols] = setup(lib, which, (Q, cols)).T
        assert close(dec[b][:, :Q], ref), b
    frag, ex = tc_table(lib, 8)
    dec = decode(frag, ex, 3, KTq, MTw)
    for b, (which, rows) in enumerate(((6, D), (5, D), (8, R))):  # Wqp, Wq, Wr
        ref = np.zeros((Q, R))
        ref[:, :rows] = setup(lib, which, (rows, Q)).T
        assert close(dec[b][:, :R], ref), b


def test_short_buffer_is_refused(lib):
    """A non-null buffer shorter than its table is an error (-2), not a
    silent success that leaves the caller's memory unwritten; null buffers
    stay a size query."""
    L = lib
    sizes = (ctypes.c_longlong * 2)()
    assert L.c_setup_tc_table(*GRID, 2, None, 0, None, 0, sizes) == 0
    frag = np.full(sizes[0], 7, np.uint32)
    ex = np.full(sizes[1], 7, np.int32)
    assert L.c_setup_tc_table(*GRID, 2, frag.ctypes.data, sizes[0] - 1, ex.ctypes.data, sizes[1], sizes) == -2
    assert L.c_setup_tc_table(*GRID, 2, frag.ctypes.data, sizes[0], ex.ctypes.data, sizes[1] - 1, sizes) == -2
    assert (frag == 7).all() and (ex == 7).all()
    assert L.c_setup_tc_table(*GRID, 2, frag.ctypes.data, sizes[0], None, 0, sizes) == 0
    assert not (frag == 7).all()


def decode_umma(words, ex, rows, K):
    """The tcgen05 inverse's stacked B-operand table back to its matrix:
    k-tile blocks of 7 Np / 8 row groups x 256 bytes, element (row' = i Np
    + r, k) of digit plane i at ((row'/8) 2 + (k%16)/8) 128 + (row'%8) 16
    + (k%8) 2 in its block (8 x 16-byte core matrices, K-major)."""
    b = np.ascontiguousarray(words).view(np.uint8)
    Np = (rows + 15) // 16 * 16
    KT = K // 16
    rg = 7 * Np // 8
    assert b.size == KT * rg * 256
    bits = b.view(np.uint16).astype(np.uint32) << 16
    dig = bits.view(np.float32).astype(np.int64)
    val = np.zeros((Np, K), np.int64)
    for i in range(7):
        for r in range(Np):
            for k in range(K):
                rp = i * Np + r
                off = (((k // 16) * rg + rp // 8) * 2 + (k % 16) // 8) * 128 + (rp % 8) * 16 + (k % 8) * 2
                val[r, k] += dig[off // 2] * 256 ** (6 - i)
    assert np.all(val[rows:] == 0)
    return val[:rows].astype(np.float64) * np.exp2(ex.astype(np.float64) - 56.0)[:, None]


@pytest.mark.parametrize("which, mma_which", [(9, 2), (10, 3)])
def test_tcgen05_tables_decode_to_the_same_matrices(lib, which, mma_which):
    """The stacked tables of the tcgen05 inverse hold, digit for digit, the
    matrices of the mma.sync inverse's tables (same rows, exponents, K order)"""
    Nx, Ny, Nz = GRID[:3]
    pz, px, X = 3 * Nz // 2, 3 * Nx // 2, Nx // 2
    words, ex = tc_table(lib, which)
    frag2, ex2 = tc_table(lib, mma_which)
    assert np.array_equal(ex, ex2)
    if which == 9:
        rows = 2 * (pz // 2)
        nE = sum(1 for kk in range(Nz - 1) if (kk if kk < Nz // 2 else kk + 1 + Nz // 2) % 2 == 0)
        K = ((2 * nE + 15) // 16 + (2 * (Nz - 1 - nE) + 15) // 16) * 16
    else:
        rows = px // 2
        nxE = (X + 1) // 2
        K = ((2 * nxE + 15) // 16 + (2 * (X - nxE) + 15) // 16) * 16
    dec = decode_umma(words, ex, rows, K)
    ref = decode(frag2, ex2, 1, (rows + 15) // 16, K // 16)[0][:rows]
    assert np.array_equal(dec, ref)
