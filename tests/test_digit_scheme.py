"""The exact digit-GEMM scheme of the tensor-core contractions, modelled on
the host (tc_common.cuh): operands scaled to 56-bit integers, seven balanced
base-256 digits, level sums of digit products accumulated in FP32 in chunks
of at most 7 k-tiles (112 terms), folded into 64-bit integers (H, L) and
rounded once.  The model checks, against exact rational arithmetic, that
every FP32 partial sum of a chunk is an integer below 2^24 (so FP32 holds it
exactly), that the folded integers are the exact sum of the kept levels, and
that the rounded result is within one unit in the last place of the exact
dot product of the 56-bit operands (plus the dropped levels' bound).
"""
import math
from fractions import Fraction

import numpy as np

K_CHUNK = 112


def scaled56(v, ex):
    """round(v * 2^(56 - ex)) for |v| < 2^ex (ties away from zero)."""
    if v == 0.0:
        return 0
    m = Fraction(v) * Fraction(2) ** (56 - ex)
    s = 1 if m > 0 else -1
    return s * int(abs(m) + Fraction(1, 2))


def digits(x):
    """Balanced base-256 digits d0..d6 of |x| < 2^56, most significant first."""
    xb = x + 0x808080808080
    lo = xb & 0xFFFFFFFF
    hi = (xb >> 32) & 0xFFFFFFFF
    d = [0] * 7
    d[6], d[5], d[4], d[3] = [((lo >> (8 * k)) & 255) - 128 for k in range(4)]
    d[2], d[1] = [((hi >> (8 * k)) & 255) - 128 for k in range(2)]
    d[0] = xb >> 48
    assert sum(v * 256 ** (6 - i) for i, v in enumerate(d)) == x
    assert -256 <= d[0] <= 256 and all(-128 <= v <= 127 for v in d[1:])
    return d


def contract(a, b):
    """Exact level sums of sum_j a_j b_j as the kernels form them; returns
    the rounded value and the exact value of the kept levels."""
    ea = math.frexp(max(abs(v) for v in a))[1]
    eb = math.frexp(max(abs(v) for v in b))[1]
    ia = [scaled56(v, ea) for v in a]
    ib = [scaled56(v, eb) for v in b]
    da = [digits(x) for x in ia]
    db = [digits(x) for x in ib]
    H = L = 0
    for c0 in range(0, len(a), K_CHUNK):
        acc = np.zeros(7, np.float32)
        for j in range(c0, min(len(a), c0 + K_CHUNK)):
            for i in range(7):
                for k in range(7 - i):
                    acc[i + k] = np.float32(acc[i + k] + np.float32(da[j][i] * db[j][k]))
                    assert abs(float(acc[i + k])) < 2 ** 24  # every partial sum exact in FP32
        lv = [int(v) for v in acc]
        H += (lv[0] << 16) + (lv[1] << 8) + lv[2]
        L += (lv[3] << 24) + (lv[4] << 16) + (lv[5] << 8) + lv[6]
    kept = Fraction(H * 2 ** 32 + L) * Fraction(2) ** (ea + eb - 64)
    exact56 = sum(Fraction(x) * y for x, y in zip(ia, ib)) * Fraction(2) ** (ea + eb - 112)
    return float(kept), kept, exact56, ea, eb, len(a)


def test_digits_cover_the_range():
    rng = np.random.default_rng(0)
    for x in [0, 1, -1, 2 ** 56 - 1, -(2 ** 56) + 1, 0x7F7F7F7F7F7F7F, -0x808080808080]:
        digits(x)
    for x in rng.integers(-(2 ** 56) + 1, 2 ** 56, size=2000, dtype=np.int64):
        digits(int(x))


def test_contraction_is_faithful():
    rng = np.random.default_rng(1)
    for n, spread in ((16, 0), (97, 3), (128, 8), (250, 20)):
        a = (rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))).tolist()
        b = (rng.standard_normal(n) * np.exp2(rng.integers(-spread, spread + 1, n))).tolist()
        v, kept, exact56, ea, eb, _ = contract(a, b)
        # the dropped levels (i + k >= 7) lie below n * 28 * 2^(-56) of the scale
        scale = Fraction(2) ** (ea + eb)
        assert abs(kept - exact56) <= n * 28 * Fraction(2) ** -56 * scale
        # one rounding of the kept levels
        assert abs(Fraction(v) - kept) <= abs(kept) * Fraction(2) ** -52 + Fraction(2) ** -1074
        # against the FP64 values' exact dot product: the 56-bit quantisation
        true = sum(Fraction(x) * Fraction(y) for x, y in zip(a, b))
        assert abs(Fraction(v) - true) <= 2 * n * Fraction(2) ** -55 * scale + abs(true) * Fraction(2) ** -52


def test_level_bounds_below_2_24():
    """The analytic bound of every level: with |d0| <= 256 and |d_i| <= 128
    (i >= 1) a term of level l contributes at most
    sum_{i+k=l} max|a_i| max|b_k|; level 6 is the largest,
    2 * 256 * 128 + 5 * 128^2 = 147456 per term, and 112 terms give
    16,515,072 < 2^24: every partial sum of a chunk is an integer FP32 holds
    exactly."""
    top = [256] + [128] * 6
    bounds = [K_CHUNK * sum(top[i] * top[l - i] for i in range(l + 1) if l - i < 7) for l in range(7)]
    assert bounds[6] == 16_515_072 == max(bounds)
    assert all(b < 2 ** 24 for b in bounds)


def _chunk_sums_exact(da, db):
    """FP32 level sums of K_CHUNK equal terms, against exact integers"""
    acc = np.zeros(7, np.float32)
    exact = [0] * 7
    for _ in range(K_CHUNK):
        for i in range(7):
            for k in range(7 - i):
                acc[i + k] = np.float32(acc[i + k] + np.float32(da[i] * db[k]))
                exact[i + k] += da[i] * db[k]
    return acc, exact


def test_chunk_bound_worst_case():
    """The extreme digit vectors a 56-bit operand can take, each summed over
    a full chunk of 112 terms: every FP32 level sum stays an exact integer
    below 2^24.  Cases: top digit 256 with every lower digit -128 (the
    largest magnitudes, reachable because the lower digits pull |x| below
    2^56); the sign-aligned maximum of |level 6| (top digit -255, lower
    digits -128: every product of level 6 positive; a top digit of -256
    with them would leave the range); the largest same-sign positive digits
    (255, 127, ...); and mixed pairs of them."""
    S = sum(256 ** i for i in range(6))
    cases = {
        "256,-128": 256 * 256 ** 6 - 128 * S,
        "-255,-128": -255 * 256 ** 6 - 128 * S,
        "255,127": sum(d * 256 ** (6 - i) for i, d in enumerate([255] + [127] * 6)),
        "-256,127": -256 * 256 ** 6 + 127 * S,
    }
    want = {"256,-128": [256] + [-128] * 6, "-255,-128": [-255] + [-128] * 6,
            "255,127": [255] + [127] * 6, "-256,127": [-256] + [127] * 6}
    dig = {}
    for name, x in cases.items():
        assert abs(x) < 2 ** 56, name
        dig[name] = digits(x)
        assert dig[name] == want[name], name
    worst6 = 0
    for na, da in dig.items():
        for nb, db in dig.items():
            acc, exact = _chunk_sums_exact(da, db)
            assert max(abs(v) for v in exact) < 2 ** 24, (na, nb)
            assert [int(v) for v in acc] == exact, (na, nb)
            worst6 = max(worst6, abs(exact[6]))
    # the sign-aligned case reaches 112 * (2 * 255 * 128 + 5 * 128^2)
    assert worst6 == K_CHUNK * (2 * 255 * 128 + 5 * 128 * 128)