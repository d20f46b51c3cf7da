"""CPU model of the plain form's tensor-core slice products (zone_gram_oz.cu): the same integer
steps as the kernels, in Python integers and NumPy, checked against exact arithmetic.

* fixed_prod: round(s h 2^(54 - E)) from the two FP64 significands equals exact rational
  rounding (half away from zero); zero and subnormal factors give 0, out-of-range and
  non-finite factors are flagged.
* The balanced base-256 digits of F + 0x80808080808080 reconstruct F; d_0 lies in [-64, 64],
  the others in [-128, 127]; the BF16 bit trick gives the digit's value exactly.
* Exactness budgets at their worst case (every digit at its bound, one sign): the Gram's
  levels 0..3 over the 256 observations between accumulator reads, and every level of the
  square-root transform's single 64-row K-tile, stay integers representable in FP32.
* The square-root transform (k_zone_tsym_oz): exponents from the exponent fields bound every
  element; the levels 0..6, the integer recombination v 2^16 + round(256 V456) and the scale
  2^(E_a + E_b - 52) give U diag(q^2) U^T to the error the kernel documents (the dropped
  levels and the fixed point's rounding), far inside the 1e-10 parity bar.
* The Gram (k_zone_gram_oz): the 4-tile accumulator reads into 64-bit level sums and the FP32
  sum of levels 4..6 give X^T X for 700 observations with columns over five decades.
* The transform kernel's integer recombination into FP64 (leading-zero count, shift,
  round-to-nearest-even) equals the correctly rounded conversion, ties included.
"""
import struct
from fractions import Fraction

import numpy as np

M64 = (1 << 64) - 1
BIAS = 0x80808080808080


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def fixed_prod(s, h, E):
    """The kernel's steps (64-bit words); None where the kernel sets its bad flag."""
    sb, hb = _bits(s), _bits(h)
    es, eh = (sb >> 52) & 0x7FF, (hb >> 52) & 0x7FF
    if es == 0x7FF or eh == 0x7FF:
        return None
    if es == 0 or eh == 0:
        return 0
    ms = (sb & 0xFFFFFFFFFFFFF) | 0x10000000000000
    mh = (hb & 0xFFFFFFFFFFFFF) | 0x10000000000000
    r = 2096 + E - es - eh
    if r >= 107:
        return 0
    if r < 50:
        return None
    lo, hi = (ms * mh) & M64, (ms * mh) >> 64
    if r - 1 < 64:
        lo2 = (lo + (1 << (r - 1))) & M64
        hi = (hi + (1 if lo2 < lo else 0)) & M64
        lo = lo2
    else:
        hi = (hi + (1 << (r - 1 - 64))) & M64
    F = (((hi << (64 - r)) & M64) | (lo >> r)) if r < 64 else (hi >> (r - 64))
    if F > (1 << 54):
        return None
    return -F if hb >> 63 else F


def digits(F):
    U = (F + BIAS) & M64
    return [((U >> (8 * (6 - p))) & 255) - 128 for p in range(7)]


def _round_half_away(q):
    a = abs(q)
    fl = a.numerator // a.denominator
    r = fl + (1 if a - fl >= Fraction(1, 2) else 0)
    return -r if q < 0 else r


def test_fixed_prod_is_exact_rounding():
    rng = np.random.default_rng(11)
    n = 0
    for _ in range(6000):
        E = int(rng.integers(-30, 31))
        s = float(rng.uniform(0, 1)) * 2.0 ** int(rng.integers(-20, 1))
        h = float(rng.uniform(-1, 1)) * 2.0 ** E / max(s, 1e-300) * float(
            rng.choice([1.0, 1e-3, 1e-9, 1e-16]))
        if abs(s * h) > 2.0 ** E or s == 0.0:
            continue
        ref = _round_half_away(Fraction(s) * Fraction(h) * Fraction(2) ** (54 - E))
        assert fixed_prod(s, h, E) == ref, (s, h, E)
        n += 1
    assert n > 4000
    assert fixed_prod(0.0, 1.0, 0) == 0 and fixed_prod(1.0, 5e-324, 0) == 0
    assert fixed_prod(1.0, 2.0 ** -60, 0) == 0                 # below half a fixed-point unit
    assert fixed_prod(1.0, 1.0, 0) == 1 << 54                  # the bound itself
    assert fixed_prod(1.0, 4.0, 0) is None                     # above the bound
    assert fixed_prod(float("nan"), 1.0, 0) is None and fixed_prod(1.0, float("inf"), 0) is None


def test_balanced_digits():
    rng = np.random.default_rng(12)
    cases = [0, 1, -1, 1 << 54, -(1 << 54), (1 << 54) - 1, -(1 << 54) + 1]
    cases += [int(x) for x in rng.integers(-(1 << 54), 1 << 54, 5000, dtype=np.int64)]
    for F in cases:
        d = digits(F)
        assert sum(dp * 256 ** (6 - p) for p, dp in enumerate(d)) == F
        assert -64 <= d[0] <= 64 and all(-128 <= x <= 127 for x in d[1:])
    # BF16 bits of (byte - 128): the FP32 value 0x4B3FFF80 + byte minus 1.5 2^23, exact
    byte = np.arange(256, dtype=np.uint32)
    v = (byte + np.uint32(0x4B3FFF80)).view(np.float32) - np.float32(12582912.0)
    assert np.array_equal(v, byte.astype(np.float32) - np.float32(128))
    assert np.array_equal((v.view(np.uint32) & np.uint32(0xFFFF)), np.zeros(256, np.uint32))


def _levels(D, K):
    """level_L = sum_{p+q=L} D_p^T D_q over the first K rows (exact int64)."""
    lev = np.zeros((13,) + (D.shape[2], D.shape[2]), dtype=np.int64)
    for p in range(7):
        for q in range(7):
            lev[p + q] += D[p, :K].T @ D[q, :K]
    return lev


def test_exactness_budgets_at_the_worst_case():
    # every digit at its bound with one sign: d_0 = -64, the others -128
    for K, top in ((256, 3), (64, 6)):    # Gram: levels 0..3 over 256 rows; transform: 0..6
        D = np.empty((7, K, 2), dtype=np.int64)
        D[0], D[1:] = -64, -128
        lev = _levels(D, K)
        assert np.abs(lev[:top + 1]).max() <= 2 ** 24
    # ... and the transform's single K-tile stays below 2^23 (level 6: 7 pairs)
    assert 64 * (2 * 64 * 128 + 5 * 128 * 128) < 2 ** 23


def _f32_fma(a, b, c):
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def test_square_root_transform_model():
    rng = np.random.default_rng(13)
    N = 64
    U, _ = np.linalg.qr(rng.standard_normal((N, N)))
    lam = np.concatenate([10.0 ** rng.uniform(-16, 0, 40), 10.0 ** rng.uniform(0, 8, 24)])
    q = (1.0 / (1.0 + lam)) ** 0.25
    X = q[:, None] * U.T                                     # X[k, a] = q_k U_ak
    # exponents from the exponent fields (k_zone_tsym_oz)
    eq = np.array([(_bits(x) >> 52) & 0x7FF for x in q])
    eu = np.array([[(_bits(x) >> 52) & 0x7FF for x in row] for row in U.T])
    E = (eq[:, None] + eu).max(axis=0) - 2044
    assert np.all(np.abs(X) < 2.0 ** E[None, :])
    D = np.zeros((7, N, N), dtype=np.int64)
    for k in range(N):
        for a in range(N):
            F = fixed_prod(q[k], U[a, k], int(E[a]))
            assert F is not None and abs(F) <= 1 << 54
            D[:, k, a] = digits(F)
    lev = _levels(D, N)
    assert np.abs(lev[:7]).max() < 2 ** 23
    l = lev.astype(np.float32)
    v = ((lev[0] * 256 + lev[1]) * 256 + lev[2]) * 256 + lev[3]
    f456 = np.vectorize(_f32_fma)(l[6], np.float32(1 / 65536), _f32_fma_v(l[5], l[4]))
    vt = v * 65536 + np.rint(f456.astype(np.float64) * 256).astype(np.int64)
    T = vt.astype(np.float64) * 2.0 ** (E[:, None] + E[None, :] - 52)
    Tx = (X.astype(np.longdouble).T @ X.astype(np.longdouble))
    err = np.abs((T - Tx).astype(np.float64))
    # the documented bound: per row, the dropped levels 7..12 (at most 6 2^14 256^5 / 2^108 of
    # 2^(E_a + E_b)) plus the fixed point's rounding (2^-54 of it), over the 64 rows
    bound = 64 * (6 * 2.0 ** -54 * 1.01 + 2.0 ** -53) * 2.0 ** (E[:, None] + E[None, :])
    assert np.all(err <= bound)
    assert err.max() < 1e-14 * np.abs(Tx).max()
    assert np.array_equal(T, T.T)                            # the levels are symmetric


def _f32_fma_v(l5, l4):
    return np.vectorize(_f32_fma)(l5, np.float32(1 / 256), l4)


def test_gram_model_with_accumulator_reads():
    rng = np.random.default_rng(14)
    rows, N = 700, 64
    H = rng.standard_normal((rows, N)) * (10.0 ** rng.uniform(-3, 2, N))[None, :]
    s = rng.uniform(0.01, 3.0, rows)
    X = s[:, None] * H
    cmax = np.abs(X).max(axis=0) * (1 + 2.0 ** -20)
    E = np.array([((_bits(c) >> 52) & 0x7FF) - 1022 for c in cmax])
    assert np.all(np.abs(X) <= 2.0 ** E[None, :])
    D = np.zeros((7, rows, N), dtype=np.int64)
    for k in range(rows):
        for a in range(N):
            F = fixed_prod(s[k], H[k, a], int(E[a]))
            assert F is not None
            D[:, k, a] = digits(F)
    acc64 = np.zeros((4, N, N), dtype=np.int64)
    accf = np.zeros((N, N), dtype=np.float32)
    for r0 in range(0, rows, 256):                          # reads every 4 K-tiles
        lev = _levels(D[:, r0:r0 + 256], min(256, rows - r0))
        assert np.abs(lev[:4]).max() < 2 ** 24               # FP32 accumulators exact
        acc64 += lev[:4]
        l = lev.astype(np.float32)
        part = np.vectorize(_f32_fma)(l[6], np.float32(1 / 65536), _f32_fma_v(l[5], l[4]))
        accf = (accf + part).astype(np.float32)
    v = ((acc64[0] * 256 + acc64[1]) * 256 + acc64[2]) * 256 + acc64[3]
    G = (v.astype(np.float64) + accf.astype(np.float64) / 256) * 2.0 ** (
        E[:, None] + E[None, :] - 36)
    Gx = X.astype(np.longdouble).T @ X.astype(np.longdouble)
    rel = np.abs((G - Gx).astype(np.float64)) / 2.0 ** (E[:, None] + E[None, :])
    assert rel.max() < rows * 2.0 ** -50
    assert np.abs((G - Gx).astype(np.float64)).max() < 1e-14 * float(np.abs(Gx).max())


def scaled_i64(vt, e2):
    """The transform kernel's integer recombination: vt 2^e2 rounded to nearest even."""
    if vt == 0:
        return 0.0
    sgn = (1 << 63) if vt < 0 else 0
    m = -vt if vt < 0 else vt
    lz = 64 - m.bit_length()
    be = 63 - lz + e2 + 1023
    assert 1 <= be <= 2045
    mm = (m << lz) & M64
    mant = (mm >> 11) & 0xFFFFFFFFFFFFF
    rem = mm & 0x7FF
    up = 1 if (rem > 0x400 or (rem == 0x400 and (mant & 1))) else 0
    bits = sgn | ((be << 52) + mant + up)
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def test_integer_recombination_rounds_as_fp64():
    rng = np.random.default_rng(15)
    cases = [1, -1, 3, (1 << 53) + 1, (1 << 53) + 3, (1 << 62) - 1, -(1 << 62) + 1,
             (1 << 54) + (1 << 1), (1 << 54) + (3 << 1), (1 << 61) + (1 << 8)]
    cases += [int(x) for x in rng.integers(-(1 << 62), 1 << 62, 20000, dtype=np.int64)]
    cases += [int(x) >> int(s) for x, s in zip(rng.integers(1, 1 << 62, 2000, dtype=np.int64),
                                               rng.integers(0, 60, 2000))]
    for vt in cases:
        for e2 in (-52, -60, 0, 7):
            # Python's int -> float conversion rounds to nearest even; the power of two is exact
            assert scaled_i64(vt, e2) == float(vt) * 2.0 ** e2, (vt, e2)
