"""CPU restatement of the FP64-accurate digit scheme of the tensor-core products
(gcge_old_gb300/csrc/gcge_cuda_ozaki.cu: d8_digits, the level sums of the
skewed MMAs and their combination), checked against exact rational arithmetic.
It pins the numbers the kernels rely on: the digits rebuild the scaled mantissa
exactly and are exact bf16 values, a level summed over 128 products fits the
FP32 accumulator exactly, and the kept levels 2..9 give a dot product within
2^-54 K 2^(Ex+Ey) of the exact one."""
from fractions import Fraction

import numpy as np
import pytest

NDIG = 7  # balanced base-256 digits of m = trunc(x 2^(55-E))


def scale_exponent(v):
    """E with |v_k| < 2^E for every k (the group's power of two)."""
    m = np.max(np.abs(v))
    return int(np.frexp(m)[1]) if m > 0 else 0


def digits(x, E):
    """d[k, a] (a = 0..6, most significant first) with
    trunc(x_k 2^(55-E)) = sum_a d[k, a] 256^(6-a); top digit in [-128, 128],
    the others in [-128, 127] (the bytes of m + 0x808080808080, minus 128)."""
    m = np.trunc(np.ldexp(x, 55 - E)).astype(np.int64)
    u = m + np.int64(0x808080808080)
    d = np.empty((len(x), NDIG), np.int64)
    d[:, 0] = u >> 48  # arithmetic shift: the signed top digit
    for a in range(1, NDIG):
        d[:, a] = ((u >> (8 * (6 - a))) & 0xFF) - 128
    return m, d


def as_bf16(v):
    f = np.asarray(v, np.float32).view(np.uint32) & np.uint32(0xFFFF0000)
    return f.view(np.float32)


def levels(dx, dy):
    """S[L] = sum_k sum_{a+b=L} dx[k,a] dy[k,b] for L = 2..14 (digits numbered
    1..7 as in the kernels: digit a is column a-1)."""
    S = {}
    for L in range(2, 2 * NDIG + 1):
        s = 0
        for a in range(1, NDIG + 1):
            b = L - a
            if 1 <= b <= NDIG:
                s += int(np.dot(dx[:, a - 1], dy[:, b - 1]))
        S[L] = s
    return S


def combine(S, Ex, Ey):
    """y = T 2^(Ex+Ey-55), T = sum_{L=2..9} S_L 2^(57-8L), levels 8 and 9 rounded
    to the integer unit (the kernels' 64-bit fixed-point combination)."""
    T = sum(S[L] << (57 - 8 * L) for L in range(2, 8))
    T += round(Fraction(S[8], 1 << 7)) + round(Fraction(S[9], 1 << 15))
    return Fraction(T) * Fraction(2) ** (Ex + Ey - 55)


def exact_dot(x, y):
    return sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(x, y))


@pytest.mark.parametrize("seed", range(6))
def test_digits_rebuild_the_mantissa_and_are_bf16(seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(4096) * np.exp2(rng.integers(-30, 30, 4096))
    x[:4] = [0.0, -0.0, 5e-324, -1e-310]  # zero and subnormals
    E = scale_exponent(x)
    m, d = digits(x, E)
    w = np.array([256 ** (6 - a) for a in range(NDIG)], dtype=object)
    assert all(int(sum(int(v) * int(c) for v, c in zip(d[k], w))) == int(m[k])
               for k in range(len(x)))
    assert d[:, 0].min() >= -128 and d[:, 0].max() <= 128
    assert d[:, 1:].min() >= -128 and d[:, 1:].max() <= 127
    assert np.array_equal(as_bf16(d.astype(np.float32)), d.astype(np.float32))
    # truncation: |x - m 2^(E-55)| < 2^(E-55)
    r = np.abs(x - np.ldexp(m.astype(np.float64), E - 55))
    assert (r < np.ldexp(1.0, E - 55)).all()


def test_level_sums_fit_the_fp32_accumulator():
    """A level over K = 128 products of extreme digits stays below 2^24."""
    K = 128
    dx = np.full((K, NDIG), -128, np.int64)
    dx[:, 0] = 128
    dy = dx.copy()
    S = levels(dx, dy)
    assert max(abs(v) for v in S.values()) < 2 ** 24


@pytest.mark.parametrize("K,spread,seed", [(128, 0, 1), (128, 20, 2), (64, 40, 3),
                                           (1000, 10, 4), (16, 0, 5)])
def test_kept_levels_give_fp64_accurate_dot_products(K, spread, seed):
    rng = np.random.default_rng(seed)
    worst = 0.0
    for _ in range(8):
        x = rng.standard_normal(K) * np.exp2(rng.integers(-spread, spread + 1, K))
        y = rng.standard_normal(K) * np.exp2(rng.integers(-spread, spread + 1, K))
        Ex, Ey = scale_exponent(x), scale_exponent(y)
        _, dx = digits(x, Ex)
        _, dy = digits(y, Ey)
        S = levels(dx, dy)
        got = combine(S, Ex, Ey)
        err = abs(got - exact_dot(x, y)) / (K * Fraction(2) ** (Ex + Ey))
        worst = max(worst, float(err))
        # the dropped levels 10..14 are below 2^-61 of the scale
        dropped = sum(abs(S[L]) * Fraction(2) ** (112 - 8 * L) for L in range(10, 15))
        assert dropped * Fraction(2) ** -110 < K * Fraction(2) ** -61
    assert worst < 2.0 ** -54, np.log2(worst)


# ---------------------------------------------------------------- digit planes
# CPU restatement of the plane records of k_cut_planes (gcge_cuda_ozaki.cu): per
# column and 64-row chunk, E (|x| < 2^E, one more when the largest m would not
# fit seven biased bytes) and, per 16-row stage s and digit a, 16 bytes of
# u = m + 0x0080808080808080 (byte 6 - a of row 16 s + r at 16 + 112 s + 16 a + r).
PL_MAXM = 0x007F7F7F7F7F7F7F


def cut_record(x):
    """x: 64 values of one chunk -> (E, record bytes[464])."""
    nz = np.abs(x[np.isfinite(x)])
    nz = nz[nz >= np.finfo(np.float64).tiny]  # subnormals count as zero
    if not np.all(np.isfinite(x)):
        E = 4096
    elif len(nz) == 0:
        E = -2000
    else:
        E = int(np.frexp(nz.max())[1])
    m = np.zeros(64, np.int64)
    if -2000 < E < 4096:
        keep = np.abs(x) >= np.finfo(np.float64).tiny
        m = np.where(keep, np.trunc(np.ldexp(x, 55 - E)), 0).astype(np.int64)
        if m.max() > PL_MAXM:
            E += 1
            m = np.where(keep, np.trunc(np.ldexp(x, 55 - E)), 0).astype(np.int64)
    u = (m + np.int64(0x0080808080808080)).astype(np.uint64)
    rec = np.zeros(464, np.uint8)
    rec[:4] = np.frombuffer(np.int32(E).tobytes(), np.uint8)
    for r in range(64):
        s, rr = divmod(r, 16)
        for a in range(NDIG):
            rec[16 + 112 * s + 16 * a + rr] = (int(u[r]) >> (8 * (6 - a))) & 0xFF
    return E, m, rec


def f16_digit(b):
    """The Gram kernel's conversion: the f16 with bits 0x6400 | b, minus 1152."""
    h = np.array([0x6400 | int(b)], np.uint16).view(np.float16)[0]
    return float(np.float16(h - np.float16(1152.0)))


def test_plane_bytes_convert_to_exact_f16_digits():
    assert all(f16_digit(b) == b - 128 for b in range(256))


@pytest.mark.parametrize("seed", range(4))
def test_plane_records_rebuild_the_mantissa(seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(64) * np.exp2(rng.integers(-20, 20, 64))
    if seed == 1:
        x *= 2.0 ** 6 / np.abs(x).max()
        x[5] = np.nextafter(2.0 ** 7, 0.0)  # largest m would be 2^55 - 4: needs E + 1
    if seed == 2:
        x[:] = -x.max()  # all negative at the scale: no bump needed
    if seed == 3:
        x[:3] = [0.0, 5e-324, -1e-310]
    E, m, rec = cut_record(x)
    assert int(m.max()) <= PL_MAXM
    w = [256 ** (6 - a) for a in range(NDIG)]
    for r in range(64):
        s, rr = divmod(r, 16)
        d = [int(rec[16 + 112 * s + 16 * a + rr]) - 128 for a in range(NDIG)]
        assert sum(di * wi for di, wi in zip(d, w)) == int(m[r])
    # truncation: at most one unit of 2^(E-55) (two when the exponent was bumped)
    r = np.abs(x - np.ldexp(m.astype(np.float64), E - 55))
    assert (r < np.ldexp(1.0, E - 55)).all()
    if seed == 1:
        assert E == 8
    # planes agree with the per-call digits wherever both apply
    if seed != 1:
        m2, _ = digits(x, E)
        assert np.array_equal(m, m2)
