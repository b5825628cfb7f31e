"""Exact CPU model of the digit arithmetic of the tensor-memory pass
(umma_pass.cu: digits6, digits6_df, level_sum_to_df + df_to_double_scaled;
workspace.cpp: gate_digits9).

State reals: six balanced base-2^9 digits of X' = v 2^(1030 - E_row), computed
with the kernel's FP32 operations (numpy float32, round to nearest even).
Gate reals: six digits of a = rint(|b| 2^(1074 - E_col)) (integers, top digit
<= 128). Level sums S_L = sum over i + j = L of the 64-term digit products;
the output double is assembled from the six level sums with the kernel's
FP32 fast two-sums and integer bit assembly. Checked against exact rational
products of the same doubles: digit bounds (|d| <= 256, |d_2| <= 260), level
sums 0-3 below 2^24 (exact in the tensor cores' fp32 accumulators), and the
error per output below 2^-45 of the row scale, on Haar-random gates, on
aligned worst cases (flat rows and flat gate columns, rounding ties) and on
outputs just below a power of two."""
import math
import struct
from fractions import Fraction

import numpy as np

F = np.float32
M0, M9, M27 = F(12582912.0), F(24576.0), F(0.09375)


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def _f32_from_bits(u):
    return np.frombuffer(struct.pack("<I", u & 0xFFFFFFFF), dtype=np.float32)[0]


def _f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", float(x)))[0]


def rnd_with(x, m):
    return F(F(x + m) - m)


def digits6(v, eb_row):
    """umma_pass.cu digits6, operation by operation."""
    u = _bits(v)
    hi, lo = u >> 32, u & 0xFFFFFFFF
    eb = (hi >> 20) & 0x7FF
    dh = eb - eb_row + 134
    dh = 0 if eb == 0 else max(dh, 0)
    sgn = hi & 0x80000000
    mant = ((hi << 3) | (lo >> 29)) & 0xFFFFFFFF
    H = _f32_from_bits((mant & 0x7FFFFF) | (dh << 23) | sgn)
    dl = max(dh - 52, 0)
    L = F(F(lo & 0x1FFFFFFF) * _f32_from_bits((dl << 23) | sgn))
    T0 = rnd_with(H, M9)
    R0 = F(H - T0)
    R27 = rnd_with(R0, M27)
    D = F(F(R0 - R27) + L)
    D27 = rnd_with(D, M27)
    T1 = F(R27 + D27)
    T2 = F(D - D27)
    d0 = rnd_with(T0, M0)
    d1 = F(F(T0 - d0) * F(512))
    u2 = F(T1 * F(262144))
    d2 = rnd_with(u2, M0)
    d3 = F(F(u2 - d2) * F(512))
    u4 = F(T2 * F(68719476736.0))
    d4 = rnd_with(u4, M0)
    d5 = rnd_with(F(F(u4 - d4) * F(512)), M0)
    out = [d0, d1, d2, d3, d4, d5]
    assert all(float(x) == int(x) for x in out)
    return [int(x) for x in out]


def gate_digits9(v, ebmax):
    """workspace.cpp gate_digits9."""
    u = _bits(v)
    eb = (u >> 52) & 0x7FF
    a = 0
    sh = ebmax - eb + 1
    if eb and sh < 62:
        m = (u & ((1 << 52) - 1)) | (1 << 52)
        a = (m + (1 << (sh - 1)) - 1 + ((m >> sh) & 1)) >> sh
    r = [0] * 6
    for i in range(1, 6):
        r[i] = (a >> (9 * (5 - i))) & 511
    r[0] = a >> 45
    for i in range(5, 0, -1):
        c = (r[i] + 256) >> 9
        r[i] -= c << 9
        r[i - 1] += c
    return [-x if u >> 63 else x for x in r]


def fast_two_sum(a, b):
    s = F(a + b)
    return s, F(b - F(s - a))


def level_sum_to_double(S, off):
    """umma_pass.cu level_sum_to_df then df_to_double_scaled; S: six level
    sums as float32 (the accumulators), off = E_row + E_col - 2059."""
    S = [F(x) for x in S]
    b1 = F(S[1] * F(1.0 / 512))
    b2 = F(S[2] * F(1.0 / 262144))
    b3 = F(S[3] * F(1.0 / 134217728))
    p4 = F(S[4] * F(2.0 ** -36))
    f = F(float(Fraction(float(S[5])) * Fraction(2) ** -45 + Fraction(float(p4))))
    s1, e1 = fast_two_sum(S[0], b1)
    s2, e2 = fast_two_sum(s1, b2)
    s3, e3 = fast_two_sum(s2, b3)
    t = F(F(e1 + e2) + F(e3 + f))
    h, l = fast_two_sum(s3, t)
    hb = _f32_bits(h)
    eh = (hb >> 23) & 0xFF
    be = eh + 896 + off
    if eh == 0 or be <= 0:
        return 0.0
    sg = hb & 0x80000000
    whi = (be << 20) | ((hb & 0x7FFFFF) >> 3) | sg
    wlo = (hb << 29) & 0xFFFFFFFF
    lb = _f32_bits(l)
    below = 1 if ((hb & 0x7FFFFF) == 0 and float(l) != 0.0 and ((lb ^ hb) & 0x80000000)) else 0
    se = min(306 - eh + below, 254)
    prod = F(l * _f32_from_bits((se << 23) | sg))
    delta = int(np.rint(np.float64(prod)))  # float -> int, to nearest even
    w = ((whi << 32) | wlo) & 0x7FFFFFFFFFFFFFFF
    w = (w + delta) & 0xFFFFFFFFFFFFFFFF
    w |= sg << 32
    return struct.unpack("<d", struct.pack("<Q", w))[0]


def real_form(m):
    """Real form of a complex gate: y = x B for x the interleaved (re, im)
    inputs of one group (B[2c][2r] = Re m_rc, B[2c+1][2r] = -Im m_rc, ...)."""
    d = m.shape[0]
    b = np.zeros((2 * d, 2 * d))
    for c in range(d):
        for r in range(d):
            z = m[r, c]
            b[2 * c, 2 * r] = z.real
            b[2 * c + 1, 2 * r] = -z.imag
            b[2 * c, 2 * r + 1] = z.imag
            b[2 * c + 1, 2 * r + 1] = z.real
    return b


def check_row(x, b, cols, stats):
    eb_row = max((_bits(v) >> 52) & 0x7FF for v in x)
    dx = [digits6(v, eb_row) for v in x]
    for d in dx:
        assert max(abs(d[i]) for i in (0, 1, 3, 4, 5)) <= 256
        assert abs(d[2]) <= 260
    for v, d in zip(x, dx):  # the digits carry v to ~2^-48 of the row scale
        val = sum(Fraction(di) * Fraction(2) ** (-9 * i) for i, di in enumerate(d)) * Fraction(2) ** (eb_row - 1030)
        err = abs(val - Fraction(v))
        stats["quant"] = max(stats["quant"], float(err) / 2.0 ** (eb_row - 1022))
    for n in cols:
        ebc = max((_bits(b[k, n]) >> 52) & 0x7FF for k in range(64))
        de = [gate_digits9(b[k, n], ebc) for k in range(64)]
        assert all(abs(e[0]) <= 128 and max(abs(t) for t in e[1:]) <= 256 for e in de)
        S = [0] * 6
        for i in range(6):
            for j in range(6 - i):
                S[i + j] += sum(dx[k][i] * de[k][j] for k in range(64))
        for L in range(4):
            assert abs(S[L]) < 1 << 24, (L, S[L])
        y = level_sum_to_double(S, eb_row + ebc - 2059)
        exact = sum(Fraction(x[k]) * Fraction(b[k, n]) for k in range(64))
        stats["out"] = max(stats["out"], abs(float(Fraction(y) - exact)) / 2.0 ** (eb_row - 1022))


def test_umma_digits_haar_gates():
    rng = np.random.default_rng(11)
    stats = {"quant": 0.0, "out": 0.0}
    for trial in range(3):
        q, _ = np.linalg.qr(rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32)))
        b = real_form(q)
        x = rng.standard_normal(64) * np.exp(rng.uniform(-10, 0, 64)) * 2.0 ** -int(rng.integers(0, 30))
        x[int(rng.integers(0, 64))] = 0.0
        check_row(x, b, range(0, 64, 7), stats)
    assert stats["quant"] < 2.0 ** -46, stats
    assert stats["out"] < 2.0 ** -45, stats


def test_umma_output_just_below_a_power_of_two():
    """Level sums whose double-float high part is an exact power of two with
    the low part below it (the result lies in the lower binade): the level
    sums of an amplitude met on the GPU (24 qubits), and a sweep around 2^15."""
    S = [32916, -75645, -67000, -111171, -8494, -76860]
    exact = sum(Fraction(s) * Fraction(2) ** (-9 * i) for i, s in enumerate(S)) * Fraction(2) ** (1011 + 1021 - 2059)
    y = level_sum_to_double(S, 1011 + 1021 - 2059)
    assert abs(Fraction(y) - exact) <= Fraction(2) ** -60
    for s1 in range(-75700, -75600, 7):
        S = [32916, s1, -67000, -111171, 0, 0]
        exact = sum(Fraction(s) * Fraction(2) ** (-9 * i) for i, s in enumerate(S))
        y = level_sum_to_double(S, 0)
        assert abs(Fraction(y) - exact) <= abs(exact) * Fraction(2) ** -50


def test_umma_digits_aligned_worst_cases():
    """Flat rows times flat (Hadamard-like) columns align every digit
    product; values placed on rounding ties of the 2^-9 grid exercise the
    d_2 <= 260 bound."""
    stats = {"quant": 0.0, "out": 0.0}
    h5 = np.array([[(-1) ** bin(r & c).count("1") for c in range(32)] for r in range(32)]) / math.sqrt(32.0)
    b = real_form(h5.astype(np.complex128))
    x = np.full(64, 1.0 / math.sqrt(64.0))
    check_row(x, b, range(0, 64, 9), stats)
    # rounding ties: H's bits below 2^-9 exactly one half, L nonzero
    base = 2.0 ** 7 * (1 + 2.0 ** -17)
    xt = np.array([(base + 2.0 ** -30 * (k + 1)) * 2.0 ** -40 * (-1) ** k for k in range(64)])
    check_row(xt, b, range(0, 64, 13), stats)
    assert stats["out"] < 2.0 ** -45, stats


def digits6_df(h, l, ebf_row):
    """umma_pass.cu digits6_df: the six digits of (h + l) 2^(134 - E_row)
    for a normalized double-float (|l| <= ulp(h) / 2), E_row the largest
    float exponent of the group's high parts; the scaling in two exact
    steps, then digits6's cascade."""
    k = 134 - ebf_row
    k1 = min(k, 127)
    k2 = k - k1
    s1, s2 = _f32_from_bits((k1 + 127) << 23), _f32_from_bits((k2 + 127) << 23)
    H = F(F(F(h) * s1) * s2)
    L = F(F(F(l) * s1) * s2)
    T0 = rnd_with(H, M9)
    R0 = F(H - T0)
    R27 = rnd_with(R0, M27)
    D = F(F(R0 - R27) + L)
    D27 = rnd_with(D, M27)
    T1 = F(R27 + D27)
    T2 = F(D - D27)
    d0 = rnd_with(T0, M0)
    d1 = F(F(T0 - d0) * F(512))
    u2 = F(T1 * F(262144))
    d2 = rnd_with(u2, M0)
    d3 = F(F(u2 - d2) * F(512))
    u4 = F(T2 * F(68719476736.0))
    d4 = rnd_with(u4, M0)
    d5 = rnd_with(F(F(u4 - d4) * F(512)), M0)
    out = [d0, d1, d2, d3, d4, d5]
    assert all(float(x) == int(x) for x in out)
    return [int(x) for x in out]


def test_umma_digits_from_double_float():
    """Digits of double-float amplitudes (a diagonal run applied before the
    dense gate, kept as double-floats): bounds |d| <= 256 (d_2 <= 260) and
    the value to 2^-46 of the group's scale, over groups with a wide
    exponent range, exact zeros, ties and groups of tiny amplitudes (the
    two-step scaling)."""
    rng = np.random.default_rng(17)
    worst = 0.0
    for trial in range(40):
        scale = 2.0 ** -int(rng.integers(0, 140)) if trial % 5 == 4 else 2.0 ** -int(rng.integers(0, 30))
        x = rng.standard_normal(64) * np.exp(rng.uniform(-12, 0, 64)) * scale
        x[rng.random(64) < 0.1] = 0.0
        hs = [F(v) for v in x]
        ls = [F(v - float(hv)) for v, hv in zip(x, hs)]
        if trial % 7 == 3:  # ties of the 2^-9 grid in H
            hs[0] = F(2.0 ** 7 * (1 + 2.0 ** -17) * scale)
            ls[0] = F(2.0 ** -30 * scale)
        ebf = max((_f32_bits(v) >> 23) & 0xFF for v in hs)
        if ebf == 0:
            continue
        for hv, lv in zip(hs, ls):
            d = digits6_df(hv, lv, ebf)
            assert max(abs(d[i]) for i in (0, 1, 3, 4, 5)) <= 256 and abs(d[2]) <= 260, d
            val = sum(Fraction(di) * Fraction(2) ** (-9 * i) for i, di in enumerate(d)) * Fraction(2) ** (ebf - 134)
            err = abs(val - (Fraction(float(hv)) + Fraction(float(lv))))
            worst = max(worst, float(err / Fraction(2) ** (ebf - 126)))
    assert worst < 2.0 ** -46, worst


# ---------------------------------------------------------------- complex64

def digits3(x, ef_row):
    """umma_pass.cu digits3 with the group scale 2^k, k = min(134 - Ef, 126)."""
    k = min(134 - ef_row, 126)
    X = F(F(x) * _f32_from_bits((k + 127) << 23))
    d0 = F(F(X + M0) - M0)
    r = F(X - d0)
    d1 = F(F(r * F(512) + M0) - M0)            # the FMA: r * 512 is exact
    u = F(float(r) * 512.0 - float(d1))        # exact
    d2 = F(F(u * F(512) + M0) - M0)
    return [int(d0), int(d1), int(d2)], k


def level_sum4_scaled(S, k, ebc):
    """umma_pass.cu level_sum4, then times the column scale 2^(E_col - 1029)
    and the group scale 2^-k."""
    S = [float(F(x)) for x in S]
    t = F(S[2] * 2.0 ** -18 + float(F(S[3] * 2.0 ** -27)))   # FMA: one rounding
    v = F(S[0] + float(F(S[1] * 2.0 ** -9 + float(t))))
    cs = 2.0 ** (ebc - 1029)
    return F(F(float(v) * cs) * F(2.0 ** -k))


def gate_digits4(v, ebmax):
    """workspace.cpp gate_digits9 with nd = 4 (complex64)."""
    u = _bits(v)
    eb = (u >> 52) & 0x7FF
    a = 0
    sh = ebmax - eb + 1 + 18
    if eb and sh < 62:
        m = (u & ((1 << 52) - 1)) | (1 << 52)
        a = (m + (1 << (sh - 1)) - 1 + ((m >> sh) & 1)) >> sh
    r = [a >> 27, (a >> 18) & 511, (a >> 9) & 511, a & 511]
    for i in (3, 2, 1):
        c = (r[i] + 256) >> 9
        r[i] -= c << 9
        r[i - 1] += c
    return [-x if u >> 63 else x for x in r]


def test_umma_complex64_digits_levels_and_outputs():
    """complex64 tensor-memory pass: three digits per state real and four
    per gate real, levels 0-3 exact (every level sum below 2^24, also for flat rows
    against flat columns); the output (level sums by an FMA chain, times the
    column and group scales)'s error against the exact product of
    the same float inputs and double gate entries is below 2^-23 of
    sum_k |x_k b_kn| (the scale an FP32 dot product's own rounding is
    measured against: a 64-term FP32 sum is accurate to 64 2^-24 of it in
    the worst case)."""
    rng = np.random.default_rng(23)
    h5 = np.array([[(-1) ** bin(r & c).count("1") for c in range(32)] for r in range(32)]) / math.sqrt(32.0)
    worst = 0.0
    cases = []
    for trial in range(4):
        q, _ = np.linalg.qr(rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32)))
        x = (rng.standard_normal(64) * np.exp(rng.uniform(-8, 0, 64)) * 2.0 ** -int(rng.integers(0, 20))).astype(np.float32)
        cases.append((real_form(q), x))
    cases.append((real_form(h5.astype(np.complex128)), np.full(64, 1 / 8.0, dtype=np.float32)))
    for b, x in cases:
        ef = max((_f32_bits(v) >> 23) & 0xFF for v in x)
        dx = [digits3(v, ef)[0] for v in x]
        k = digits3(x[0], ef)[1]
        assert all(abs(d) <= 256 for dd in dx for d in dd)
        for n in range(0, 64, 5):
            ebc = max((_bits(b[k, n]) >> 52) & 0x7FF for k in range(64))
            de = [gate_digits4(b[k, n], ebc) for k in range(64)]
            assert all(abs(e[0]) <= 128 and max(abs(t) for t in e[1:]) <= 256 for e in de)
            S = [0] * 4
            for i in range(3):
                for j in range(4):
                    if i + j <= 3:
                        S[i + j] += sum(dx[k][i] * de[k][j] for k in range(64))
            assert all(abs(v) < 1 << 24 for v in S), S
            y = level_sum4_scaled(S, k, ebc)
            exact = sum(Fraction(float(x[k])) * Fraction(b[k, n]) for k in range(64))
            scale = sum(abs(float(x[k]) * b[k, n]) for k in range(64))
            worst = max(worst, abs(float(Fraction(float(y)) - exact)) / scale)
    assert worst < 2.0 ** -23, worst
