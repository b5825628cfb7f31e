"""Exact models, on the CPU, of the tensor-core digit arithmetic of apply_tc
(kernels.cu) for complex128 and complex64 (TC64, the second test below).
complex128, with the host gate digits of convert_tc
(workspace.cpp): state reals as five balanced base-2^10 digits of
X = rint(|v| 2^(48 - E_row)) (ties to even) via the biased 10-bit fields,
gate reals as five digits of a = rint(|b| 2^(49 - E_col)), digit products
summed per level with levels 0-4 kept, level 4 shifted right by 10, and
value = S 2^(E_row + E_col - 47). Against exact rational products of the
same doubles: every kept pair sum fits the fp32 accumulator exactly
(|sum| <= 2^24), and the error per output stays below 2^-45 of the row
scale for unitary 5-qubit gates. The GPU tests check the kernel itself."""
import struct
from fractions import Fraction

import numpy as np

FIELD_BIAS = 512 * sum(1 << (10 * i) for i in range(5))


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", float(v)))[0]


def _rne_shift(m, sh):
    return (m + (1 << (sh - 1)) - 1 + ((m >> sh) & 1)) >> sh


def state_digits(v, ebrow):
    u = _bits(v)
    eb, a = (u >> 52) & 0x7FF, 0
    sh = 5 + ebrow - eb
    if eb and sh < 62:
        a = _rne_shift((u & ((1 << 52) - 1)) | (1 << 52), sh)
    y = (-a if u >> 63 else a) + FIELD_BIAS
    return [((y >> (10 * (4 - i))) & 1023) - 512 for i in range(5)]


def gate_digits(v, ebmax):
    u = _bits(v)
    eb, a = (u >> 52) & 0x7FF, 0
    sh = 4 + ebmax - eb
    if eb and sh < 62:
        a = _rne_shift((u & ((1 << 52) - 1)) | (1 << 52), sh)
    r = [(a >> (10 * (4 - i))) & 1023 for i in range(5)]
    r[0] = a >> 40
    for i in range(4, 0, -1):
        c = (r[i] + 512) >> 10
        r[i] -= c << 10
        r[i - 1] += c
    return [-x if u >> 63 else x for x in r]


def real_form(m):
    """B with y = x B for x the interleaved (re, im) inputs of one group."""
    d = m.shape[0]
    b = np.zeros((2 * d, 2 * d))
    for c in range(d):
        for r in range(d):
            z = m[r, c]
            b[2 * c, 2 * r], b[2 * c + 1, 2 * r] = z.real, -z.imag
            b[2 * c, 2 * r + 1], b[2 * c + 1, 2 * r + 1] = z.imag, z.real
    return b


def test_digit_scheme_error_bound():
    rng = np.random.default_rng(3)
    worst = 0.0
    for trial in range(4):
        q, _ = np.linalg.qr(rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32)))
        b = real_form(q)
        x = rng.standard_normal(64) * np.exp(rng.uniform(-8, 0, 64)) * 2.0 ** -int(rng.integers(0, 20))
        ebrow = max((_bits(v) >> 52) & 0x7FF for v in x)
        dx = [state_digits(v, ebrow) for v in x]
        for v, d in zip(x, dx):  # the digits carry |v| to 2^-49 of the row scale
            val = Fraction(sum(di << (10 * (4 - i)) for i, di in enumerate(d))) * Fraction(2) ** (ebrow - 1022 - 48)
            assert abs(val - Fraction(v)) <= Fraction(2) ** (ebrow - 1022 - 49)
        for j in range(0, 64, 5):
            ebc = max((_bits(b[k, j]) >> 52) & 0x7FF for k in range(64))
            de = [gate_digits(b[k, j], ebc) for k in range(64)]
            lev = [0] * 5
            for i in range(5):
                for jj in range(5 - i):
                    s = sum(dx[k][i] * de[k][jj] for k in range(64))
                    if i + jj <= 2:
                        assert abs(s) <= 1 << 24
                    lev[i + jj] += s
            S = (lev[0] << 30) + (lev[1] << 20) + (lev[2] << 10) + lev[3] + (lev[4] >> 10)
            y = Fraction(S) * Fraction(2) ** ((ebrow - 1022) + (ebc - 1022) - 47)
            exact = sum(Fraction(x[k]) * Fraction(b[k, j]) for k in range(64))
            worst = max(worst, abs(float(y - exact)) / 2.0 ** (ebrow - 1022))
    assert worst < 2.0 ** -45, worst


def _f32(v):
    return float(np.float32(v))


MAGIC = 12582912.0  # 1.5 * 2^23


def state_digits_c64(v, ebrow):
    """digits2f: x = rint(v 2^(19 - E_row)) on the FP32 pipe, hi = rint(x / 1024),
    lo = x - 1024 hi (each fmaf computed exactly in double, rounded once)."""
    s = 2.0 ** (145 - ebrow) if ebrow >= 20 else 0.0
    x = _f32(v * s + MAGIC) - MAGIC
    hi = _f32(x / 1024.0 + MAGIC) - MAGIC
    return int(hi), int(x - 1024.0 * hi)


def gate_digits_c64(v, ebmax):
    """Host digits with three digits: a = rint(|b| 2^(29 - E_col))."""
    u = _bits(v)
    eb, a = (u >> 52) & 0x7FF, 0
    sh = 24 + ebmax - eb
    if eb and sh < 62:
        a = _rne_shift((u & ((1 << 52) - 1)) | (1 << 52), sh)
    r = [a >> 20, (a >> 10) & 1023, a & 1023]
    for i in range(2, 0, -1):
        c = (r[i] + 512) >> 10
        r[i] -= c << 10
        r[i - 1] += c
    return [-x if u >> 63 else x for x in r]


def test_c64_digit_scheme_error_bound():
    """complex64 (TC64): two state digits x three gate digits, products (0,0),
    (0,1), (1,0), (0,2), FP32 epilogue. The gate's digits are exact to 2^-29 of
    the column scale; the output error stays below 2^-17 of the row scale."""
    rng = np.random.default_rng(4)
    worst, worst_gate = 0.0, 0.0
    for trial in range(4):
        q, _ = np.linalg.qr(rng.standard_normal((32, 32)) + 1j * rng.standard_normal((32, 32)))
        b = real_form(q)
        x = (rng.standard_normal(64) * np.exp(rng.uniform(-6, 0, 64))).astype(np.float32)
        ebrow = max((struct.unpack("<I", struct.pack("<f", float(v)))[0] >> 23) & 0xFF for v in x)
        erow = ebrow - 126
        dx = [state_digits_c64(float(v), ebrow) for v in x]
        for j in range(0, 64, 5):
            ebc = max((_bits(b[k, j]) >> 52) & 0x7FF for k in range(64))
            ecol = ebc - 1022
            de = [gate_digits_c64(b[k, j], ebc) for k in range(64)]
            for k in range(64):
                g = Fraction((de[k][0] << 20) + (de[k][1] << 10) + de[k][2]) * Fraction(2) ** (ecol - 29)
                worst_gate = max(worst_gate, abs(float(g - Fraction(b[k, j]))) / 2.0 ** ecol)
            acc = [sum(dx[k][i] * de[k][jj] for k in range(64)) for i, jj in ((0, 0), (0, 1), (1, 0), (0, 2))]
            assert all(abs(a) <= 1 << 24 for a in acc)  # exact in the FP32 accumulators
            t = _f32(acc[1] + acc[2])
            S = _f32(acc[0] * 1048576.0 + _f32(t * 1024.0 + acc[3]))
            y = Fraction(S) * Fraction(2) ** (erow - 19) * Fraction(2) ** (ecol - 19)
            exact = sum(Fraction(float(x[k])) * Fraction(b[k, j]) for k in range(64))
            worst = max(worst, abs(float(y - exact)) / 2.0 ** erow)
    assert worst_gate <= 2.0 ** -29, worst_gate
    assert worst < 2.0 ** -17, worst
