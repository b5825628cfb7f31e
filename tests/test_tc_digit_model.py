"""An exact model, on the CPU, of the complex128 tensor-core digit arithmetic
of apply_tc (kernels.cu) with the host gate digits of convert_tc
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
