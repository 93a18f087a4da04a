"""Host restatement of the integer-slicing arithmetic of the tensor-core
overlap matrix m = C^T W (csrc/k_ozaki.cu), checked exactly with Python
integers and fractions: the digit expansion of every entry, the bound that
keeps every digit-pair sum exact in the tensor cores' fp32 accumulator, and
the accuracy of the two-sum recombination (fp32, as the kernel's epilogue
does it) against the exact product.  No GPU: this pins the scheme the kernel
implements; the GPU tests pin the kernel against binary64."""
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

OFF = 64 * ((1 << 49) - 1) // 127  # balanced base-128 digits as plain digits of X + OFF, minus 64


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", float(x)))[0]


def _eb(x):
    return (_bits(x) >> 52) & 0x7FF


def _w_digits(x, E):
    """w_1..w_7 of x 2^-E as the kernel's producers cut them: the digits of
    |x| (truncated at 2^-49) times the sign of x."""
    u = _bits(x)
    e = (u >> 52) & 0x7FF
    rs = E + 1026 - e
    X = 0
    if e != 0 and e != 0x7FF and rs < 64:
        X = ((u & ((1 << 52) - 1)) | (1 << 52)) >> rs
    Y = X + OFF
    assert 0 <= Y < (1 << 49)
    sg = -1 if u >> 63 else 1
    return [sg * (((Y >> (7 * (7 - s))) & 127) - 64) for s in range(1, 8)]


def _c_digits(x, F):
    """c_1..c_7 of x 2^-F as k_oz_split_c cuts them: balanced digits of the
    signed truncated value."""
    u = _bits(x)
    e = (u >> 52) & 0x7FF
    rs = F + 1026 - e
    X = 0
    if e != 0 and e != 0x7FF and rs < 64:
        X = ((u & ((1 << 52) - 1)) | (1 << 52)) >> rs
        if u >> 63:
            X = -X
    Y = X + OFF
    return [((Y >> (7 * (7 - t))) & 127) - 64 for t in range(1, 8)]


def _recombine(D, sc):
    """The epilogue: sum D_d 2^-7d (d = 2..9, exact fp32 terms) by two-sums
    from the smallest, as a double-float pair, scaled by 2^sc."""
    f = np.float32
    sm, er = f(D[7]) * f(2.0 ** -63), f(0.0)
    for d in range(8, 1, -1):
        tt = f(f(D[d - 2]) * f(2.0 ** (-7 * d)))
        s2 = f(sm + tt)
        bb = f(s2 - sm)
        er = f(er + f(f(sm - f(s2 - bb)) + f(tt - bb)))
        sm = s2
    hi = f(sm + er)
    lo = f(er - f(hi - sm))
    return Fraction(float(hi)) * Fraction(2) ** sc + Fraction(float(lo)) * Fraction(2) ** sc


def test_digit_sums_fit_fp32_up_to_584_orbitals():
    # |w_s c_t| <= 64 * 64 and at most 7 pairs (s, t) share a d = s + t: every partial sum is an
    # integer of magnitude <= 2^24, exact in fp32, up to 585 orbitals (the engine takes <= 584)
    assert 7 * 585 * 64 * 64 <= 2 ** 24 < 7 * 586 * 64 * 64


@pytest.mark.parametrize("n,o,seed", [(45, 5, 1), (12, 3, 2), (200, 2, 3)])
def test_integer_slicing_matches_exact_product(n, o, seed):
    rng = np.random.default_rng(seed)
    C = rng.standard_normal((n, o))
    W = rng.standard_normal((n, o)) + 1j * rng.standard_normal((n, o))
    W[:, 0] *= 1e-3           # a small column: its own scale E_r
    W[n // 2, :] = -W[n // 2, :]
    if o > 2:
        W[:, 2] = 0.0         # an all-zero column
    F = [max(_eb(C[i, a]) for i in range(n)) - 1020 for a in range(o)]
    worst = 0.0
    for b in range(o):
        for part in (0, 1):
            col = [(W[i, b].imag if part else W[i, b].real) for i in range(n)]
            E = max(_eb(v) for v in col) - 1020
            wd = [_w_digits(v, E) for v in col]
            for a in range(o):
                cd = [_c_digits(C[i, a], F[a]) for i in range(n)]
                D = [sum(wd[i][s - 1] * cd[i][d - s - 1] for i in range(n) for s in range(1, 8) if 1 <= d - s <= 7)
                     for d in range(2, 10)]
                assert max(abs(x) for x in D) < 2 ** 24
                m = _recombine(D, E + F[a])
                exact = sum(Fraction(C[i, a]) * Fraction(col[i]) for i in range(n))
                scale = max(abs(C[i, a]) for i in range(n)) * max(abs(v) for v in col)
                if scale == 0.0:
                    assert m == 0
                    continue
                worst = max(worst, abs(float(m - exact)) / scale)
    assert worst < 2.0 ** -42, math.log2(worst)
