"""The digit arithmetic of the tensor-core mode products (QT_PREC_DF64_TC),
restated in exact integer arithmetic and checked against exact rational
products: every double-float value (hi + lo float pair) becomes an integer
m = round(v 2^(49 - E)) against the largest exponent E of its row, cut into
seven 7-bit digits; the digit products of one level L = s + t sum exactly in
fp32 (magnitude below 2^24); the levels L <= 6 combined give the product
within 2^-44 of |row max of X| |row max of h| per real product term (the
dropped pairs s + t >= 7 and the rounding of both operands, with 2^(E + F)
at most 4 times the product of the row maxima).  The GPU kernel
(qt_umma.cu, tcgen05) sums levels 0, 1 and 2 exactly and levels 3..6 in one
fp32 accumulator, whose rounding adds at most about 2^-45 of the level-0
scale per accumulation step; it is held to the oracle by the sweep parity
tests, this file pins the digit arithmetic those tests rely on."""
import struct
from fractions import Fraction

import numpy as np

DIGITS = 7


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", np.float32(x)))[0]


def row_exponent(his):
    """Largest biased exponent of the row's hi parts (at least 1)."""
    return max([1] + [(f32_bits(h) >> 23) & 0xFF for h in his])


def mag49(hi, lo, eb):
    """(negative, |hi + lo| in units of 2^(eb - 126 - 49), rounded): the
    parts taken with four guard bits from the float bits, then rounded."""
    bh, bl = f32_bits(hi), f32_bits(lo)
    eh, el = (bh >> 23) & 0xFF, (bl >> 23) & 0xFF
    mh = (bh & 0x7FFFFF) | (0x800000 if eh else 0)
    ml = (bl & 0x7FFFFF) | (0x800000 if el else 0)
    sh, sl = max(eh, 1) - eb + 29, max(el, 1) - eb + 29
    uh = mh << sh if sh >= 0 else (mh >> -sh if sh > -24 else 0)
    ul = ml << sl if sl >= 0 else (ml >> -sl if sl > -24 else 0)
    if ((bh ^ bl) >> 31) == 0:
        neg, u2 = bh >> 31, uh + ul
    elif uh >= ul:
        neg, u2 = bh >> 31, uh - ul
    else:
        neg, u2 = bl >> 31, ul - uh
    return neg, (u2 + 8) >> 4


def digits(neg, u):
    """Seven signed digits, most significant first (|q_0| <= 128, others <= 127)."""
    q = [u >> 42] + [(u >> (42 - 7 * s)) & 127 for s in range(1, DIGITS)]
    return [-x if neg else x for x in q]


def split(v):
    hi = np.float32(v)
    lo = np.float32(v - np.float64(hi))
    return hi, lo


def exact(hi, lo):
    return Fraction(float(hi)) + Fraction(float(lo))


def complex_row_digits(row):
    """Digits of a row of complex double-float values: (E, re digits, im digits)."""
    parts = [(split(z.real), split(z.imag)) for z in row]
    eb = row_exponent([p[0][0] for p in parts] + [p[1][0] for p in parts])
    re = [digits(*mag49(h, l, eb)) for (h, l), _ in parts]
    im = [digits(*mag49(h, l, eb)) for _, (h, l) in parts]
    exact_row = [(exact(*r), exact(*i)) for r, i in parts]
    return eb - 126, re, im, exact_row


def test_digits_reconstruct_within_one_unit():
    rng = np.random.default_rng(5)
    worst = Fraction(0)
    for trial in range(400):
        row = rng.standard_normal(16) * 10.0 ** rng.uniform(-6.0, 6.0, 16)  # 12 decades within a row
        row *= 10.0 ** int(rng.integers(-30, 30))
        if trial % 5 == 0:
            row[rng.integers(16)] = 0.0
        parts = [split(v) for v in row]
        eb = row_exponent([h for h, _ in parts])
        E = eb - 126
        for h, lo in parts:
            neg, u = mag49(h, lo, eb)
            assert u <= 2 ** 49
            q = digits(neg, u)
            assert abs(q[0]) <= 128 and all(abs(x) <= 127 for x in q[1:])
            rec = sum(Fraction(x) * Fraction(2) ** (-7 * (s + 1)) for s, x in enumerate(q)) * Fraction(2) ** E
            worst = max(worst, abs(rec - exact(h, lo)) / Fraction(2) ** (E - 49))
    assert worst <= Fraction(57, 100)


def test_level_sums_fit_fp32_exactly():
    # one level of one output: at most 7 digit pairs, 64 products each for the
    # real part X_re H_re and 64 for (-X_im) H_im, digits up to 128
    worst = 7 * (64 + 64) * 128 * 128
    assert worst < 2 ** 24
    assert float(np.float32(worst)) == worst


def test_emulated_mode_product_meets_bound():
    """Y[r, j] = sum_a X[r, a] h[j, a] from digits, levels combined exactly,
    against the exact product: error <= 2^-43 * K * max|X row| * max|h row|
    (two real products per complex term, each within 2^-44)."""
    rng = np.random.default_rng(11)
    R, K, N = 6, 40, 5
    X = (rng.standard_normal((R, K)) + 1j * rng.standard_normal((R, K))) * 10.0 ** rng.integers(-3, 3, (R, 1))
    H = (rng.standard_normal((N, K)) + 1j * rng.standard_normal((N, K))) * 10.0 ** rng.integers(-3, 3, (N, 1))
    X[0, :10] *= 1e-9  # a row with a wide dynamic range
    xr = [complex_row_digits(X[r]) for r in range(R)]
    hr = [complex_row_digits(H[j]) for j in range(N)]
    for r in range(R):
        Ex, xre, xim, xex = xr[r]
        for j in range(N):
            Fh, hre, him, hex_ = hr[j]
            # level sums: real = X_re H_re + (-X_im) H_im, imaginary = X_re H_im + X_im H_re
            re_lv, im_lv = [0] * DIGITS, [0] * DIGITS
            for L in range(DIGITS):
                for s in range(L + 1):
                    u = L - s
                    re_lv[L] += sum(xre[a][s] * hre[a][u] - xim[a][s] * him[a][u] for a in range(K))
                    im_lv[L] += sum(xre[a][s] * him[a][u] + xim[a][s] * hre[a][u] for a in range(K))
                assert abs(re_lv[L]) < 2 ** 24 and abs(im_lv[L]) < 2 ** 24
            scale = Fraction(2) ** (Ex + Fh)
            yre = sum(Fraction(v) * Fraction(2) ** (-7 * (L + 2)) for L, v in enumerate(re_lv)) * scale
            yim = sum(Fraction(v) * Fraction(2) ** (-7 * (L + 2)) for L, v in enumerate(im_lv)) * scale
            tre = sum(xex[a][0] * hex_[a][0] - xex[a][1] * hex_[a][1] for a in range(K))
            tim = sum(xex[a][0] * hex_[a][1] + xex[a][1] * hex_[a][0] for a in range(K))
            xmax = max(max(abs(p[0]), abs(p[1])) for p in xex)
            hmax = max(max(abs(p[0]), abs(p[1])) for p in hex_)
            bound = Fraction(2) ** -43 * K * xmax * hmax
            assert abs(yre - tre) <= bound and abs(yim - tim) <= bound
