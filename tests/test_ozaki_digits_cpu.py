"""The digit arithmetic of the tensor-core mode products (QT_PREC_DF64_TC),
restated on the CPU and checked against exact rational arithmetic.

Every double-float value v = hi + lo of a row is scaled by 2^-E (E from the
row's largest exponent) and cut by error-free splits
x_s = fl(fl(r + sigma_s) - sigma_s), sigma_s = 1.5 * 2^(16 - 7s), into seven
signed digits q_s = x_s 2^(7(s+1)) (the low part joining from s = 3).  The
checks: the digits reconstruct v within 2^-49 of the row scale, they are
integers of at most 128 in magnitude (exact in bf16), the digit products of
one level sum below 2^24 (exact in fp32), and a complex mode product built
from them stays within 2^-43 of the product of the row maxima per term.  The
GPU kernel (qt_umma.cu, tcgen05) sums as many levels separately as tensor
memory holds and the rest in one fp32 accumulator; the sweep parity tests
hold it to the oracle, this file pins the digits those tests rely on."""
import struct
from fractions import Fraction

import numpy as np

DIGITS = 7


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", np.float32(x)))[0]


def row_exponent(his):
    """Largest biased exponent of the row's hi parts (at least 1)."""
    return max([1] + [(f32_bits(h) >> 23) & 0xFF for h in his])


def fsplit(r, sigma):
    x = np.float32(np.float32(r + sigma) - sigma)
    return x, np.float32(r - x)


def digits(hi, lo, eb):
    """Signed digits q_0..q_6 (Python ints) of hi + lo, as the device cuts them."""
    sc = np.float32(2.0 ** (126 - eb))
    rh, rl = np.float32(hi * sc), np.float32(lo * sc)
    q = []
    for s in range(DIGITS):
        sigma = np.float32(1.5 * 2.0 ** (16 - 7 * s))
        x, rh = fsplit(rh, sigma)
        if s >= 3:
            xl, rl = fsplit(rl, sigma)
            x = np.float32(x + xl)
        v = Fraction(float(x)) * 2 ** (7 * (s + 1))
        assert v.denominator == 1
        q.append(int(v))
    return q


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
    re = [digits(h, l, eb) for (h, l), _ in parts]
    im = [digits(h, l, eb) for _, (h, l) in parts]
    exact_row = [(exact(*r), exact(*i)) for r, i in parts]
    return eb - 126, re, im, exact_row


def test_digits_reconstruct_within_the_last_digit():
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
            q = digits(h, lo, eb)
            assert all(abs(x) <= 128 for x in q)
            rec = sum(Fraction(x) * Fraction(2) ** (-7 * (s + 1)) for s, x in enumerate(q)) * Fraction(2) ** E
            worst = max(worst, abs(rec - exact(h, lo)) / Fraction(2) ** (E - 49))
    assert worst <= 1


def test_digits_are_exact_in_bf16():
    # the stored digit x_s = q_s 2^(-7(s+1)), |q_s| <= 128, has at most eight
    # significant bits
    for q in range(-128, 129):
        for s in range(DIGITS):
            v = np.float32(q * 2.0 ** (-7 * (s + 1)))
            trunc = np.frombuffer(np.uint32(f32_bits(v) & 0xFFFF0000).tobytes(), np.float32)[0]
            assert trunc == v


def test_level_sums_fit_fp32_exactly():
    # one level of one output: at most 7 digit pairs, 64 products each for the
    # real part X_re H_re and 64 for (-X_im) H_im, digits up to 128
    worst = 7 * (64 + 64) * 128 * 128
    assert worst < 2 ** 24
    assert float(np.float32(worst)) == worst


def test_emulated_mode_product_meets_bound():
    """Y[r, j] = sum_a X[r, a] h[j, a] from digits, levels combined exactly,
    against the exact product: error <= 2^-43 * K * max|X row| * max|h row|."""
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
