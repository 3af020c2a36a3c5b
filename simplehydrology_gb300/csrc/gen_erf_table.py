"""Generate shy_erf_table.h: coefficient tables for the library's erf.

The erosion model evaluates erf(0.4 * discharge) (reference:
source/cellpool.h:242-244).  The library needs an erf that gives the same bits
on the host and on the GPU, so it evaluates erf with IEEE double additions and
multiplications only, in a fixed order, and rounds the result to float.  The
coefficients come from the mathematics, computed here in 60-digit decimal
arithmetic:

* |x| < 0.5: the Maclaurin series erf(x) = 2/sqrt(pi) * sum_n (-1)^n
  x^(2n+1) / (n! (2n+1)), evaluated as x * P(x^2) with 14 terms.
* 0.5 <= |x| < 4: 14 segments of width 0.25, each a degree-18 Taylor
  polynomial in u = x - c about the segment centre c.  erf(c) comes from the
  Maclaurin series (60 digits, enough terms to converge), and the derivatives
  from erf^(k)(x) = 2/sqrt(pi) (-1)^(k-1) H_{k-1}(x) exp(-x^2), H the
  physicists' Hermite polynomials.
* |x| >= 4: erf rounds to +-1 in float (erfc(3.85) < 2^-25).

Each double coefficient is also written as a pair of floats (the float
nearest it, then the float nearest the remainder), for the float-float
evaluation of the same polynomials (shy_erff_ff in shy_math.h).

Run:  python gen_erf_table.py > shy_erf_table.h
"""
import struct
from decimal import Decimal, getcontext

getcontext().prec = 60

SMALL_TERMS = 14
SEG_START = Decimal("0.5")
SEG_WIDTH = Decimal("0.25")
SEG_COUNT = 14
SEG_DEGREE = 18


def pi_decimal():
    # Machin: pi = 16 atan(1/5) - 4 atan(1/239)
    def atan_inv(n):
        x = Decimal(1) / n
        x2 = x * x
        term, total, k = x, x, 1
        while True:
            term *= -x2
            t = term / (2 * k + 1)
            if abs(t) < Decimal(10) ** -(getcontext().prec + 2):
                break
            total += t
            k += 1
        return total

    return 16 * atan_inv(5) - 4 * atan_inv(239)


PI = pi_decimal()
TWO_OVER_SQRT_PI = 2 / PI.sqrt()


def factorial(n):
    r = Decimal(1)
    for i in range(2, n + 1):
        r *= i
    return r


def erf_series(x):
    x = Decimal(x)
    x2 = x * x
    total = Decimal(0)
    power = x  # x^(2n+1)
    n = 0
    while True:
        term = power / (factorial(n) * (2 * n + 1))
        if n % 2:
            term = -term
        total += term
        if abs(term) < Decimal(10) ** -55 and n > 4:
            break
        power *= x2
        n += 1
    return TWO_OVER_SQRT_PI * total


def taylor_coeffs(c, degree):
    c = Decimal(c)
    coeffs = [erf_series(c)]
    ex = (-(c * c)).exp()
    h_prev, h = Decimal(1), 2 * c  # H_0, H_1
    herm = [h_prev, h]
    for n in range(1, degree):
        herm.append(2 * c * herm[n] - 2 * n * herm[n - 1])
    for k in range(1, degree + 1):
        sign = 1 if (k - 1) % 2 == 0 else -1
        deriv = TWO_OVER_SQRT_PI * sign * herm[k - 1] * ex
        coeffs.append(deriv / factorial(k))
    return coeffs


def fmt(d):
    return repr(float(d))


def f32(x):
    # round a double to the nearest float (ties to even)
    return struct.unpack("f", struct.pack("f", x))[0]


def fmt_pair(d):
    c = float(d)
    hi = f32(c)
    lo = f32(c - hi)  # c - hi is exact in double
    return "{" + repr(hi) + "f, " + repr(lo) + "f}"


def main():
    out = []
    out.append("// Generated by gen_erf_table.py -- do not edit by hand.")
    out.append("// Coefficients of the library's erf; see that script for the method.")
    out.append("// No include guard: shy_math.h includes it once per table namespace,")
    out.append("// with SHY_ERF_TABLE_QUAL set to the storage class wanted.")
    out.append(f"#define SHY_ERF_SMALL_TERMS {SMALL_TERMS}")
    out.append(f"#define SHY_ERF_SEG_COUNT {SEG_COUNT}")
    out.append(f"#define SHY_ERF_SEG_DEGREE {SEG_DEGREE}")
    small = []
    for n in range(SMALL_TERMS):
        c = TWO_OVER_SQRT_PI / (factorial(n) * (2 * n + 1))
        small.append(-c if n % 2 else c)
    out.append("// erf(x) = x * sum_n SMALL[n] * (x*x)^n for |x| < 0.5")
    out.append("SHY_ERF_TABLE_QUAL double shy_erf_small[SHY_ERF_SMALL_TERMS] = {")
    out.append("  " + ", ".join(fmt(c) for c in small))
    out.append("};")
    out.append("// segment s covers [0.5 + 0.25 s, 0.75 + 0.25 s); erf = sum_k SEG[s][k] * u^k,")
    out.append("// u = x - (0.625 + 0.25 s)")
    out.append("SHY_ERF_TABLE_QUAL double shy_erf_seg[SHY_ERF_SEG_COUNT][SHY_ERF_SEG_DEGREE + 1] = {")
    segs = []
    for s in range(SEG_COUNT):
        centre = SEG_START + SEG_WIDTH * s + SEG_WIDTH / 2
        co = taylor_coeffs(centre, SEG_DEGREE)
        segs.append(co)
        out.append("  {" + ", ".join(fmt(c) for c in co) + "},")
    out.append("};")
    out.append("// the same coefficients as float pairs {hi, lo}, hi + lo = the double to")
    out.append("// about 48 bits")
    out.append("SHY_ERF_TABLE_QUAL float shy_erf_small_f[SHY_ERF_SMALL_TERMS][2] = {")
    out.append("  " + ", ".join(fmt_pair(c) for c in small))
    out.append("};")
    out.append("SHY_ERF_TABLE_QUAL float shy_erf_seg_f[SHY_ERF_SEG_COUNT][SHY_ERF_SEG_DEGREE + 1][2] = {")
    for co in segs:
        out.append("  {" + ", ".join(fmt_pair(c) for c in co) + "},")
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
