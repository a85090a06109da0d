"""CPU checks (NumPy FP32, exact rational reference) of the double-float arithmetic the mixed SVD
and the double-float GEMM use (csrc/df.cuh): Knuth's TwoSum and Dekker's FastTwoSum are
error-free, the FMA TwoProd is error-free, the double-float product is accurate to ~2^-46, and the
compensated (Dot2, Ogita-Rump-Oishi) accumulation of double-float inner products stays near
2^-46 of sum |x||y| where a plain FP32 sum loses ~2^-24 sqrt(n).  The FMA is emulated by one
rounding to FP32 of the product and sum formed in FP64; where that is exact (the TwoProd error) the
emulation is exact."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def fma(a, b, c):
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def df_mul(ah, al, bh, bl):
    p = f32(ah * bh)
    e = fma(ah, bh, -p)
    e = fma(ah, bl, e)
    e = fma(al, bh, e)
    return fast_two_sum(p, e)


def dot2(xh, xl, yh, yl):
    s, lo = f32(0), f32(0)
    for i in range(len(xh)):
        p = f32(xh[i] * yh[i])
        e = fma(xh[i], yh[i], -p)
        t = f32(s + p)
        bv = f32(t - s)
        err = f32(f32(s - f32(t - bv)) + f32(p - bv))
        s = t
        lo = f32(lo + f32(err + e))
        lo = fma(xh[i], yl[i], lo)
        lo = fma(xl[i], yh[i], lo)
    return fast_two_sum(s, lo)


def split(x):
    h = x.astype(np.float32)
    return h, (x - h.astype(np.float64)).astype(np.float32)


def _samples(g, n):
    mant = g.uniform(-1, 1, n)
    return (mant * np.exp2(g.integers(-20, 20, n))).astype(np.float32)


def test_two_sum_and_fast_two_sum_are_exact():
    g = np.random.default_rng(1)
    a, b = _samples(g, 2000), _samples(g, 2000)
    for x, y in zip(a, b):
        s, e = two_sum(x, y)
        assert Fraction(float(s)) + Fraction(float(e)) == Fraction(float(x)) + Fraction(float(y))
        big, small = (x, y) if abs(x) >= abs(y) else (y, x)
        s, e = fast_two_sum(big, small)
        assert Fraction(float(s)) + Fraction(float(e)) == Fraction(float(big)) + Fraction(float(small))


def test_fma_two_prod_is_exact_and_df_mul_accurate():
    g = np.random.default_rng(2)
    a, b = _samples(g, 2000), _samples(g, 2000)
    for x, y in zip(a, b):
        p = f32(x * y)
        e = fma(x, y, -p)
        assert Fraction(float(p)) + Fraction(float(e)) == Fraction(float(x)) * Fraction(float(y))
    xs, ys = g.standard_normal(500), g.standard_normal(500)
    (xh, xl), (yh, yl) = split(xs), split(ys)
    for i in range(500):
        h, l = df_mul(xh[i], xl[i], yh[i], yl[i])
        exact = (Fraction(float(xh[i])) + Fraction(float(xl[i]))) * (Fraction(float(yh[i])) + Fraction(float(yl[i])))
        got = Fraction(float(h)) + Fraction(float(l))
        assert abs(float(got - exact)) <= 2.0 ** -45 * abs(float(exact))


def test_compensated_dot_stays_near_double_float_accuracy():
    g = np.random.default_rng(3)
    n = 1000
    x, y = g.standard_normal(n), g.standard_normal(n)
    (xh, xl), (yh, yl) = split(x), split(y)
    exact = sum((Fraction(float(xh[i])) + Fraction(float(xl[i]))) * (Fraction(float(yh[i])) + Fraction(float(yl[i])))
                for i in range(n))
    scale = float(np.sum(np.abs(x * y)))
    s, lo = dot2(xh, xl, yh, yl)
    err = abs(float(Fraction(float(s)) + Fraction(float(lo)) - exact))
    assert err <= 2.0 ** -44 * scale, (err / scale)
    naive = f32(0)
    for i in range(n):
        naive = f32(naive + f32(xh[i] * yh[i]))
    naive_err = abs(float(Fraction(float(naive)) - exact))
    assert naive_err > 1e4 * err  # the plain FP32 sum is far less accurate
