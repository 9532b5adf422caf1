"""The error model of the double-float products (xerus_gb300/csrc/df.cuh) that the
mixed solves' drift budget rests on, checked on the CPU: a step-by-step NumPy
restatement of the split (an FP64 value as an FP32 pair, the low part from the
next 29 significand bits) and of the TwoSum accumulation with renormalisation
every fourth product, against exact rational sums. The GPU kernels themselves are
checked against FP64 products in tests/test_tc_gemm.py."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def split(d):
    u = int(np.float64(d).view(np.uint64))
    e = ((u >> 52) & 0x7FF) - 1023
    if -74 <= e <= 127:
        sign = (u >> 32) & 0x80000000
        hi = np.uint32(sign | ((e + 127) << 23) | ((u >> 29) & 0x7FFFFF)).view(np.float32)
        scale = np.uint32(sign | ((e + 75) << 23)).view(np.float32)
        return hi, f32(f32(u & 0x1FFFFFFF) * scale)
    return f32(d), f32(0)


def fmaf(a, b, c):
    # one rounding of the exact a b + c to FP32
    return f32(float(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))))


def df_fma(a, b, s, c):
    p = f32(a[0] * b[0])
    e = fmaf(a[0], b[0], -p)
    e = fmaf(a[0], b[1], e)
    e = fmaf(a[1], b[0], e)
    t = f32(s + p)
    bp = f32(t - s)
    err = f32(f32(s - f32(t - bp)) + f32(p - bp))
    return t, f32(c + f32(err + e))


def df_dot(a, b):
    s, c = f32(0), f32(0)
    for k, (x, y) in enumerate(zip(a, b)):
        s, c = df_fma(split(x), split(y), s, c)
        if k % 4 == 3:
            t = f32(s + c)
            c = f32(c - f32(t - s))
            s = t
    return Fraction(float(s)) + Fraction(float(c))


def test_split_is_exact_to_2_pow_minus_47():
    rng = np.random.default_rng(3)
    vals = rng.standard_normal(2000) * np.exp2(rng.integers(-70, 120, 2000))
    for v in vals:
        if abs(v) < 2.0 ** -74:
            continue  # no FP32 low part there (checked below)
        hi, lo = split(v)
        assert abs(Fraction(float(hi)) + Fraction(float(lo)) - Fraction(float(v))) <= abs(Fraction(float(v))) * Fraction(1, 2 ** 47)
    assert split(0.0) == (0.0, 0.0) and split(-0.0)[1] == 0.0
    # below 2^-74 the value has no FP32 low part: FP32 precision
    hi, lo = split(3e-25)
    assert lo == 0.0 and abs(float(hi) / 3e-25 - 1) < 2.0 ** -23


def test_dot_products_within_the_stated_bound():
    rng = np.random.default_rng(5)
    worst = 0.0
    for K in (32, 384):
        for _ in range(6):
            a = rng.standard_normal(K)
            b = rng.standard_normal(K)
            exact = sum(Fraction(float(x)) * Fraction(float(y)) for x, y in zip(a, b))
            err = abs(float(df_dot(a, b) - exact)) / float(np.sum(np.abs(a * b)))
            worst = max(worst, err)
    # the kernels' documented accuracy: ~1e-15 of sum |a b| (mean), 1.5e-14 at most
    assert worst < 1.5e-14, worst
