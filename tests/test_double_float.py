"""The double-float (FP32 pair) arithmetic of the mixed Lanczos buffers,
restated in numpy float32 (boundstate-lanczos_gb300/csrc/bsl_device.cuh:
Knuth's TwoSum, Dekker's fast two-sum and exact product through FMA, the
accurate addition of Hida, Li and Bailey, and the fast addition), checked
against FP64 on random operands: a stored value keeps ~48 bits, the accurate
addition, the product and the square are within ~2^-46 of the exact result,
and the fast addition within ~2^-44 of |a| + |b|.

FMA is emulated exactly where the device uses it for an error term: the
product of two float32 numbers is exact in float64.
"""
import numpy as np

F = np.float32


def fma32(a, b, c):
    return F(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = F(a + b)
    bb = F(s - a)
    return s, F(F(a - F(s - bb)) + F(b - bb))


def fast_two_sum(a, b):
    s = F(a + b)
    return s, F(b - F(s - a))


def df_of(d):
    hi = F(d)
    return hi, F(d - np.float64(hi))


def val(x):
    return np.float64(x[0]) + np.float64(x[1])


def df_add(a, b):
    s1, s2 = two_sum(a[0], b[0])
    t1, t2 = two_sum(a[1], b[1])
    s2 = F(s2 + t1)
    s1, s2 = fast_two_sum(s1, s2)
    s2 = F(s2 + t2)
    return fast_two_sum(s1, s2)


def df_add_fast(a, b):
    s, e = two_sum(a[0], b[0])
    e = F(e + F(a[1] + b[1]))
    return fast_two_sum(s, e)


def df_mul(a, b):
    p = F(a[0] * b[0])
    e = fma32(a[0], b[0], -p)
    e = fma32(a[0], b[1], e)
    e = fma32(a[1], b[0], e)
    return fast_two_sum(p, e)


def df_sqr(a):
    p = F(a[0] * a[0])
    e = fma32(a[0], a[0], -p)
    e = fma32(F(2 * a[0]), a[1], e)
    return fast_two_sum(p, e)


def samples(n=2000, seed=0):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(n) * np.exp2(rng.integers(-20, 20, n)), rng.standard_normal(n) * np.exp2(
        rng.integers(-20, 20, n))


def test_stored_value_keeps_48_bits():
    x, _ = samples()
    err = max(abs(val(df_of(v)) - v) / abs(v) for v in x)
    assert err <= 2.0 ** -48


def test_accurate_add_mul_sqr():
    x, y = samples(seed=1)
    e_add = e_mul = e_sqr = 0.0
    for u, v in zip(x, y):
        a, b = df_of(u), df_of(v)
        ua, ub = val(a), val(b)  # the exact values the pairs hold
        s = val(df_add(a, b))
        if ua + ub != 0:
            e_add = max(e_add, abs(s - (ua + ub)) / abs(ua + ub))
        e_mul = max(e_mul, abs(val(df_mul(a, b)) - ua * ub) / abs(ua * ub))
        e_sqr = max(e_sqr, abs(val(df_sqr(a)) - ua * ua) / (ua * ua))
    # cancellation in ua + ub is handled by the accurate addition; FP64 is the reference
    assert e_add <= 2.0 ** -45, np.log2(e_add)
    assert e_mul <= 2.0 ** -45, np.log2(e_mul)
    assert e_sqr <= 2.0 ** -45, np.log2(e_sqr)


def test_fast_add_error_is_relative_to_the_operands():
    x, y = samples(seed=2)
    worst = 0.0
    for u, v in zip(x, y):
        a, b = df_of(u), df_of(v)
        ua, ub = val(a), val(b)
        worst = max(worst, abs(val(df_add_fast(a, b)) - (ua + ub)) / (abs(ua) + abs(ub)))
    assert worst <= 2.0 ** -44, np.log2(worst)
