"""The double-float summation the mixed solve's CGLS products use (ls.cu df_mad).

A product a * x with a an FP32 matrix entry and x an FP64 operand split into
floats x = xh + xl is formed as p + e (p = fl(a xh), e its FMA-recovered error
plus a xl) and added to the float pair (sh, sl) with Knuth's TwoSum followed by
a Fast2Sum renormalisation; the pair is flushed into an FP64 sum every 32
terms.  These host checks restate the steps in numpy float32 (every operation
rounded to nearest, none contracted, as the device code's _rn intrinsics
guarantee) and compare with exact rational sums: the scheme's error stays at
the 2^-48 level per flushed group, well below FP32 (2^-24), and the
renormalisation is what keeps it there over long groups.
"""
from fractions import Fraction

import numpy as np

F = np.float32


def round32(q):
    """The float32 nearest to the rational q, ties to even (one rounding)."""
    f = F(float(q))
    cands = [f, np.nextafter(f, F(np.inf)), np.nextafter(f, F(-np.inf))]
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - q), int(np.array(c).view(np.int32)) & 1))


def fma32(a, b, c):
    """fl32(a * b + c) with a single rounding (the device's fmaf)."""
    return round32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def split(x):
    """x (FP64) = xh + xl: xh = fl32(x), xl = fl32(x - xh)."""
    xh = F(x)
    return xh, F(x - float(xh))


def df_mad(a, xh, xl, sh, sl, renorm=True):
    p = F(a * xh)
    e = fma32(a, xh, -p)
    e = fma32(a, xl, e)
    t = F(sh + p)
    z = F(t - sh)
    err = F(F(sh - F(t - z)) + F(p - z))
    if renorm:
        u = F(sl + F(err + e))
        s2 = F(t + u)
        return s2, F(u - F(s2 - t))
    return t, F(sl + F(err + e))


def df_dot(a, x, flush=32, renorm=True):
    """sum_j a_j x_j as the device computes it: float pairs, FP64 flushes."""
    acc = 0.0
    for g0 in range(0, len(a), flush):
        sh = sl = F(0)
        for j in range(g0, min(len(a), g0 + flush)):
            xh, xl = split(x[j])
            sh, sl = df_mad(F(a[j]), xh, xl, sh, sl, renorm)
        acc += float(sh) + float(sl)
    return acc


def exact_dot(a, x):
    return sum(Fraction(float(F(aj))) * Fraction(float(xj)) for aj, xj in zip(a, x))


def rel_err(v, a, x):
    ex = exact_dot(a, x)
    scale = sum(abs(Fraction(float(F(aj))) * Fraction(float(xj))) for aj, xj in zip(a, x))
    return float(abs(Fraction(v) - ex) / scale)


def test_split_is_exact_to_48_bits():
    rng = np.random.default_rng(0)
    for x in rng.standard_normal(200) * 10.0 ** rng.integers(-8, 8, 200):
        xh, xl = split(float(x))
        assert abs(float(xh) + float(xl) - x) <= 2.0 ** -47 * abs(x)


def test_two_sum_steps_are_error_free():
    rng = np.random.default_rng(1)
    for _ in range(500):
        sh, p = F(rng.standard_normal()), F(rng.standard_normal() * 10.0 ** rng.integers(-6, 6))
        t = F(sh + p)
        z = F(t - sh)
        err = F(F(sh - F(t - z)) + F(p - z))
        assert Fraction(float(t)) + Fraction(float(err)) == Fraction(float(sh)) + Fraction(float(p))


def test_dot_error_at_double_float_level():
    rng = np.random.default_rng(2)
    n = 256
    for trial in range(6):
        a = rng.standard_normal(n).astype(np.float32)
        x = rng.standard_normal(n)
        if trial % 2:
            x = x * 1e-10 + 1.0          # operands with long FP64 mantissas
        e = rel_err(df_dot(a, x), a, x)
        assert e < 2.0 ** -44, e         # FP32 arithmetic alone would give ~2^-24


def test_renormalisation_keeps_long_groups_accurate():
    """Without the Fast2Sum step the low word accumulates FP32 rounding over a
    flushed group; with it the group error stays at the double-float level."""
    rng = np.random.default_rng(3)
    n = 512
    worst = {True: 0.0, False: 0.0}
    for _ in range(4):
        a = rng.standard_normal(n).astype(np.float32)
        x = rng.standard_normal(n)
        for renorm in (True, False):
            worst[renorm] = max(worst[renorm], rel_err(df_dot(a, x, flush=n, renorm=renorm), a, x))
    assert worst[True] < 2.0 ** -44
    assert worst[True] <= worst[False]
