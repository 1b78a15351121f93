"""Model of the double-float arithmetic of csrc/df64.cuh in numpy float32
(IEEE round to nearest, as on the GPU), checked against exact rational
arithmetic: every operation of the FP64 passes' double-float kernels keeps a
relative error near 2^-47 (a few 2^-48 ulps), ~48 significant bits.  No
device is needed."""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def fma(a, b, c):
    """fmaf: the product is exact in float64, one rounding to float32 after
    the sum (a float64 rounding of the sum first can differ in rare ties,
    which does not matter at the tolerances below)."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def two_prod(a, b):
    p = f32(a * b)
    return p, fma(a, b, -p)


def from_double(x):
    h = f32(x)
    return h, f32(np.float64(x) - np.float64(h))


def df_add(a, b):
    s = two_sum(a[0], b[0])
    t = two_sum(a[1], b[1])
    u = two_sum(s[0], f32(s[1] + t[0]))
    return two_sum(u[0], f32(u[1] + t[1]))


def df_mul(a, b):
    p = two_prod(a[0], b[0])
    return two_sum(p[0], fma(a[0], b[1], fma(a[1], b[0], p[1])))


def df_rank2(a, vi, wj, wi, vj):
    p1 = two_prod(vi[0], wj[0])
    p2 = two_prod(wi[0], vj[0])
    c = fma(vi[0], wj[1], fma(vi[1], wj[0], fma(wi[0], vj[1], f32(wi[1] * vj[0]))))
    s1 = two_sum(a[0], -p1[0])
    s2 = two_sum(s1[0], -p2[0])
    lo = f32(f32(a[1] + f32(s1[1] + s2[1])) - f32(f32(p1[1] + p2[1]) + c))
    return two_sum(s2[0], lo)


def df_dot(xs, ys):
    hi, lo = f32(0), f32(0)
    for a, b in zip(xs, ys):
        p = two_prod(a[0], b[0])
        c = fma(a[0], b[1], f32(a[1] * b[0]))
        s = two_sum(hi, p[0])
        hi = s[0]
        lo = f32(lo + f32(s[1] + f32(p[1] + c)))
    return two_sum(hi, lo)


def exact(x):
    return Fraction(float(x[0])) + Fraction(float(x[1]))


def rel(got, ref, scale):
    return float(abs(exact(got) - ref) / scale)


EPS = 2.0 ** -45  # four units of 2^-47


@pytest.fixture(scope="module")
def values():
    rng = np.random.default_rng(2024)
    mags = 10.0 ** rng.uniform(-6, 2, size=400)
    return [from_double(x) for x in rng.choice([-1.0, 1.0], size=400) * mags * rng.uniform(0.5, 1.0, size=400)]


def test_split_is_exact_to_48_bits(values):
    rng = np.random.default_rng(1)
    for x in rng.normal(size=200) * 10.0 ** rng.uniform(-8, 4, size=200):
        h, lo = from_double(x)
        assert abs(Fraction(float(h)) + Fraction(float(lo)) - Fraction(float(x))) <= abs(Fraction(float(x))) * 2.0 ** -48


def test_add_and_mul(values):
    worst_add = worst_mul = 0.0
    for a, b in zip(values[::2], values[1::2]):
        ea, eb = exact(a), exact(b)
        s = df_add(a, b)
        worst_add = max(worst_add, rel(s, ea + eb, abs(ea) + abs(eb)))
        m = df_mul(a, b)
        worst_mul = max(worst_mul, rel(m, ea * eb, abs(ea * eb)))
        assert abs(s[1]) <= abs(s[0]) * 2.0 ** -23 + 1e-45  # normalised
    assert worst_add < EPS and worst_mul < EPS, (worst_add, worst_mul)


def test_rank2_update_under_cancellation(values):
    """a - v_i w_j - w_i v_j with a chosen to cancel most of the products:
    the error stays relative to the terms, not to the small result."""
    worst = 0.0
    for k in range(0, 396, 4):
        vi, wj, wi, vj = values[k:k + 4]
        prods = exact(vi) * exact(wj) + exact(wi) * exact(vj)
        a = from_double(float(prods) * (1 + 1e-7))
        got = df_rank2(a, vi, wj, wi, vj)
        ref = exact(a) - prods
        scale = abs(exact(a)) + abs(exact(vi) * exact(wj)) + abs(exact(wi) * exact(vj))
        worst = max(worst, rel(got, ref, scale))
    assert worst < EPS, worst


def test_dot_product(values):
    """The matrix-vector product's running dot product over 300 terms:
    error relative to the sum of |terms|, within a few 2^-47 per term
    count's square root (the low part is renormalised once at the end)."""
    xs, ys = values[:300], values[100:400]
    got = df_dot(xs, ys)
    ref = sum(exact(a) * exact(b) for a, b in zip(xs, ys))
    scale = sum(abs(exact(a) * exact(b)) for a, b in zip(xs, ys))
    assert rel(got, ref, scale) < EPS * 4, rel(got, ref, scale)
