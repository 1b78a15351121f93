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


# --- the whole Householder reduction in double-float arithmetic -----------
# Vectorised forms of the operations above (float32 arrays, the same
# formulas), used to run tridiag_cluster_onchip's FP64-pass arithmetic on a
# random symmetric matrix.

def v_two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    return s, ((a - (s - bb)).astype(f32) + (b - bb)).astype(f32)


def v_fma(a, b, c):
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def v_two_prod(a, b):
    p = (a * b).astype(f32)
    return p, v_fma(a, b, -p)


def v_add(a, b):
    s = v_two_sum(a[0], b[0])
    t = v_two_sum(a[1], b[1])
    u = v_two_sum(s[0], (s[1] + t[0]).astype(f32))
    return v_two_sum(u[0], (u[1] + t[1]).astype(f32))


def v_mul(a, b):
    p = v_two_prod(a[0], b[0])
    return v_two_sum(p[0], v_fma(a[0], b[1], v_fma(a[1], b[0], p[1])))


def v_rank2(a, vi, wj, wi, vj):
    p1 = v_two_prod(vi[0], wj[0])
    p2 = v_two_prod(wi[0], vj[0])
    c = v_fma(vi[0], wj[1], v_fma(vi[1], wj[0], v_fma(wi[0], vj[1], (wi[1] * vj[0]).astype(f32))))
    s1 = v_two_sum(a[0], -p1[0])
    s2 = v_two_sum(s1[0], -p2[0])
    lo = ((a[1] + (s1[1] + s2[1]).astype(f32)).astype(f32) - ((p1[1] + p2[1]).astype(f32) + c).astype(f32)).astype(f32)
    return v_two_sum(s2[0], lo)


def split(x):
    h = np.asarray(x, dtype=np.float64).astype(f32)
    return h, (np.asarray(x, dtype=np.float64) - h.astype(np.float64)).astype(f32)


def to64(a):
    return a[0].astype(np.float64) + a[1].astype(np.float64)


def df64_tridiagonal(a64):
    """d, e of the Householder reduction with the matrix, v, p and w held as
    double-float pairs and the reflector's scalars formed in FP64, as in the
    kernel's double-float FP64 passes."""
    n = a64.shape[0]
    A = split(a64)
    d, e = np.zeros(n), np.zeros(n - 1)
    for k in range(n - 2):
        col = (A[0][k + 1:, k], A[1][k + 1:, k])
        xn2 = float(np.sum(to64((col[0][1:], col[1][1:])) ** 2))
        alpha = float(to64((col[0][:1], col[1][:1]))[0])
        d[k] = to64((A[0][k:k + 1, k], A[1][k:k + 1, k]))[0]
        if xn2 == 0.0:
            e[k] = alpha
            continue
        beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
        tk, scale = (beta - alpha) / beta, 1.0 / (alpha - beta)
        e[k] = beta
        sc = split(np.full(len(col[0]), scale))
        v = v_mul(col, sc)
        v[0][0], v[1][0] = f32(1), f32(0)
        # p = tau A22 v: row sums of products (pairs), then times tau
        B = (A[0][k + 1:, k + 1:], A[1][k + 1:, k + 1:])
        m1 = n - k - 1
        prod = v_mul(B, (np.broadcast_to(v[0], (m1, m1)), np.broadcast_to(v[1], (m1, m1))))
        acc = (np.zeros(m1, f32), np.zeros(m1, f32))
        for j in range(m1):
            acc = v_add(acc, (prod[0][:, j], prod[1][:, j]))
        tks = split(np.full(m1, tk))
        p = v_mul(acc, tks)
        K = float(np.sum(to64(p) * to64(v)))
        half = split(np.full(m1, 0.5 * tk * K))
        hv = v_mul(half, v)
        w = v_add(p, (-hv[0], -hv[1]))
        vi = (np.broadcast_to(v[0][:, None], (m1, m1)), np.broadcast_to(v[1][:, None], (m1, m1)))
        vj = (np.broadcast_to(v[0][None, :], (m1, m1)), np.broadcast_to(v[1][None, :], (m1, m1)))
        wi = (np.broadcast_to(w[0][:, None], (m1, m1)), np.broadcast_to(w[1][:, None], (m1, m1)))
        wj = (np.broadcast_to(w[0][None, :], (m1, m1)), np.broadcast_to(w[1][None, :], (m1, m1)))
        nb = v_rank2(B, vi, wj, wi, vj)
        A[0][k + 1:, k + 1:], A[1][k + 1:, k + 1:] = nb
    d[n - 2] = to64((A[0][n - 2:n - 1, n - 2], A[1][n - 2:n - 1, n - 2]))[0]
    d[n - 1] = to64((A[0][n - 1:, n - 1], A[1][n - 1:, n - 1]))[0]
    e[n - 2] = to64((A[0][n - 1:, n - 2], A[1][n - 1:, n - 2]))[0]
    return d, e


@pytest.mark.parametrize("n", [24, 60])
def test_df64_householder_eigenvalues(n):
    """The double-float Householder reduction of a symmetric matrix with the
    spread of an orthogonalised Fock matrix (eigenvalues -20..5 Eh) keeps
    its eigenvalues within 1e-12 of LAPACK's (measured 1e-13 to 2e-13, about
    1e-14 relative to the matrix norm; native FP64 reaches ~1e-15)."""
    rng = np.random.default_rng(n)
    q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    lam = np.sort(rng.uniform(-20.0, 5.0, size=n))
    a = (q * lam) @ q.T
    a = 0.5 * (a + a.T)
    d, e = df64_tridiagonal(a)
    t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    err = np.abs(np.linalg.eigvalsh(t) - np.linalg.eigvalsh(a)).max()
    assert err < 1e-12, err
