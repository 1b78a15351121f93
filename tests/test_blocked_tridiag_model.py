"""A numpy model of the blocked cluster tridiagonalisation
(``k_tridiag_cluster_blocked`` in ``dxtb_gb300/csrc/linalg.cu``), phase by
phase in the kernel's order, checked against LAPACK on CPU.

The kernel splits the Householder reduction like LAPACK's dsytrd/dlatrd:
within a panel of columns the trailing matrix is left as it was at the panel
start; column c is corrected with the panel's earlier (v, w) pairs before
its reflector is built; w = tau (A22 v - V (W^T v) - W (V^T v)) - tau/2 (p.v) v;
and the rank-2 updates are applied at the panel end.  Two details are the
kernel's own and are modelled here exactly:
- the previous column's pair enters the next column's correction before any
  barrier, with its w at row c taken from the value every CTA computes
  (``wnext``) and its v from the previous reflector still in shared memory;
- v of column c is stored in row c right of the diagonal, w in the scratch
  W[l][i] (the eigenvector matrix in the kernel).
The outputs (d, e, tau and the reflectors) must give Q T Q^T = A with
Q = H_0 ... H_{n-3}, the back-transformation's convention."""
import numpy as np
import pytest


def blocked_tridiag(a0: np.ndarray, nb: int):
    n = a0.shape[0]
    a = a0.copy()
    wmat = np.zeros((max(nb, 1), n))
    d = np.zeros(n)
    e = np.zeros(n)
    tau = np.zeros(n)
    vs = np.zeros(n + 1)
    wnext = 0.0
    p0 = 0
    while p0 + 2 < n:
        pw = min(nb, n - 2 - p0)
        for jj in range(pw):
            c = p0 + jj
            m1 = n - c - 1
            # A: row c's coefficients, then the corrected column (own rows)
            coef_w = np.array([wnext if l == jj - 1 else wmat[l, c] for l in range(jj)])
            coef_v = np.array([1.0 if l == jj - 1 else a[p0 + l, c] for l in range(jj)])
            x = np.empty(m1)
            for i in range(c + 1, n):
                xi = a[i, c]
                for l in range(jj - 1):
                    xi -= a[p0 + l, i] * coef_w[l] + wmat[l, i] * coef_v[l]
                if jj > 0:
                    xi -= vs[i - c] * coef_w[jj - 1] + wmat[jj - 1, i] * coef_v[jj - 1]
                x[i - c - 1] = xi
            # B: reflector, A22 v, partial sums
            alpha, xn2 = x[0], float(np.sum(x[1:] ** 2))
            tk, scale, beta = 0.0, 0.0, alpha
            if xn2 != 0.0:
                beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
                tk = (beta - alpha) / beta
                scale = 1.0 / (alpha - beta)
            d[c] = a[c, c] - 2.0 * float(np.dot(coef_w, coef_v))
            e[c], tau[c] = beta, tk
            vs = np.zeros(n + 1)
            vs[:m1] = x * scale
            vs[0] = 1.0
            rows = np.arange(c + 1, n)
            v = vs[:m1]
            y = a[c + 1:, c + 1:] @ v
            x1 = wmat[:jj, rows] @ v          # W^T v
            x2 = a[p0:p0 + jj, rows] @ v      # V^T v
            k = tk * (float(v @ y) - 2.0 * float(x1 @ x2))
            # C: w of every row > c (row c + 1 is the redundant wnext)
            corr = a[p0:p0 + jj, rows].T @ x1 + wmat[:jj, rows].T @ x2
            wmat[jj, rows] = tk * (y - corr) - 0.5 * tk * k * v
            wnext = wmat[jj, c + 1]
            a[c, c + 1:] = v
        pe = p0 + pw
        vp, wp = a[p0:pe, pe:], wmat[:pw, pe:]
        a[pe:, pe:] -= vp.T @ wp + wp.T @ vp
        p0 += nb
    if n >= 2:
        d[n - 2], d[n - 1], e[n - 2] = a[n - 2, n - 2], a[n - 1, n - 1], a[n - 1, n - 2]
    else:
        d[0] = a[0, 0]
    return d, e[:max(n - 1, 0)], tau, a


def q_from_reflectors(a: np.ndarray, tau: np.ndarray) -> np.ndarray:
    n = a.shape[0]
    q = np.eye(n)
    for k in range(n - 3, -1, -1):
        v = np.zeros(n)
        v[k + 1:] = a[k, k + 1:]
        q = q - tau[k] * np.outer(v, v @ q)
    return q


@pytest.mark.parametrize("n,nb", [(2, 32), (3, 32), (5, 2), (12, 4), (40, 8), (70, 32), (97, 32)])
def test_blocked_model_matches_lapack(n, nb):
    rng = np.random.default_rng(n)
    m = rng.normal(size=(n, n))
    m = (m + m.T) / 2
    d, e, tau, a = blocked_tridiag(m, nb)
    t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(np.linalg.eigvalsh(t) - np.linalg.eigvalsh(m)).max() < 1e-12
    if n > 2:
        q = q_from_reflectors(a, tau)
        assert np.abs(q @ t @ q.T - m).max() < 1e-12


def test_blocked_model_zero_column():
    # a column that is already reduced (tau = 0, w = 0) inside a panel
    n = 20
    rng = np.random.default_rng(3)
    m = rng.normal(size=(n, n))
    m = (m + m.T) / 2
    m[2:, 0] = m[0, 2:] = 0.0
    d, e, tau, a = blocked_tridiag(m, 8)
    assert tau[0] == 0.0
    t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    assert np.abs(np.linalg.eigvalsh(t) - np.linalg.eigvalsh(m)).max() < 1e-12


def onchip_cluster_tridiag(a: np.ndarray, csize: int = 8):
    """Phase-by-phase model of tridiag_cluster_onchip (csrc/linalg.cu): rows
    owned cyclically by `csize` CTAs in their shared memory, one exchange per
    step.  Before it every CTA publishes p_k of its rows, its partial p.v and
    a copy of column k+1 of its rows as they are before the step's update;
    after it every CTA forms w_k, applies the update to that copy of column
    k+1 itself (for all rows) and builds reflector k+1 from it, while the
    owners update their rows.  Without reflection tau = 0 and v = e_1 (the
    update is then the identity).  Returns d, e, tau and the reflector rows,
    in the kernel's index conventions."""
    n = a.shape[0]
    own = [[i for i in range(n) if i % csize == r] for r in range(csize)]
    rows = {i: a[i].copy() for i in range(n)}  # row i on CTA i % csize
    d, e, tau = np.zeros(n), np.zeros(n), np.zeros(n)
    refl = np.zeros((n, n))

    def reflector(k, x):
        """x: column k of rows k+1.. (identical in every CTA) -> tau_k, v_k."""
        xn2 = float(np.dot(x[1:], x[1:]))
        alpha = x[0]
        tk, scale, beta = 0.0, 0.0, alpha
        if xn2 != 0.0:
            beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
            tk = (beta - alpha) / beta
            scale = 1.0 / (alpha - beta)
        e[k], tau[k] = beta, tk
        return tk, np.concatenate([[1.0], x[1:] * scale])

    d[0] = rows[0][0]
    tk, v = reflector(0, np.array([rows[i][0] for i in range(1, n)]))
    for k in range(n - 2):
        m1 = n - k - 1
        refl[k, k + 1:] = v
        if k > 0:
            d[k] = rows[k][k]
        # before the exchange: p_k and p.v partials of own rows, column k+1 copies
        ps, kp, col = {}, [0.0] * csize, {}
        for r in range(csize):
            for i in own[r]:
                if i >= k + 1:
                    ps[i] = tk * np.dot(rows[i][k + 1:], v)
                    kp[r] += ps[i] * v[i - (k + 1)]
                if i >= k + 2:
                    col[i] = rows[i][k + 1]
        # after it: w_k, the updated column k+1 and reflector k+1 (every CTA)
        half = 0.5 * tk * sum(kp)
        wv = np.array([ps[k + 1 + t] - half * v[t] for t in range(m1)])
        vnext = None
        if k + 3 < n:
            x = np.array([col[i] - v[i - (k + 1)] * wv[0] - wv[i - (k + 1)] * v[0] for i in range(k + 2, n)])
            tnext, vnext = reflector(k + 1, x)
        # owners' update
        for r in range(csize):
            for i in own[r]:
                if i >= k + 1:
                    t = i - (k + 1)
                    rows[i][k + 1:] -= v[t] * wv + wv[t] * v
        if vnext is not None:
            tk, v = tnext, vnext
    d[n - 2], d[n - 1], e[n - 2] = rows[n - 2][n - 2], rows[n - 1][n - 1], rows[n - 1][n - 2]
    return d, e, tau, refl


@pytest.mark.parametrize("n", [13, 40, 67])
def test_onchip_cluster_model_against_lapack(n):
    """The model's tridiagonal has the eigenvalues of A, and the reflectors
    (v_k with v_0 = 1 in row k, tau_k) rebuild A = Q T Q^T."""
    rng = np.random.default_rng(n)
    a = rng.normal(size=(n, n))
    a = a + a.T
    a[:5, 5:] = 0.0  # two decoupled blocks: column 4 is zero below the
    a[5:, :5] = 0.0  # diagonal at step 4 (the tau = 0 branch)
    d, e, tau, refl = onchip_cluster_tridiag(a)
    assert tau[4] == 0.0
    t = np.diag(d) + np.diag(e[:-1], 1) + np.diag(e[:-1], -1)
    assert np.allclose(np.linalg.eigvalsh(t), np.linalg.eigvalsh(a), atol=1e-10)
    q = np.eye(n)
    for k in range(n - 2):
        v = np.zeros(n)
        v[k + 1:] = refl[k, k + 1:]
        q = q @ (np.eye(n) - tau[k] * np.outer(v, v))
    assert np.allclose(q @ t @ q.T, a, atol=1e-10)
