"""numpy models of two eigensolver kernels of ``dxtb_gb300/csrc/linalg.cu``,
checked against LAPACK on CPU.

1. ``k_tridiag_smem``: Householder tridiagonalisation on the packed lower
   triangle with the fused look-ahead.  Each step makes one pass over the
   triangle that applies the previous step's rank-2 update to every element,
   stores it, and accumulates this step's A v (the row part, and the column
   part by symmetry).  Only the next column receives this step's update at
   once, since the next reflector needs it; the last diagonal element gets
   its final update after the loop.
2. ``k_bisect``: an eigenvalue is bracketed by Sturm counts in FP32 to a
   few FP32 ulps of |T|, then polished by Newton steps on the FP64
   characteristic polynomial (with its derivative by the same three-term
   recurrence, rescaled against overflow), and accepted only if two FP64
   Sturm counts place it at the right index.
"""
import numpy as np
import scipy.linalg

from dxtb_gb300 import molgen
from oracle import gfn1_oracle as go


# ---------------------------------------------------------------------------
# 1. on-chip tridiagonalisation with the fused look-ahead
# ---------------------------------------------------------------------------
def fused_tridiag(a: np.ndarray):
    n = a.shape[0]
    low = np.tril(a).astype(float)           # low[i, j], j <= i: the packed triangle
    d, e, tau = np.zeros(n), np.zeros(n), np.zeros(n)
    refl = np.zeros((n, n))                  # reflector k in row k (back-transformation layout)
    v_buf, w_buf = np.zeros((2, n)), np.zeros((2, n))
    cur = 0
    xn2 = float((low[2:, 0] ** 2).sum())
    for k in range(n - 2):
        m1 = n - k - 1
        vc, wc, vp, wp = v_buf[cur], w_buf[cur], v_buf[cur ^ 1], w_buf[cur ^ 1]
        alpha = low[k + 1, k]
        tk, scale, beta = 0.0, 0.0, alpha
        if xn2 != 0.0:
            beta = -np.copysign(np.sqrt(alpha * alpha + xn2), alpha)
            tk = (beta - alpha) / beta
            scale = 1.0 / (alpha - beta)
        d[k], e[k], tau[k] = low[k, k], beta, tk
        for t in range(m1):
            v = 0.0 if tk == 0.0 else (1.0 if t == 0 else low[k + 1 + t, k] * scale)
            vc[k + 1 + t] = v
            refl[k, k + 1 + t] = v
        # one pass: pending update of the previous step, then A v
        j0 = k + 1
        prow, pcol = np.zeros(n), np.zeros(n)
        for i in range(j0, n):
            for j in range(j0, i + 1):
                x = low[i, j] - (vp[i] * wp[j] + wp[i] * vp[j])
                low[i, j] = x
                prow[i] += x * vc[j]
                if j < i:
                    pcol[j] += x * vc[i]
        p = tk * (prow + pcol)
        half = 0.5 * tk * float(p[j0:] @ vc[j0:])
        wc[j0:] = p[j0:] - half * vc[j0:]
        # look-ahead: the next column gets this step's update now
        vj, wj = vc[j0], wc[j0]
        xn2 = 0.0
        for i in range(j0, n):
            x = low[i, j0] - (vc[i] * wj + wc[i] * vj)
            low[i, j0] = x
            if i >= j0 + 2:
                xn2 += x * x
        cur ^= 1
    if n >= 3:
        low[n - 1, n - 1] -= 2.0 * v_buf[cur ^ 1][n - 1] * w_buf[cur ^ 1][n - 1]
    d[n - 2], d[n - 1], e[n - 2] = low[n - 2, n - 2], low[n - 1, n - 1], low[n - 1, n - 2]
    return d, e[:n - 1], tau, refl


def test_fused_lookahead_tridiagonalisation():
    rng = np.random.default_rng(2)
    for n in (3, 4, 7, 20, 45):
        a = rng.normal(size=(n, n))
        a = a + a.T
        d, e, tau, refl = fused_tridiag(a)
        t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
        assert np.abs(np.linalg.eigvalsh(t) - np.linalg.eigvalsh(a)).max() < 1e-12
        q = np.eye(n)
        for k in range(n - 3, -1, -1):
            v = np.zeros(n)
            v[k + 1:] = refl[k, k + 1:]
            q = q - tau[k] * np.outer(v, v @ q)
        assert np.abs(q @ t @ q.T - a).max() < 1e-12


# ---------------------------------------------------------------------------
# 2. FP32 bracket, FP64 Newton polish, FP64 Sturm check
# ---------------------------------------------------------------------------
def sturm_count(d, e2, x, pivmin, dt) -> int:
    """Eigenvalues of the tridiagonal below x: sign changes of the leading
    principal minors, rescaled to stay in range."""
    d = d.astype(dt)
    e2 = e2.astype(dt)
    x = dt(x)
    big, small = dt(2.0 ** 40), dt(2.0 ** -40)
    pm, pc = dt(1), d[0] - x
    if pc == 0:
        pc = -dt(pivmin)
    cnt = int(np.signbit(pc))
    for j in range(1, len(d)):
        pn = (d[j] - x) * pc - e2[j - 1] * pm
        if pn == 0:
            pn = dt(pivmin) if np.signbit(pc) else -dt(pivmin)
        cnt += int(np.signbit(pn) != np.signbit(pc))
        pm, pc = pc, pn
        m = max(abs(pm), abs(pc))
        if m > big:
            pm, pc = pm * small, pc * small
        elif 0 < m < small:
            pm, pc = pm * big, pc * big
    return cnt


def newton_step(d, e2, x) -> float:
    """-p(x) / p'(x) of the characteristic polynomial, both by the three-term
    recurrence."""
    pm, pc, qm, qc = 1.0, d[0] - x, 0.0, -1.0
    for j in range(1, len(d)):
        a, b = d[j] - x, e2[j - 1]
        pn = a * pc - b * pm
        qn = a * qc - (b * qm + pc)
        pm, pc, qm, qc = pc, pn, qc, qn
        m = max(abs(pc), abs(qc), abs(pm), abs(qm))
        if m > 2.0 ** 400:
            pm, pc, qm, qc = (y * 2.0 ** -400 for y in (pm, pc, qm, qc))
        elif 0 < m < 2.0 ** -400:
            pm, pc, qm, qc = (y * 2.0 ** 400 for y in (pm, pc, qm, qc))
    return -pc / qc if qc != 0 else 0.0


def test_fp32_bracket_fp64_polish_matches_lapack():
    eps, eps32 = np.finfo(np.float64).eps, np.finfo(np.float32).eps
    num, pos = molgen.c1_single()[0]
    b = go.Basis(num)
    s = go.overlap(b, pos)
    h = go.core_hamiltonian(b, pos, s, go.coordination_number(num, pos)).h0
    li = np.linalg.inv(np.linalg.cholesky(s))
    a = li @ h @ li.T
    t, _ = scipy.linalg.hessenberg(0.5 * (a + a.T), calc_q=True)
    d, e = np.diag(t).copy(), np.diag(t, -1).copy()
    e2 = np.append(e * e, 0.0)
    ref = scipy.linalg.eigvalsh_tridiagonal(d, e)
    n = len(d)
    radius = np.abs(np.append(0.0, e)) + np.abs(np.append(e, 0.0))
    glo, ghi = float((d - radius).min()), float((d + radius).max())
    tnorm = max(abs(glo), abs(ghi))
    for idx in range(0, n, max(1, n // 12)):
        lo = np.float32(glo - 4 * eps32 * tnorm * n)
        hi = np.float32(ghi + 1.0)
        ftol = np.float32(2 * eps32 * tnorm)
        for _ in range(96):
            if hi - lo <= ftol:
                break
            mid = np.float32(0.5) * (lo + hi)
            if mid <= lo or mid >= hi:
                break
            if sturm_count(d, e2, mid, 1e-37, np.float32) <= idx:
                lo = mid
            else:
                hi = mid
        x = 0.5 * (float(lo) + float(hi))
        assert abs(x - ref[idx]) < 1e-5 * tnorm  # the FP32 bracket
        for _ in range(6):
            dx = newton_step(d, e2, x)
            x += dx
            if not abs(dx) > 4 * eps * tnorm:
                break
        delta = 64 * eps * tnorm
        assert sturm_count(d, e2, x - delta, 1e-300, np.float64) <= idx
        assert idx < sturm_count(d, e2, x + delta, 1e-300, np.float64)
        assert abs(x - ref[idx]) < 1e-13 * tnorm
