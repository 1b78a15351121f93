"""CPU restatement of dxtb's GFN1-xTB single point (energy + forces) in numpy.

TEST INFRASTRUCTURE: this is the oracle.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline legs of ``bench.py`` may
import it, and only as the checker or the timed CPU baseline; the GPU engine
(``dxtb_gb300``) never calls it.

It restates, function by function, the float64 path that dxtb runs for
``GFN1Calculator.get_energy``/``get_forces`` (file:line citations are into the
reference project).  It was pinned against (i) the reference's own golden
files (``test/test_overlap/overlap.npz``, ``test/test_hamiltonian/h0.npz``,
``grad_no_overlap.npz``) and (ii) outputs of the reference itself, run in the
development container through ``oracle/reference_run.py`` and stored under
``tests/golden`` by ``tests/golden/make_golden.py``.

Deliberate choices (all leave the converged result unchanged):
* The generalised eigenproblem is solved with LAPACK ``dsygvd`` (scipy)
  instead of the reference's explicit Cholesky + ``eigh``
  (``scf/unrolling/base.py:141-175``); only invariants (E, q, P) are used.
* Forces use the analytic adjoint of ``calculators/types/analytical.py:63-222``
  instead of autograd through the unrolled SCF (``types/autograd.py:82-201``);
  both give the gradient of the converged free energy.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np
import scipy.linalg

PARAM_FILE = Path(__file__).resolve().parent.parent / "dxtb_gb300" / "data" / "gfn1_params.json"

# --- constants (CODATA 2010; see oracle/shims/tad_mctc/units) --------------
BOHR_AA = 0.52917721092
AA2AU = 1.0 / BOHR_AA
EV2AU = 1.0 / 27.21138505
KELVIN2AU = 1.3806488e-23 / 4.35974434e-18
EPS = float(np.finfo(np.float64).eps)
TINY = float(np.finfo(np.float64).tiny)

INTCUTOFF = 50.0          # integral/driver cutoff, constants/defaults.py:93
REP_CUTOFF = 25.0         # constants/xtb.py:33
CN_CUTOFF = 25.0          # D3 coordination-number cutoff
CN_KCN = 16.0             # D3 counting steepness

# Radii in Angstrom (see oracle/shims/tad_mctc/data/radii.py for sources).
_ATOMIC_RAD = [
    0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60, 0.62,
    1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01,
    2.00, 1.74,
    1.59, 1.48, 1.44, 1.30, 1.29, 1.24, 1.18, 1.17, 1.22, 1.20,
    1.23, 1.20, 1.20, 1.18, 1.17, 1.16,
    2.15, 1.90,
    1.76, 1.64, 1.56, 1.46, 1.38, 1.36, 1.34, 1.30, 1.36, 1.40,
    1.42, 1.40, 1.40, 1.37, 1.32, 1.36,
    2.38, 2.06,
    1.94, 1.84, 1.90, 1.88, 1.86, 1.85, 1.83, 1.82, 1.81, 1.80, 1.79, 1.77, 1.77, 1.78, 1.74,
    1.64, 1.58, 1.50, 1.41, 1.36, 1.32, 1.30, 1.30, 1.32,
    1.44, 1.45, 1.50, 1.42, 1.48, 1.46,
]
_COV_D3 = [
    0.32, 0.46, 1.20, 0.94, 0.77, 0.75, 0.71, 0.63, 0.64, 0.67,
    1.40, 1.25, 1.13, 1.04, 1.10, 1.02, 0.99, 0.96,
    1.76, 1.54,
    1.33, 1.22, 1.21, 1.10, 1.07, 1.04, 1.00, 0.99, 1.01, 1.09,
    1.12, 1.09, 1.15, 1.10, 1.14, 1.17,
    1.89, 1.67,
    1.47, 1.39, 1.32, 1.24, 1.15, 1.13, 1.13, 1.08, 1.15, 1.23,
    1.28, 1.26, 1.26, 1.23, 1.32, 1.31,
    2.09, 1.76,
    1.62, 1.47, 1.58, 1.57, 1.56, 1.55, 1.51, 1.52, 1.51, 1.50, 1.49, 1.49, 1.48, 1.53, 1.46,
    1.37, 1.31, 1.23, 1.18, 1.16, 1.11, 1.12, 1.13, 1.32,
    1.30, 1.30, 1.36, 1.31, 1.38, 1.42,
]
ATOMIC_RADII = np.array([0.0] + _ATOMIC_RAD) * AA2AU
COV_D3 = np.array([0.0] + _COV_D3) * (4.0 / 3.0) * AA2AU

# Cartesian -> real spherical transformation, rows in the reference's
# ordering (integral/driver/pytorch/impls/md/trafo.py:63-90, NLM_CART 165-182).
_S3 = math.sqrt(3.0)
# The reference keeps its double factorials (basis/slater.py:53-55) and this
# table in float32 tensors, so its d shells are normalised with
# 1/float32(sqrt(3)) and the xy-type rows carry float32(sqrt(3)): those two
# roundings cancel, but the d_z2 row (-xx/2 - yy/2 + zz) keeps a factor
# sqrt(3)/float32(sqrt(3)) = 1 + 1.8e-8, which shows in every integral and
# energy of a molecule with d shells.  It is reproduced here.
DZ2_SCALE = _S3 / float(np.float32(np.sqrt(np.float32(3.0))))
CART = {
    0: [(0, 0, 0)],
    1: [(1, 0, 0), (0, 1, 0), (0, 0, 1)],
    2: [(2, 0, 0), (0, 2, 0), (0, 0, 2), (1, 1, 0), (1, 0, 1), (0, 1, 1)],
}
TRAFO = {
    0: np.array([[1.0]]),
    1: np.array([[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]]),  # (y, z, x)
    2: np.array([
        [-0.5 * DZ2_SCALE, -0.5 * DZ2_SCALE, DZ2_SCALE, 0.0, 0.0, 0.0],
        [0.0, 0.0, 0.0, 0.0, _S3, 0.0],
        [0.0, 0.0, 0.0, 0.0, 0.0, _S3],
        [0.5 * _S3, -0.5 * _S3, 0.0, 0.0, 0.0, 0.0],
        [0.0, 0.0, 0.0, _S3, 0.0, 0.0],
    ]),
}
DFACT = [1.0, 1.0, 3.0, 15.0, 105.0]


# ---------------------------------------------------------------------------
# parameters and basis
# ---------------------------------------------------------------------------
_PAR = None


def params() -> dict:
    global _PAR
    if _PAR is None:
        _PAR = json.loads(PARAM_FILE.read_text())
    return _PAR


def _s_overlap(a1, c1, a2, c2) -> float:
    """Overlap of two s-type contractions (basis/ortho.py:36-71)."""
    return float(np.sum((np.pi / (a1[:, None] + a2[None, :])) ** 1.5 * c1[:, None] * c2[None, :]))


def element_basis(z: int) -> list[dict]:
    """Contracted shells of element ``z`` (basis/bas.py:149-193,
    basis/slater.py:69-135, basis/ortho.py:74-110): alpha = alpha_sto*zeta^2,
    primitive norm (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!); a non-valence
    shell is Gram-Schmidt orthogonalised to the shell before it."""
    par = params()
    el = par["elements"][str(z)]
    shells = []
    for sh in el["shells"]:
        coeff0, alpha0 = (np.array(v) for v in par["sto"][sh["sto"]])
        l = sh["l"]
        alpha = alpha0 * sh["slater"] ** 2
        coeff = coeff0 * (2.0 / np.pi * alpha) ** 0.75 * np.sqrt(4.0 * alpha) ** l / np.sqrt(DFACT[l])
        if not sh["valence"]:
            prev = shells[-1]
            ov = _s_overlap(prev["alpha"], prev["coeff"], alpha, coeff)
            alpha = np.concatenate([alpha, prev["alpha"]])
            coeff = np.concatenate([coeff, -ov * prev["coeff"]])
            coeff = coeff / math.sqrt(_s_overlap(alpha, coeff, alpha, coeff))
        shells.append({**sh, "alpha": alpha, "coeff": coeff})
    return shells


@dataclass
class Basis:
    """Atom -> shell -> AO maps for one molecule (basis/indexhelper.py:337-491)."""

    numbers: np.ndarray
    sh_atom: np.ndarray = field(default=None)
    sh_l: np.ndarray = field(default=None)
    sh_ao0: np.ndarray = field(default=None)
    sh_par: list = field(default=None)
    ao_sh: np.ndarray = field(default=None)
    ao_atom: np.ndarray = field(default=None)
    nao: int = 0

    def __post_init__(self):
        sh_atom, sh_l, sh_ao0, sh_par, ao_sh = [], [], [], [], []
        nao = 0
        cache = {}
        for a, z in enumerate(self.numbers):
            z = int(z)
            if z not in cache:
                cache[z] = element_basis(z)
            for sh in cache[z]:
                s = len(sh_atom)
                sh_atom.append(a)
                sh_l.append(sh["l"])
                sh_ao0.append(nao)
                sh_par.append(sh)
                ao_sh.extend([s] * (2 * sh["l"] + 1))
                nao += 2 * sh["l"] + 1
        self.sh_atom = np.array(sh_atom, dtype=np.int64)
        self.sh_l = np.array(sh_l, dtype=np.int64)
        self.sh_ao0 = np.array(sh_ao0, dtype=np.int64)
        self.sh_par = sh_par
        self.ao_sh = np.array(ao_sh, dtype=np.int64)
        self.ao_atom = self.sh_atom[self.ao_sh]
        self.nao = nao

    @property
    def nsh(self) -> int:
        return len(self.sh_atom)


# ---------------------------------------------------------------------------
# overlap (integral/driver/pytorch/impls/overlap.py:147-349)
# ---------------------------------------------------------------------------
def _os1d(lmax_a: int, lmax_b: int, xpa, xpb, oo2p):
    """1D Obara-Saika overlap recursion without the Gaussian prefactor:
    returns E[i][j] for i <= lmax_a, j <= lmax_b (arrays over primitive
    pairs).  Same quantity as the McMurchie-Davidson E^{ij}_0 of
    impls/md/explicit.py:61-187."""
    e = [[None] * (lmax_b + 1) for _ in range(lmax_a + 1)]
    e[0][0] = np.ones_like(xpa)
    for i in range(lmax_a + 1):
        for j in range(lmax_b + 1):
            if i == 0 and j == 0:
                continue
            if i > 0:
                v = xpa * e[i - 1][j]
                if i > 1:
                    v = v + (i - 1) * oo2p * e[i - 2][j]
                if j > 0:
                    v = v + j * oo2p * e[i - 1][j - 1]
            else:
                v = xpb * e[i][j - 1]
                if j > 1:
                    v = v + (j - 1) * oo2p * e[i][j - 2]
            e[i][j] = v
    return e


def shell_pair_block(sha: dict, shb: dict, rab: np.ndarray, grad: bool = False):
    """Spherical overlap block <a(A)|b(B)> for displacement rab = B - A
    (shape (npair, 3)); with ``grad`` also d/dA (shape (npair, 3, na, nb))."""
    la, lb = sha["l"], shb["l"]
    a = sha["alpha"][None, :, None]
    b = shb["alpha"][None, None, :]
    ca = sha["coeff"][None, :, None]
    cb = shb["coeff"][None, None, :]
    p = a + b
    oo2p = 0.5 / p
    r2 = np.sum(rab * rab, axis=-1)[:, None, None]
    pref = np.exp(-a * b / p * r2) * (np.pi / p) ** 1.5 * ca * cb
    la_ext = la + (1 if grad else 0)
    comps = []
    for x in range(3):
        d = rab[:, x][:, None, None]
        xpa = b / p * d        # P - A
        xpb = -a / p * d       # P - B
        comps.append(_os1d(la_ext, lb, xpa, xpb, oo2p))
    ca_list, cb_list = CART[la], CART[lb]
    npair = rab.shape[0]
    s_cart = np.zeros((npair, len(ca_list), len(cb_list)))
    g_cart = np.zeros((npair, 3, len(ca_list), len(cb_list))) if grad else None
    for i, (ix, iy, iz) in enumerate(ca_list):
        for j, (jx, jy, jz) in enumerate(cb_list):
            ex, ey, ez = comps[0][ix][jx], comps[1][iy][jy], comps[2][iz][jz]
            s_cart[:, i, j] = np.sum(pref * ex * ey * ez, axis=(1, 2))
            if grad:
                # d/dA_x of x_A^i e^{-a x_A^2} = 2a x_A^{i+1} - i x_A^{i-1}
                idx = (ix, iy, iz)
                e3 = (ex, ey, ez)
                for x in range(3):
                    lo = comps[x][idx[x] - 1][(jx, jy, jz)[x]] if idx[x] > 0 else 0.0
                    hi = comps[x][idx[x] + 1][(jx, jy, jz)[x]]
                    dx = 2.0 * a * hi - idx[x] * lo
                    others = [e3[k] for k in range(3) if k != x]
                    g_cart[:, x, i, j] = np.sum(pref * dx * others[0] * others[1], axis=(1, 2))
    ta, tb = TRAFO[la], TRAFO[lb]
    s = np.einsum("ai,nij,bj->nab", ta, s_cart, tb)
    if grad:
        g = np.einsum("ai,nxij,bj->nxab", ta, g_cart, tb)
        return s, g
    return s


def overlap(basis: Basis, positions: np.ndarray, grad: bool = False):
    """Full AO overlap matrix.  Blocks between atoms with 0.1 < R < 50 bohr;
    every same-atom block is the identity (impls/overlap.py:186-242)."""
    n = basis.nao
    smat = np.zeros((n, n))
    dmat = np.zeros((n, n, 3)) if grad else None  # d S_mn / d R_atom(m)
    nsh = basis.nsh
    # group shell pairs by (element-shell, element-shell) type to vectorise
    groups: dict = {}
    pos = positions
    for si in range(nsh):
        for sj in range(si + 1, nsh):
            ai, aj = basis.sh_atom[si], basis.sh_atom[sj]
            if ai == aj:
                continue
            d = pos[aj] - pos[ai]
            r = math.sqrt(float(d @ d))
            if not (0.1 < r < INTCUTOFF):
                continue
            key = (id(basis.sh_par[si]), id(basis.sh_par[sj]))
            groups.setdefault(key, []).append((si, sj))
    for pairs in groups.values():
        si0, sj0 = pairs[0]
        sha, shb = basis.sh_par[si0], basis.sh_par[sj0]
        si_arr = np.array([p[0] for p in pairs])
        sj_arr = np.array([p[1] for p in pairs])
        rab = pos[basis.sh_atom[sj_arr]] - pos[basis.sh_atom[si_arr]]
        res = shell_pair_block(sha, shb, rab, grad=grad)
        blk, gblk = (res if grad else (res, None))
        na, nb = 2 * sha["l"] + 1, 2 * shb["l"] + 1
        for k, (si, sj) in enumerate(pairs):
            i0, j0 = basis.sh_ao0[si], basis.sh_ao0[sj]
            smat[i0:i0 + na, j0:j0 + nb] = blk[k]
            smat[j0:j0 + nb, i0:i0 + na] = blk[k].T
            if grad:
                g = np.moveaxis(gblk[k], 0, -1)  # (na, nb, 3) = dS/dA
                dmat[i0:i0 + na, j0:j0 + nb] = g
                dmat[j0:j0 + nb, i0:i0 + na] = -np.swapaxes(g, 0, 1)
    np.fill_diagonal(smat, 1.0)
    return (smat, dmat) if grad else smat


# ---------------------------------------------------------------------------
# coordination number, H0, Coulomb, repulsion
# ---------------------------------------------------------------------------
def distances(positions: np.ndarray):
    diff = positions[:, None, :] - positions[None, :, :]
    return np.sqrt(np.sum(diff * diff, axis=-1)), diff


def coordination_number(numbers, positions, grad: bool = False):
    """Exponential-counting D3 CN (xtb/gfn1.py:62-64 -> tad_mctc cn_d3):
    CN_A = sum_B 1/(1+exp(-16 (R0_AB/R_AB - 1))), R_AB <= 25 bohr.
    With ``grad`` also dCN_A/dR_AB (the radial derivative, (n, n))."""
    n = len(numbers)
    r, _ = distances(positions)
    rc = COV_D3[numbers]
    r0 = rc[:, None] + rc[None, :]
    mask = (~np.eye(n, dtype=bool)) & (r <= CN_CUTOFF)
    rs = np.where(mask, r, 1.0)
    ex = np.exp(-CN_KCN * (r0 / rs - 1.0))
    cn = np.where(mask, 1.0 / (1.0 + ex), 0.0).sum(-1)
    if not grad:
        return cn
    dcn = np.where(mask, -CN_KCN * r0 * ex / (rs * rs * (1.0 + ex) ** 2), 0.0)
    return cn, dcn


def _ksh(shi: dict, shj: dict) -> float:
    """Shell-pair scaling K_ll' (xtb/gfn1.py:66-165)."""
    par = params()
    lab = "spdfg"

    def kii(sh):
        if not sh["valence"]:
            return par["kpol"]
        return par["shell"].get(lab[sh["l"]] * 2, 1.0)

    if shi["valence"] and shj["valence"]:
        k1 = lab[shi["l"]] + lab[shj["l"]]
        k2 = lab[shj["l"]] + lab[shi["l"]]
        if k1 in par["shell"]:
            return par["shell"][k1]
        if k2 in par["shell"]:
            return par["shell"][k2]
    return 0.5 * (kii(shi) + kii(shj))


def kpair(za: int, zb: int) -> float:
    return params()["kpair"].get(f"{min(za, zb)}-{max(za, zb)}", 1.0)


@dataclass
class H0Terms:
    h0: np.ndarray          # core Hamiltonian (N, N)
    hsh: np.ndarray         # shell self-energies h_i (CN shifted)
    ksh_pi: np.ndarray      # off-site factor K * X * Pi per shell pair (nsh, nsh), 1 on-site
    dpi_over_pi: np.ndarray  # (dPi/dR)/(Pi R) per shell pair (nsh, nsh)


def core_hamiltonian(basis: Basis, positions, smat, cn) -> H0Terms:
    """GFN1 H0 (xtb/base.py:251-360 with xtb/gfn1.py:66-183)."""
    par = params()
    numbers = basis.numbers
    nsh = basis.nsh
    r, _ = distances(positions)
    rad = ATOMIC_RADII[numbers]
    en = np.array([par["elements"][str(int(z))]["en"] for z in numbers])
    level = np.array([sh["level"] for sh in basis.sh_par]) * EV2AU
    kcn = np.array([sh["kcn"] for sh in basis.sh_par]) * EV2AU
    shpoly = np.array([sh["shpoly"] for sh in basis.sh_par])
    hsh = level - kcn * cn[basis.sh_atom]
    fac = np.ones((nsh, nsh))
    dpi = np.zeros((nsh, nsh))
    for i in range(nsh):
        a = basis.sh_atom[i]
        for j in range(nsh):
            b = basis.sh_atom[j]
            if a == b:
                continue
            rr = math.sqrt(r[a, b] / (rad[a] + rad[b]))
            pa, pb = 1.0 + shpoly[i] * rr, 1.0 + shpoly[j] * rr
            pi = pa * pb
            shi, shj = basis.sh_par[i], basis.sh_par[j]
            k = _ksh(shi, shj)
            if shi["valence"] and shj["valence"]:
                x = 1.0 + par["enscale"] * (en[a] - en[b]) ** 2
                k = k * kpair(int(numbers[a]), int(numbers[b])) * x
            fac[i, j] = pi * k
            dpi[i, j] = (pa * shpoly[j] + pb * shpoly[i]) * rr * 0.5 / (r[a, b] * r[a, b]) / pi
    hvar = 0.5 * (hsh[:, None] + hsh[None, :])
    hfull = (fac * hvar)[basis.ao_sh][:, basis.ao_sh]
    h0 = hfull * smat
    h0 = 0.5 * (h0 + h0.T)
    return H0Terms(h0=h0, hsh=hsh, ksh_pi=fac, dpi_over_pi=dpi)


def gamma_matrix(basis: Basis, positions) -> np.ndarray:
    """Shell-resolved ES2 matrix (coulomb/secondorder.py:799-870, gexp = 2,
    harmonic average coulomb/average.py:41-56), including the reference's
    machine-epsilon guards."""
    par = params()
    numbers = basis.numbers
    r, _ = distances(positions)
    gam = np.array([par["elements"][str(int(z))]["gam"] for z in numbers])
    lgam = np.array([sh["lgam"] for sh in basis.sh_par])
    h = lgam * gam[basis.sh_atom] + EPS
    avg = 2.0 / (1.0 / h[:, None] + 1.0 / h[None, :])
    at = basis.sh_atom
    same = at[:, None] == at[None, :]
    d2 = np.where(same, EPS, (r[at][:, at] + EPS) ** 2)
    return 1.0 / np.sqrt(d2 + avg ** -2.0)


def repulsion(numbers, positions, grad: bool = False):
    """GFN1 repulsion (classicals/repulsion/base.py:269-406, rep.py:60-95):
    E_AB = Z_A Z_B exp(-sqrt(a_A a_B) R^1.5) / R for R <= 25 bohr, each pair
    counted once."""
    par = params()
    n = len(numbers)
    r, diff = distances(positions)
    arep = np.array([par["elements"][str(int(z))]["arep"] for z in numbers])
    zeff = np.array([par["elements"][str(int(z))]["zeff"] for z in numbers])
    kexp = par["kexp"]
    mask = (~np.eye(n, dtype=bool)) & (r <= REP_CUTOFF)
    rs = np.where(mask, r, 1.0)
    a = np.sqrt(arep[:, None] * arep[None, :] + TINY)
    r1k = rs ** kexp
    e = np.where(mask, zeff[:, None] * zeff[None, :] * np.exp(-a * r1k) / rs, 0.0)
    eat = 0.5 * e.sum(-1)
    if not grad:
        return eat
    dedr = -(a * r1k * kexp + 1.0) * e / (rs * rs)   # (dE/dR)/R
    g = np.einsum("ab,abx->ax", dedr, diff)
    return eat, g


XB_DONORS = (17, 35, 53, 85)       # components/classicals/halogen/hal.py:117
XB_ACCEPTORS = (7, 8, 15, 16)      # hal.py:118
XB_CUTOFF = 20.0                   # constants/xtb.py:33


def halogen_bond(numbers, positions, grad: bool = False):
    """GFN1 halogen-bond correction (classicals/halogen/hal.py:168-364).
    Triples (X, J, K): donor X, acceptor J within the cutoff (hal.py:213-226)
    and the atom K nearest to X at a non-zero distance, first of equals
    (hal.py:235-246).  E_X += xbond_X lj fdamp with lj = (s^12 - damp s^6) /
    (1 + s^12), s = rscale (R_X + R_J) / R_XJ and fdamp = (0.5 - 0.25
    cosa)^6, cosa = (d_XK^2 + d_XJ^2 - d_KJ^2) / (d_XK d_XJ) (hal.py:
    321-359).  The gradient is that expression differentiated by hand."""
    par = params()
    hal = par["halogen"]
    numbers = np.asarray(numbers)
    pos = np.asarray(positions, dtype=np.float64)
    n = len(numbers)
    eat = np.zeros(n)
    g = np.zeros((n, 3))
    rads = ATOMIC_RADII[numbers] * hal["rscale"]
    for x in range(n):
        zx = int(numbers[x])
        if zx not in XB_DONORS:
            continue
        xb = par["elements"][str(zx)].get("xbond", 0.0)
        # nearest neighbour of the donor (hal.py:235-246)
        k, dist = 0, np.finfo(np.float64).max
        for b in range(n):
            r1 = float(np.linalg.norm(pos[x] - pos[b]))
            if 0.0 < r1 < dist:
                k, dist = b, r1
        for j in range(n):
            if int(numbers[j]) not in XB_ACCEPTORS or np.linalg.norm(pos[x] - pos[j]) > XB_CUTOFF:
                continue
            u, v = pos[j] - pos[x], pos[k] - pos[x]
            d2xj, d2xk, d2kj = u @ u, v @ v, (pos[k] - pos[j]) @ (pos[k] - pos[j])
            rxj = np.sqrt(d2xj)
            s = (rads[x] + rads[j]) / rxj
            s6 = s ** 6
            s12 = s6 * s6
            lj = (s12 - hal["damping"] * s6) / (1.0 + s12)
            cosa = (d2xk + d2xj - d2kj) / np.sqrt(d2xk * d2xj)
            h = 0.5 - 0.25 * cosa
            eat[x] += xb * lj * h ** 6
            if grad:
                rv = np.sqrt(d2xk)
                c = 0.5 * cosa  # cosine of the angle J-X-K
                dlj = -(12 * s12 - 6 * hal["damping"] * s6 + 6 * hal["damping"] * s6 * s12) / (
                    rxj * (1.0 + s12) ** 2)
                dfd = -3.0 * h ** 5  # d h^6 / d c, with h = 0.5 - 0.5 c
                dcdu = v / (rxj * rv) - c * u / d2xj
                dcdv = u / (rxj * rv) - c * v / d2xk
                du = xb * (dlj * u / rxj * h ** 6 + lj * dfd * dcdu)
                dv = xb * lj * dfd * dcdv
                g[j] += du
                g[k] += dv
                g[x] -= du + dv
    return (eat, g) if grad else eat


# ---------------------------------------------------------------------------
# SCF pieces
# ---------------------------------------------------------------------------
def reference_occupation(basis: Basis, chrg: float, spin):
    """n0 per AO and (n_alpha, n_beta) (scf/iterator.py:147-189,
    wavefunction/filling.py:41-113)."""
    refocc = np.array([sh["refocc"] for sh in basis.sh_par])
    nao_sh = 2 * basis.sh_l + 1
    n0 = (refocc / nao_sh)[basis.ao_sh]
    nel = round(float(n0.sum() - chrg))
    if spin is None:
        uhf = nel % 2
    else:
        uhf = int(spin)
        if uhf % 2 != nel % 2:
            uhf = nel % 2
    uhf = min(uhf, nel)
    nb = (nel - uhf) / 2.0
    na = nb + uhf
    return n0, np.array([na, nb])


def fermi_occupation(emo: np.ndarray, nab: np.ndarray, kt: float, maxiter: int = 200,
                     thr: float | None = None):
    """Fermi-Dirac occupations per spin channel, Newton on E_F from the
    HOMO/LUMO midpoint until |sum f - n| <= sqrt(eps) in every channel
    (wavefunction/filling.py:201-366).  ``thr`` overrides the reference's
    threshold sqrt(eps) (finite-difference checks use a tighter one: the
    electron-count error of sqrt(eps) moves the energy by ~1e-8 Eh)."""
    nmo = emo.shape[0]
    thr = math.sqrt(EPS) if thr is None else thr
    res = 5.0 * 1e-15  # 5 * finfo(float64).resolution
    emos, efs, targets, nonempty = [], [], [], []
    for nel in nab:
        occ_cs = np.arange(1, nmo + 1, dtype=np.float64) - nel
        homo = int(np.argmax(occ_cs >= -res))
        if nel != 0:
            lumo = homo if nmo - 1 <= homo else homo + 1
            ef = 0.5 * (emo[homo] + emo[lumo])
        else:
            ef = 0.0
        emos.append(emo if nel != 0 else np.zeros_like(emo))
        efs.append(ef)
        targets.append(homo + 1.0)
        nonempty.append(nel != 0)
    efs = np.array(efs)
    for _ in range(maxiter):
        occ, done = [], True
        for s in range(len(nab)):
            x = (emos[s] - efs[s]) / kt
            small = x < 50.0
            et = np.exp(np.where(small, x, 0.0))
            f = np.where(small, 1.0 / (et + 1.0), 0.0)
            df = np.where(small, et / (kt * (et + 1.0) ** 2), EPS)
            err = targets[s] - f.sum()
            efs[s] += err / df.sum()
            if abs(err) > thr:
                done = False
            occ.append(f if nonempty[s] else np.zeros_like(f))
        if done:
            return np.array(occ)
    raise RuntimeError("Fermi energy failed to converge.")


def free_energy(occ: np.ndarray, kt: float) -> float:
    """-TS summed over channels and orbitals (scf/base.py:558-623)."""
    o = np.maximum(occ, EPS)
    o1 = np.maximum(1.0 - occ, EPS)
    return float(np.sum(np.log(o ** o * o1 ** o1)) * kt)


class Anderson:
    """Anderson/Eyert mixer with soft start, as run by the reference in full
    SCF mode (scf/mixer/anderson.py:102-317, defaults.py:143-175)."""

    def __init__(self, generations=5, damp=0.5, damp_init=0.1, offset=0.01):
        self.g, self.damp, self.damp_init, self.offset = generations, damp, damp_init, offset
        self.step = 0
        self.x_hist = None
        self.f = None
        self.delta = None

    def iter(self, x_new, x_old):
        if self.step == 0:
            self.x_hist = np.zeros((self.g + 1, x_new.size))
            self.f = np.zeros((self.g + 1, x_new.size))
            self.x_hist[0] = x_old
        self.step += 1
        self.f[0] = x_new - x_old
        if self.step > self.g:
            n = min(self.step - 1, self.g)
            df = self.f[0] - self.f[1:n + 1]
            a = df @ df.T
            b = df @ self.f[0]
            a[np.diag_indices(n)] *= 1.0 + self.offset ** 2
            th = np.linalg.solve(a, b)
            x_bar = th @ (self.x_hist[1:n + 1] - self.x_hist[0]) + self.x_hist[0]
            f_bar = th @ (-df) + self.f[0]
            x_mix = x_bar + self.damp * f_bar
        else:
            x_mix = self.x_hist[0] + self.f[0] * self.damp_init
        self.f = np.roll(self.f, 1, axis=0)
        self.x_hist = np.roll(self.x_hist, 1, axis=0)
        self.x_hist[0] = x_mix
        self.delta = self.f[1].copy()
        return x_mix

    def converged(self, x_atol, x_atol_max) -> bool:
        return bool(np.linalg.norm(self.delta) < x_atol and np.max(np.abs(self.delta)) < x_atol_max)


@dataclass
class Result:
    energy: float
    energy_atoms: np.ndarray
    e_rep: float
    e_h0: float
    e_es2: float
    e_es3: float
    e_fermi: float
    charges: np.ndarray
    iterations: int
    converged: bool
    forces: np.ndarray | None = None
    emo: np.ndarray | None = None
    charges_orbital: np.ndarray | None = None  # q per AO before the reduction to atoms


class Broyden:
    """Modified Broyden mixer (Johnson, Phys. Rev. B 38, 12807 (1988)) as run
    by the GPU engine: step alpha, weights 1, w0 = 0.01, ``memory`` most
    recent difference pairs."""

    def __init__(self, alpha=0.2, memory=20, w0=0.01):
        self.alpha, self.memory, self.w0 = alpha, memory, w0
        self.df: list = []
        self.u: list = []
        self.xprev = None
        self.fprev = None

    def step(self, x, f):
        if self.xprev is None:
            self.xprev, self.fprev = x.copy(), f.copy()
            return x + self.alpha * f
        dfv = f - self.fprev
        nrm = float(np.sqrt(dfv @ dfv))
        inv = 1.0 / nrm if nrm > 0.0 else 0.0
        self.df.append(dfv * inv)
        self.u.append(self.alpha * dfv * inv + (x - self.xprev) * inv)
        if len(self.df) > self.memory:
            self.df.pop(0)
            self.u.pop(0)
        d = np.array(self.df)
        a = d @ d.T + self.w0 ** 2 * np.eye(len(self.df))
        gam = np.linalg.solve(a, d @ f)
        self.xprev, self.fprev = x.copy(), f.copy()
        return x + self.alpha * f - gam @ np.array(self.u)


def singlepoint(numbers, positions, chrg: float = 0.0, spin=None, forces: bool = True,
                etemp: float = 300.0, maxiter: int = 300, x_atol: float = 1e-10,
                x_atol_max: float = 1e-10, mixer: str = "anderson",
                broyden_alpha: float = 0.2, broyden_memory: int = 20,
                v_init: np.ndarray | None = None, fermi_thr: float | None = None) -> Result:
    """GFN1 single point without dispersion (calculators/types/energy.py:78-402).

    ``mixer="anderson"`` replays the reference's single-system SCF loop
    (scf/unrolling/default.py:71-136) step for step; ``mixer="broyden"``
    replays the GPU engine's loop.  Both stop on the reference's test of the
    potential change and take the final charges from the last unmixed
    output potential, so both reach the same fixed point.  ``v_init``
    (orbital-resolved potential) restarts the Broyden loop from a given
    potential instead of zero, which checks that a state is a fixed point."""
    numbers = np.asarray(numbers, dtype=np.int64)
    positions = np.asarray(positions, dtype=np.float64)
    basis = Basis(numbers)
    par = params()
    kt = etemp * KELVIN2AU

    # classical terms: repulsion and halogen bond
    if forces:
        erep_at, grad_rep = repulsion(numbers, positions, grad=True)
        exb_at, grad_xb = halogen_bond(numbers, positions, grad=True)
        grad_rep = grad_rep + grad_xb
    else:
        erep_at = repulsion(numbers, positions)
        exb_at = halogen_bond(numbers, positions)
    erep_at = erep_at + exb_at

    # integrals
    if forces:
        smat, dsmat = overlap(basis, positions, grad=True)
        cn, dcn = coordination_number(numbers, positions, grad=True)
    else:
        smat = overlap(basis, positions)
        cn = coordination_number(numbers, positions)
    h0t = core_hamiltonian(basis, positions, smat, cn)
    h0 = h0t.h0
    gam = gamma_matrix(basis, positions)
    gam3 = np.array([par["elements"][str(int(z))]["gam3"] for z in numbers])
    n0, nab = reference_occupation(basis, chrg, spin)
    # Cholesky reduction of the generalised eigenproblem (scf/unrolling/base.py:141-175)
    linv = scipy.linalg.solve_triangular(np.linalg.cholesky(smat), np.eye(basis.nao), lower=True)

    ao_sh, sh_atom = basis.ao_sh, basis.sh_atom
    nsh, nat = basis.nsh, len(numbers)

    def reduce_sh(x):
        return np.bincount(ao_sh, weights=x, minlength=nsh)

    def reduce_at(x):
        return np.bincount(sh_atom, weights=x, minlength=nat)

    state = {}

    def pot_to_charges(v):
        f = h0 - 0.5 * smat * (v[:, None] + v[None, :])
        fp = linv @ f @ linv.T
        emo, u = np.linalg.eigh(0.5 * (fp + fp.T))
        c = linv.T @ u
        occ = fermi_occupation(emo, nab, kt, thr=fermi_thr)
        p = (c * occ.sum(0)) @ c.T
        q = n0 - np.einsum("ij,ji->i", p, smat)
        state.update(emo=emo, c=c, occ=occ, p=p, q=q)
        return q

    def charges_to_pot(q):
        qsh = reduce_sh(q)
        qat = reduce_at(qsh)
        vsh = gam @ qsh + (gam3 * qat * qat)[sh_atom]
        return vsh[ao_sh]

    converged = False
    it = 0
    if mixer == "anderson":
        mix = Anderson()
        v_guess = np.zeros(basis.nao)
        v_new = charges_to_pot(pot_to_charges(v_guess))
        v = mix.iter(v_new, v_guess)
        for it in range(1, maxiter + 1):
            v_new = charges_to_pot(pot_to_charges(v))
            v = mix.iter(v_new, v)
            if mix.converged(x_atol, x_atol_max):
                converged = True
                break
        it += 1
    elif mixer == "broyden":
        mix = Broyden(broyden_alpha, broyden_memory)
        v = np.zeros(basis.nao) if v_init is None else np.asarray(v_init, dtype=np.float64).copy()
        while True:
            v_new = charges_to_pot(pot_to_charges(v))
            f = v_new - v
            if it > 0 and np.linalg.norm(f) < x_atol and np.max(np.abs(f)) < x_atol_max:
                converged = True
                break
            if it >= maxiter:
                break
            v = mix.step(v, f)
            it += 1
        it += 1
    else:
        raise ValueError(f"unknown mixer {mixer!r}")
    # final charges from the unmixed last potential (scf/unrolling/default.py:111-114)
    q = pot_to_charges(v_new)
    p = state["p"]
    qsh = reduce_sh(q)
    qat = reduce_at(qsh)
    e_h0_ao = np.einsum("ij,ji->i", p, h0)
    e_h0 = reduce_at(reduce_sh(e_h0_ao))
    e_es2 = reduce_at(0.5 * qsh * (gam @ qsh))
    e_es3 = gam3 * qat ** 3 / 3.0
    g = free_energy(state["occ"], kt)
    e_fermi = np.full(nat, g / nat)
    eat = erep_at + e_h0 + e_es2 + e_es3 + e_fermi
    res = Result(
        energy=float(eat.sum()), energy_atoms=eat, e_rep=float(erep_at.sum()),
        e_h0=float(e_h0.sum()), e_es2=float(e_es2.sum()), e_es3=float(e_es3.sum()),
        e_fermi=g, charges=qat, iterations=it, converged=converged, emo=state["emo"],
        charges_orbital=q,
    )
    if forces:
        v_orb = charges_to_pot(q)
        res.forces = -_gradient(basis, positions, smat, dsmat, h0t, cn, dcn, state, v_orb,
                                qsh, grad_rep)
    return res


def _gradient(basis, positions, smat, dsmat, h0t, cn, dcn, state, v_orb, qsh, grad_rep):
    """Analytic gradient of the converged free energy
    (calculators/types/analytical.py:63-222, xtb/gfn1.py:185-408,
    coulomb/secondorder.py:873-926, ncoord/utils.py:31-52)."""
    par = params()
    numbers = basis.numbers
    nat = len(numbers)
    c, occ, emo, p = state["c"], state["occ"], state["emo"], state["p"]
    w = (c * (occ.sum(0) * emo)) @ c.T
    ao_atom, ao_sh, sh_atom = basis.ao_atom, basis.ao_sh, basis.sh_atom
    r, diff = distances(positions)
    rsafe = np.where(r > 0, r, 1.0)

    grad = grad_rep.copy()

    # overlap-derivative contraction: sum_{m in A, n not in A} X_mn dS_mn/dA
    htil = (h0t.ksh_pi * 0.5 * (h0t.hsh[:, None] + h0t.hsh[None, :]))[ao_sh][:, ao_sh]
    x = 2.0 * p * htil - 2.0 * w - p * (v_orb[:, None] + v_orb[None, :])
    offat = ao_atom[:, None] != ao_atom[None, :]
    x = np.where(offat, x, 0.0)
    gs = np.einsum("mn,mnx->mx", x, dsmat)
    np.add.at(grad, ao_atom, gs)

    # distance polynomial: 2 sum P H0 (dPi/dR)/Pi (R_A - R_B)/R
    ph0 = p * h0t.h0
    ph_sh = np.zeros((basis.nsh, basis.nsh))
    np.add.at(ph_sh, (ao_sh[:, None], ao_sh[None, :]), ph0)
    dpi_sh = 2.0 * ph_sh * h0t.dpi_over_pi
    dpi_at = np.zeros((nat, nat))
    np.add.at(dpi_at, (sh_atom[:, None], sh_atom[None, :]), dpi_sh)
    grad += np.einsum("ab,abx->ax", dpi_at, diff)

    # coordination number: dE/dCN_A = -sum_{i in A} kcn_i sum_{m in i, n} P S K X Pi
    kcn = np.array([sh["kcn"] for sh in basis.sh_par]) * EV2AU
    psf = p * smat * h0t.ksh_pi[ao_sh][:, ao_sh]
    dedh = np.bincount(ao_sh, weights=psf.sum(1), minlength=basis.nsh)
    dedcn = np.bincount(sh_atom, weights=-kcn * dedh, minlength=nat)
    # dCN_A/dR_A = sum_B dcn_AB (R_A - R_B)/R ; dCN_B/dR_A = dcn_AB (R_A - R_B)/R
    fac = dcn / rsafe * (dedcn[:, None] + dedcn[None, :])
    grad += np.einsum("ab,abx->ax", fac, diff)

    # ES2: q_i q_j dgamma_ij/dR with gamma = ((R+eps)^2 + avg^-2)^(-1/2)
    gam = gamma_matrix(basis, positions)
    at = sh_atom
    off = at[:, None] != at[None, :]
    rsh = r[at][:, at]
    dg = np.where(off, -(rsh + EPS) * gam ** 3, 0.0)
    t = qsh[:, None] * qsh[None, :] * dg
    t_at = np.zeros((nat, nat))
    np.add.at(t_at, (at[:, None], at[None, :]), t)
    grad += np.einsum("ab,abx->ax", t_at / rsafe, diff)
    return grad
