// Geometry-dependent terms of GFN1-xTB: coordination numbers, repulsion,
// contracted-Gaussian overlap S, core Hamiltonian H0, shell-resolved Coulomb
// matrix gamma, and the hand-written adjoint of all of them for forces.
//
// Reference behaviour reproduced (dxtb, src/dxtb/_src/...):
//   CN            xtb/gfn1.py:62-64 (D3 counting, exponential, 25 bohr cutoff)
//   repulsion     components/classicals/repulsion/base.py:173-406, rep.py:60-95
//   halogen bond  components/classicals/halogen/hal.py:168-364 (donors Cl, Br,
//                 I, At; acceptors N, O, P, S within 20 bohr; the donor's
//                 nearest atom sets the angle), with its analytic gradient
//   overlap       integral/driver/pytorch/impls/overlap.py:147-243 (pairs with
//                 0.1 < R < 50 bohr; same-atom blocks are the identity),
//                 impls/md/explicit.py:61-187, impls/md/trafo.py:63-182
//   H0            xtb/base.py:251-360, xtb/gfn1.py:66-183
//   gamma         components/interactions/coulomb/secondorder.py:799-870,
//                 coulomb/average.py:41-56
//   gradients     xtb/gfn1.py:185-408, impls/overlap.py:246-349,
//                 coulomb/secondorder.py:873-926, ncoord/utils.py:31-52
//
// Every thread of the shell-pair kernels owns one unordered shell pair and
// evaluates its primitive-pair sum with the Obara-Saika recursion in
// registers (l <= 2), so S, H0 and gamma are produced in one pass and dS/dR
// is never stored: the force kernel recomputes it and contracts it on the
// fly with the density-derived weights.
#include "internal.cuh"

#include <cmath>
#include <math_constants.h>

namespace gbxtb {

namespace {

constexpr double kEps = 2.220446049250313e-16;
constexpr double kTiny = 2.2250738585072014e-308;

__device__ __forceinline__ int ncart(int l) { return (l + 1) * (l + 2) / 2; }

// Cartesian exponents in the order xx, yy, zz, xy, xz, yz (d), x, y, z (p).
__device__ __forceinline__ void cart_exp(int l, int c, int &ex, int &ey, int &ez) {
  if (l == 0) { ex = ey = ez = 0; return; }
  if (l == 1) { ex = (c == 0); ey = (c == 1); ez = (c == 2); return; }
  const int tx[6] = {2, 0, 0, 1, 1, 0}, ty[6] = {0, 2, 0, 1, 0, 1}, tz[6] = {0, 0, 2, 0, 1, 1};
  ex = tx[c]; ey = ty[c]; ez = tz[c];
}

// Cartesian -> real spherical for one index: p ordered (y, z, x); d ordered
// (z2, xz, yz, x2-y2, xy) with the normalisation of trafo.py:63-90.  The
// reference keeps its double factorials (basis/slater.py:53-55) and that
// table in float32: its d shells are normalised with 1/float32(sqrt(3)) and
// the xy-type rows carry float32(sqrt(3)), which cancel, but its d_z2
// function keeps a factor sqrt(3)/float32(sqrt(3)) = 1 + 1.8e-8 (kDz2).  It
// is reproduced, since every d-shell integral and energy carries it.
__device__ __forceinline__ void to_sph(int l, const double *c, double *s) {
  if (l == 0) { s[0] = c[0]; return; }
  if (l == 1) { s[0] = c[1]; s[1] = c[2]; s[2] = c[0]; return; }
  const double s3 = 1.7320508075688772, s3h = 0.8660254037844386;
  const double kDz2 = 1.0000000179482318;  // sqrt(3) / float32(sqrt(3))
  s[0] = (-0.5 * c[0] - 0.5 * c[1] + c[2]) * kDz2;
  s[1] = s3 * c[4];
  s[2] = s3 * c[5];
  s[3] = s3h * (c[0] - c[1]);
  s[4] = s3 * c[3];
}

struct ShellView {
  int l, np, valence;
  const double *alpha, *coeff;
  double level, kcn, shpoly, refocc, lgam;
};

__device__ __forceinline__ ShellView shell_view(const DevParams &p, int rec) {
  ShellView v;
  const int32_t *si = p.shell_int + (size_t)rec * GBXTB_SHELL_INTS;
  const double *sd = p.shell_data + (size_t)rec * GBXTB_SHELL_DOUBLES;
  v.l = si[0]; v.np = si[1]; v.valence = si[2];
  v.alpha = sd; v.coeff = sd + 8;
  v.level = sd[16]; v.kcn = sd[17]; v.shpoly = sd[18]; v.refocc = sd[19]; v.lgam = sd[20];
  return v;
}

// Overlap block <i(A)|j(B)> (spherical, row-major [2li+1][2lj+1]) for
// r = B - A, and optionally its derivative with respect to A.
template <bool kGrad>
__device__ void overlap_block(const ShellView &si, const ShellView &sj, double rx, double ry,
                              double rz, double *sblk, double *gblk /* [3][25] */) {
  const int li = si.l, lj = sj.l;
  const int nci = ncart(li), ncj = ncart(lj);
  double sc[6][6];
  double gc[kGrad ? 3 : 1][6][6];
#pragma unroll
  for (int a = 0; a < 6; ++a)
#pragma unroll
    for (int b = 0; b < 6; ++b) {
      sc[a][b] = 0.0;
#pragma unroll
      for (int x = 0; x < (kGrad ? 3 : 1); ++x) gc[x][a][b] = 0.0;
    }
  const double r2 = rx * rx + ry * ry + rz * rz;
  const double rv[3] = {rx, ry, rz};
  const int limax = li + (kGrad ? 1 : 0);
  for (int pa = 0; pa < si.np; ++pa) {
    const double a = si.alpha[pa], ca = si.coeff[pa];
    for (int pb = 0; pb < sj.np; ++pb) {
      const double b = sj.alpha[pb], cb = sj.coeff[pb];
      const double pp = a + b, oop = 1.0 / pp, oo2p = 0.5 * oop;
      const double est = a * b * oop * r2;
      const double pref = exp(-est) * (3.14159265358979323846 * oop) *
                          sqrt(3.14159265358979323846 * oop) * ca * cb;
      if (pref == 0.0) continue;
      // 1D recursion tables E[dim][i][j], i <= li+1, j <= lj
      double E[3][4][3];
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double xpa = b * oop * rv[x], xpb = -a * oop * rv[x];
        E[x][0][0] = 1.0;
        for (int j = 1; j <= lj; ++j)
          E[x][0][j] = xpb * E[x][0][j - 1] + (j > 1 ? (j - 1) * oo2p * E[x][0][j - 2] : 0.0);
        for (int i = 1; i <= limax; ++i)
          for (int j = 0; j <= lj; ++j) {
            double v = xpa * E[x][i - 1][j];
            if (i > 1) v += (i - 1) * oo2p * E[x][i - 2][j];
            if (j > 0) v += j * oo2p * E[x][i - 1][j - 1];
            E[x][i][j] = v;
          }
      }
      for (int ca_ = 0; ca_ < nci; ++ca_) {
        int ix, iy, iz;
        cart_exp(li, ca_, ix, iy, iz);
        for (int cb_ = 0; cb_ < ncj; ++cb_) {
          int jx, jy, jz;
          cart_exp(lj, cb_, jx, jy, jz);
          const double ex = E[0][ix][jx], ey = E[1][iy][jy], ez = E[2][iz][jz];
          sc[ca_][cb_] += pref * ex * ey * ez;
          if (kGrad) {
            const double dx = 2.0 * a * E[0][ix + 1][jx] - (ix > 0 ? ix * E[0][ix - 1][jx] : 0.0);
            const double dy = 2.0 * a * E[1][iy + 1][jy] - (iy > 0 ? iy * E[1][iy - 1][jy] : 0.0);
            const double dz = 2.0 * a * E[2][iz + 1][jz] - (iz > 0 ? iz * E[2][iz - 1][jz] : 0.0);
            gc[0][ca_][cb_] += pref * dx * ey * ez;
            gc[kGrad ? 1 : 0][ca_][cb_] += pref * ex * dy * ez;
            gc[kGrad ? 2 : 0][ca_][cb_] += pref * ex * ey * dz;
          }
        }
      }
    }
  }
  const int ni = 2 * li + 1, nj = 2 * lj + 1;
  // transform rows then columns
  for (int comp = 0; comp < (kGrad ? 4 : 1); ++comp) {
    double tmp[5][6];
    for (int cb_ = 0; cb_ < ncj; ++cb_) {
      double col[6], out[5];
      for (int ca_ = 0; ca_ < nci; ++ca_) col[ca_] = comp == 0 ? sc[ca_][cb_] : gc[kGrad ? comp - 1 : 0][ca_][cb_];
      to_sph(li, col, out);
      for (int a2 = 0; a2 < ni; ++a2) tmp[a2][cb_] = out[a2];
    }
    double *dst = comp == 0 ? sblk : gblk + (comp - 1) * 25;
    for (int a2 = 0; a2 < ni; ++a2) {
      double out[5];
      to_sph(lj, tmp[a2], out);
      for (int b2 = 0; b2 < nj; ++b2) dst[a2 * nj + b2] = out[b2];
    }
  }
}

// Shell-pair scaling K_ll' (xtb/gfn1.py:66-165).
__device__ __forceinline__ double shell_k(const DevParams &p, const ShellView &a, const ShellView &b) {
  const double kpol = p.g[0];
  auto kii = [&](const ShellView &s) -> double {
    if (!s.valence) return kpol;
    if (s.l == 0) return p.g[2];
    if (s.l == 1) return p.g[3];
    if (s.l == 2) return p.g[4];
    return 1.0;
  };
  if (a.valence && b.valence) {
    if (a.l == b.l) return kii(a);
    if ((a.l == 0 && b.l == 1) || (a.l == 1 && b.l == 0)) return p.g[5];
  }
  return 0.5 * (kii(a) + kii(b));
}

// Locate the molecule owning global index `idx` given prefix offsets.
__device__ __forceinline__ int find_mol_pair(const MolDesc *mol, int nmol, int64_t idx) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mol[mid].pair0 <= idx) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Decode unordered pair index k (0-based, i <= j) of an n-shell molecule.
__device__ __forceinline__ void decode_pair(int64_t k, int n, int &i, int &j) {
  // rows i have (n - i) entries: offset(i) = i*n - i*(i-1)/2
  double disc = (2.0 * n + 1.0) * (2.0 * n + 1.0) - 8.0 * (double)k;
  int ii = (int)floor(((2.0 * n + 1.0) - sqrt(disc)) * 0.5);
  if (ii < 0) ii = 0;
  if (ii > n - 1) ii = n - 1;
  while (ii > 0 && (int64_t)ii * n - (int64_t)ii * (ii - 1) / 2 > k) --ii;
  while (ii < n - 1 && (int64_t)(ii + 1) * n - (int64_t)(ii + 1) * ii / 2 <= k) ++ii;
  const int64_t off = (int64_t)ii * n - (int64_t)ii * (ii - 1) / 2;
  i = ii;
  j = ii + (int)(k - off);
}

// ---------------------------------------------------------------------------
// halogen bond (hal.py:168-364).  For a donor X (Cl, Br, I, At) with bond
// strength xb, every acceptor J (N, O, P, S) within the cutoff and the atom K
// nearest to X (the first of equals, at a non-zero distance) contribute
//   E_X += xb lj(R_XJ) ((1 - c) / 2)^6,   c = cos(angle J-X-K),
//   lj(R) = (s^12 - damp s^6) / (1 + s^12),  s = rscale (R_X + R_J) / R
// (the reference writes (1 - c) / 2 as 0.5 - 0.25 cosa, cosa = 2c by the
// rule of cosines).
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool xb_donor(int z) { return z == 17 || z == 35 || z == 53 || z == 85; }
__device__ __forceinline__ bool xb_acceptor(int z) { return z == 7 || z == 8 || z == 15 || z == 16; }

// Nearest atom to donor a of molecule md (hal.py:241-250); the molecule's
// first atom if none lies at a non-zero distance.
__device__ int xb_nearest(const MolDesc &md, const double *__restrict__ pos, int a) {
  int best = md.atom0;
  double dist = 1.79769313486231570e308;
  for (int ib = 0; ib < md.natom; ++ib) {
    const int b = md.atom0 + ib;
    const double dx = pos[3 * b] - pos[3 * a], dy = pos[3 * b + 1] - pos[3 * a + 1],
                 dz = pos[3 * b + 2] - pos[3 * a + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    if (0.0 < r && r < dist) {
      best = b;
      dist = r;
    }
  }
  return best;
}

// One donor-acceptor term; with grad, dE/dX, dE/dJ, dE/dK are accumulated
// into gx[3], gj[3], gk[3].
template <bool kGrad>
__device__ double xb_term(const DevParams &p, const double *__restrict__ pos, int x, int j, int k, int zx,
                          int zj, double *gx, double *gj, double *gk) {
  const double *ex = p.elem_data + (size_t)zx * GBXTB_ELEM_DOUBLES;
  const double *ej = p.elem_data + (size_t)zj * GBXTB_ELEM_DOUBLES;
  const double damp = p.g[12], rscale = p.g[13];
  const double r0 = rscale * (ex[5] + ej[5]);
  double u[3], v[3];
  for (int c = 0; c < 3; ++c) {
    u[c] = pos[3 * j + c] - pos[3 * x + c];
    v[c] = pos[3 * k + c] - pos[3 * x + c];
  }
  const double uu = u[0] * u[0] + u[1] * u[1] + u[2] * u[2];
  const double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
  const double uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
  const double ru = sqrt(uu), rv = sqrt(vv);
  const double s = r0 / ru, s6 = s * s * s * s * s * s, s12 = s6 * s6;
  const double lj = (s12 - damp * s6) / (1.0 + s12);
  const double cs = uv / sqrt(uu * vv);
  const double h = 0.5 - 0.5 * cs, h2 = h * h, h5 = h2 * h2 * h;
  const double fd = h5 * h;
  const double xb = ex[7];
  if (kGrad) {
    // d lj / d R and d fd / d c
    const double dlj = -(12.0 * s12 - 6.0 * damp * s6 + 6.0 * damp * s6 * s12) / (ru * (1.0 + s12) * (1.0 + s12));
    const double dfd = -3.0 * h5;
    for (int c = 0; c < 3; ++c) {
      const double dcdu = v[c] / (ru * rv) - cs * u[c] / uu;
      const double dcdv = u[c] / (ru * rv) - cs * v[c] / vv;
      const double du = xb * (dlj * u[c] / ru * fd + lj * dfd * dcdu);
      const double dv = xb * lj * dfd * dcdv;
      gj[c] += du;
      gk[c] += dv;
      gx[c] -= du + dv;
    }
  }
  return xb * lj * fd;
}

// ---------------------------------------------------------------------------
// per-atom kernel: coordination number, repulsion and halogen-bond energy
// ---------------------------------------------------------------------------
__global__ void k_atoms(DevParams p, DevPlan pl, Work w, const double *__restrict__ pos) {
  const int m = blockIdx.x;
  if (!geom_due(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  // a molecule with a non-finite coordinate is refused here: status
  // NONFINITE, phase Done, and no later kernel works on it
  int bad = 0;
  for (int k = threadIdx.x; k < 3 * md.natom; k += blockDim.x) bad |= !isfinite(pos[3 * (int64_t)md.atom0 + k]);
  if (__syncthreads_or(bad)) {
    if (threadIdx.x == 0) {
      w.status[m] |= GBXTB_MOL_NONFINITE;
      w.phase[m] = kPhaseDone;
    }
    return;
  }
  const double kcn = p.g[7], cn_cut = p.g[8], rep_cut = p.g[9], kexp = p.g[6];
  for (int ia = threadIdx.x; ia < md.natom; ia += blockDim.x) {
    const int a = md.atom0 + ia;
    const int za = pl.atom_z[a];
    const double *ea = p.elem_data + (size_t)za * GBXTB_ELEM_DOUBLES;
    const double xa = pos[3 * a], ya = pos[3 * a + 1], za_ = pos[3 * a + 2];
    double cn = 0.0, erep = 0.0;
    for (int ib = 0; ib < md.natom; ++ib) {
      if (ib == ia) continue;
      const int b = md.atom0 + ib;
      const int zb = pl.atom_z[b];
      const double *eb = p.elem_data + (size_t)zb * GBXTB_ELEM_DOUBLES;
      const double dx = xa - pos[3 * b], dy = ya - pos[3 * b + 1], dz = za_ - pos[3 * b + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r <= cn_cut) {
        const double r0 = ea[6] + eb[6];
        cn += 1.0 / (1.0 + exp(-kcn * (r0 / r - 1.0)));
      }
      if (r <= rep_cut) {
        const double alpha = sqrt(ea[3] * eb[3] + kTiny);
        erep += ea[2] * eb[2] * exp(-alpha * pow(r, kexp)) / r;
      }
    }
    // halogen bond, attributed to the donor (hal.py:359)
    double exb = 0.0;
    if (p.g[15] == 0.0 && xb_donor(za) && ea[7] != 0.0) {
      const int k = xb_nearest(md, pos, a);
      for (int ib = 0; ib < md.natom; ++ib) {
        const int b = md.atom0 + ib;
        const int zb = pl.atom_z[b];
        if (!xb_acceptor(zb)) continue;
        const double dx = pos[3 * b] - xa, dy = pos[3 * b + 1] - ya, dz = pos[3 * b + 2] - za_;
        if (sqrt(dx * dx + dy * dy + dz * dz) > p.g[14]) continue;
        exb += xb_term<false>(p, pos, a, b, k, za, zb, nullptr, nullptr, nullptr);
      }
    }
    w.cn[a] = cn;
    w.erep[a] = 0.5 * erep + exb;  // classical energy of the atom
  }
}

// ---------------------------------------------------------------------------
// shell-pair kernel: S, H0 and gamma
// ---------------------------------------------------------------------------
__global__ void k_shellpairs(DevParams p, DevPlan pl, Work w, const double *__restrict__ pos) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= pl.npair) return;
  const int m = find_mol_pair(pl.mol, pl.nmol, gid);
  if (!geom_due(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  // (pool slots reserve pairs for their capacity; the molecule may use fewer)
  if (gid - md.pair0 >= (int64_t)md.nsh * (md.nsh + 1) / 2) return;
  int i, j;
  decode_pair(gid - md.pair0, md.nsh, i, j);
  const int si = md.sh0 + i, sj = md.sh0 + j;
  const int a = pl.sh_atom[si], b = pl.sh_atom[sj];
  const ShellView vi = shell_view(p, pl.sh_rec[si]);
  const ShellView vj = shell_view(p, pl.sh_rec[sj]);
  const int za = pl.atom_z[a], zb = pl.atom_z[b];
  const double *ea = p.elem_data + (size_t)za * GBXTB_ELEM_DOUBLES;
  const double *eb = p.elem_data + (size_t)zb * GBXTB_ELEM_DOUBLES;
  const int n = md.nao;
  const int ni = 2 * vi.l + 1, nj = 2 * vj.l + 1;
  const int oi = pl.sh_ao[si], oj = pl.sh_ao[sj];
  double *S = w.S + md.mat0, *H = w.H0 + md.mat0;

  const double hi = vi.level - vi.kcn * w.cn[a];
  const double hj = vj.level - vj.kcn * w.cn[b];

  // gamma (reference guards: eta + eps, (R + eps)^2, eps on-site)
  {
    const double etai = vi.lgam * ea[0] + kEps, etaj = vj.lgam * eb[0] + kEps;
    const double avg = 2.0 / (1.0 / etai + 1.0 / etaj);
    double d2;
    if (a == b) {
      d2 = kEps;
    } else {
      const double dx = pos[3 * b] - pos[3 * a], dy = pos[3 * b + 1] - pos[3 * a + 1],
                   dz = pos[3 * b + 2] - pos[3 * a + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz) + kEps;
      d2 = r * r;
    }
    const double g = 1.0 / sqrt(d2 + 1.0 / (avg * avg));
    w.gam[md.gam0 + (int64_t)i * md.nsh + j] = g;
    w.gam[md.gam0 + (int64_t)j * md.nsh + i] = g;
  }

  double sblk[25];
  if (a == b) {
    for (int x = 0; x < ni; ++x)
      for (int y = 0; y < nj; ++y) {
        const double sv = (i == j && x == y) ? 1.0 : 0.0;
        S[(int64_t)(oi + x) * n + oj + y] = sv;
        S[(int64_t)(oj + y) * n + oi + x] = sv;
        const double hv = (i == j && x == y) ? hi : 0.0;
        H[(int64_t)(oi + x) * n + oj + y] = hv;
        H[(int64_t)(oj + y) * n + oi + x] = hv;
      }
    return;
  }
  const double rx = pos[3 * b] - pos[3 * a], ry = pos[3 * b + 1] - pos[3 * a + 1],
               rz = pos[3 * b + 2] - pos[3 * a + 2];
  const double r = sqrt(rx * rx + ry * ry + rz * rz);
  const double int_cut = p.g[10];
  if (r > 0.1 && r < int_cut) {
    overlap_block<false>(vi, vj, rx, ry, rz, sblk, nullptr);
  } else {
    for (int x = 0; x < 25; ++x) sblk[x] = 0.0;
  }
  // H0 scaling
  const double rr = sqrt(r / (ea[5] + eb[5]));
  const double pi = (1.0 + vi.shpoly * rr) * (1.0 + vj.shpoly * rr);
  double k = shell_k(p, vi, vj);
  if (vi.valence && vj.valence) {
    const double den = ea[4] - eb[4];
    k *= p.kpair[(size_t)za * (p.max_z + 1) + zb] * (1.0 + p.g[1] * den * den);
  }
  const double fac = pi * k * 0.5 * (hi + hj);
  for (int x = 0; x < ni; ++x)
    for (int y = 0; y < nj; ++y) {
      const double sv = sblk[x * nj + y];
      const double hv = fac * sv;
      S[(int64_t)(oi + x) * n + oj + y] = sv;
      S[(int64_t)(oj + y) * n + oi + x] = sv;
      H[(int64_t)(oi + x) * n + oj + y] = hv;
      H[(int64_t)(oj + y) * n + oi + x] = hv;
    }
}

// ---------------------------------------------------------------------------
// forces: shell-pair adjoint
//   dE/dA += sum_{mu in i, nu in j} X_mn dS_mn/dA
//            + 2 sum P H0 (dPi/dR)/(Pi R) (A - B)
//            + q_i q_j dgamma/dR (A - B)/R
//   with X = 2 P Ht - 2 W - P (v_mu + v_nu), Ht = H0 / S.
//   dE/dh_i accumulates sum P S K Pi (for the CN chain rule).
// ---------------------------------------------------------------------------
__global__ void k_force_pairs(DevParams p, DevPlan pl, Work w, const double *__restrict__ pos) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= pl.npair) return;
  const int m = find_mol_pair(pl.mol, pl.nmol, gid);
  if (!force_due(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  if (gid - md.pair0 >= (int64_t)md.nsh * (md.nsh + 1) / 2) return;
  int i, j;
  decode_pair(gid - md.pair0, md.nsh, i, j);
  const int si = md.sh0 + i, sj = md.sh0 + j;
  const int a = pl.sh_atom[si], b = pl.sh_atom[sj];
  const ShellView vi = shell_view(p, pl.sh_rec[si]);
  const ShellView vj = shell_view(p, pl.sh_rec[sj]);
  const int n = md.nao;
  const int ni = 2 * vi.l + 1, nj = 2 * vj.l + 1;
  const int oi = pl.sh_ao[si], oj = pl.sh_ao[sj];
  const double *P = w.P + md.mat0, *W = w.Z + md.mat0;
  if (a == b) {
    if (i == j) {
      double t = 0.0;
      for (int x = 0; x < ni; ++x) t += P[(int64_t)(oi + x) * n + oi + x];
      atomicAdd(&w.dedh[si], t);
    }
    return;
  }
  const int za = pl.atom_z[a], zb = pl.atom_z[b];
  const double *ea = p.elem_data + (size_t)za * GBXTB_ELEM_DOUBLES;
  const double *eb = p.elem_data + (size_t)zb * GBXTB_ELEM_DOUBLES;
  const double rx = pos[3 * b] - pos[3 * a], ry = pos[3 * b + 1] - pos[3 * a + 1],
               rz = pos[3 * b + 2] - pos[3 * a + 2];
  const double r = sqrt(rx * rx + ry * ry + rz * rz);
  double sblk[25], gblk[75];
  const bool has_ovl = (r > 0.1 && r < p.g[10]);
  if (has_ovl) {
    overlap_block<true>(vi, vj, rx, ry, rz, sblk, gblk);
  } else {
    for (int x = 0; x < 25; ++x) sblk[x] = 0.0;
    for (int x = 0; x < 75; ++x) gblk[x] = 0.0;
  }
  const double hi = vi.level - vi.kcn * w.cn[a];
  const double hj = vj.level - vj.kcn * w.cn[b];
  const double rr = sqrt(r / (ea[5] + eb[5]));
  const double pa = 1.0 + vi.shpoly * rr, pb = 1.0 + vj.shpoly * rr;
  const double pi = pa * pb;
  double k = shell_k(p, vi, vj);
  if (vi.valence && vj.valence) {
    const double den = ea[4] - eb[4];
    k *= p.kpair[(size_t)za * (p.max_z + 1) + zb] * (1.0 + p.g[1] * den * den);
  }
  const double fpk = pi * k;
  const double htil = fpk * 0.5 * (hi + hj);
  const double dpi = (pa * vj.shpoly + pb * vi.shpoly) * rr * 0.5 / (r * r) / pi;
  const double vvi = w.vout[si], vvj = w.vout[sj];
  double gx = 0.0, gy = 0.0, gz = 0.0, ph0 = 0.0, psf = 0.0;
  for (int x = 0; x < ni; ++x)
    for (int y = 0; y < nj; ++y) {
      const int64_t idx = (int64_t)(oi + x) * n + oj + y;
      const double pv = P[idx], wv = W[idx];
      const double X = 2.0 * pv * htil - 2.0 * wv - pv * (vvi + vvj);
      gx += X * gblk[0 * 25 + x * nj + y];
      gy += X * gblk[1 * 25 + x * nj + y];
      gz += X * gblk[2 * 25 + x * nj + y];
      ph0 += pv * htil * sblk[x * nj + y];
      psf += pv * sblk[x * nj + y] * fpk;
    }
  // distance polynomial, A - B = -r
  const double cpi = 2.0 * ph0 * dpi;
  // ES2: gamma = ((R + eps)^2 + avg^-2)^(-1/2)
  const double etai = vi.lgam * ea[0] + kEps, etaj = vj.lgam * eb[0] + kEps;
  const double avg = 2.0 / (1.0 / etai + 1.0 / etaj);
  const double re = r + kEps;
  const double g = 1.0 / sqrt(re * re + 1.0 / (avg * avg));
  const double ces = w.qsh[si] * w.qsh[sj] * (-re * g * g * g) / r;
  const double c = cpi + ces;
  gx -= c * rx;
  gy -= c * ry;
  gz -= c * rz;
  atomicAdd(&w.grad[3 * a + 0], gx);
  atomicAdd(&w.grad[3 * a + 1], gy);
  atomicAdd(&w.grad[3 * a + 2], gz);
  atomicAdd(&w.grad[3 * b + 0], -gx);
  atomicAdd(&w.grad[3 * b + 1], -gy);
  atomicAdd(&w.grad[3 * b + 2], -gz);
  atomicAdd(&w.dedh[si], psf);
  atomicAdd(&w.dedh[sj], psf);
}

// forces: per-molecule atom terms (CN chain rule and repulsion).
__global__ void k_force_atoms(DevParams p, DevPlan pl, Work w, const double *__restrict__ pos,
                              double *__restrict__ grad_out) {
  const int m = blockIdx.x;
  if (!force_due(pl, w, m)) {
    // a failed molecule of a batch: its gradient is not a number
    if (!pl.pool)
      for (int k = threadIdx.x; k < 3 * pl.mol[m].natom; k += blockDim.x)
        grad_out[3 * (int64_t)pl.mol[m].atom0 + k] = CUDART_NAN;
    return;
  }
  const MolDesc md = pl.mol[m];
  const double kcn = p.g[7], cn_cut = p.g[8], rep_cut = p.g[9], kexp = p.g[6];
  for (int ia = threadIdx.x; ia < md.natom; ia += blockDim.x) {
    const int a = md.atom0 + ia;
    double t = 0.0;
    for (int s = 0; s < pl.atom_nsh[a]; ++s) {
      const int sh = pl.atom_sh0[a] + s;
      const ShellView v = shell_view(p, pl.sh_rec[sh]);
      t -= v.kcn * w.dedh[sh];
    }
    w.dedcn[a] = t;
    // halogen bond: the donor's terms move the donor, the acceptor and the
    // donor's nearest atom
    const int za = pl.atom_z[a];
    if (p.g[15] == 0.0 && xb_donor(za) && p.elem_data[(size_t)za * GBXTB_ELEM_DOUBLES + 7] != 0.0) {
      const int k = xb_nearest(md, pos, a);
      double gx[3] = {0.0, 0.0, 0.0};
      for (int ib = 0; ib < md.natom; ++ib) {
        const int b = md.atom0 + ib;
        const int zb = pl.atom_z[b];
        if (!xb_acceptor(zb)) continue;
        const double dx = pos[3 * b] - pos[3 * a], dy = pos[3 * b + 1] - pos[3 * a + 1],
                     dz = pos[3 * b + 2] - pos[3 * a + 2];
        if (sqrt(dx * dx + dy * dy + dz * dz) > p.g[14]) continue;
        double gj[3] = {0.0, 0.0, 0.0}, gk[3] = {0.0, 0.0, 0.0};
        xb_term<true>(p, pos, a, b, k, za, zb, gx, gj, gk);
        for (int c = 0; c < 3; ++c) {
          atomicAdd(&w.grad[3 * b + c], gj[c]);
          atomicAdd(&w.grad[3 * k + c], gk[c]);
        }
      }
      for (int c = 0; c < 3; ++c) atomicAdd(&w.grad[3 * a + c], gx[c]);
    }
  }
  __syncthreads();
  for (int ia = threadIdx.x; ia < md.natom; ia += blockDim.x) {
    const int a = md.atom0 + ia;
    const int za = pl.atom_z[a];
    const double *ea = p.elem_data + (size_t)za * GBXTB_ELEM_DOUBLES;
    const double xa = pos[3 * a], ya = pos[3 * a + 1], zpa = pos[3 * a + 2];
    const double dca = w.dedcn[a];
    double gx = 0.0, gy = 0.0, gz = 0.0;
    for (int ib = 0; ib < md.natom; ++ib) {
      if (ib == ia) continue;
      const int b = md.atom0 + ib;
      const int zb = pl.atom_z[b];
      const double *eb = p.elem_data + (size_t)zb * GBXTB_ELEM_DOUBLES;
      const double dx = xa - pos[3 * b], dy = ya - pos[3 * b + 1], dz = zpa - pos[3 * b + 2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      double c = 0.0;
      if (r <= cn_cut) {
        const double r0 = ea[6] + eb[6];
        const double ex = exp(-kcn * (r0 / r - 1.0));
        const double dcn = -kcn * r0 * ex / (r * r * (1.0 + ex) * (1.0 + ex));
        c += dcn / r * (dca + w.dedcn[b]);
      }
      if (r <= rep_cut) {
        const double alpha = sqrt(ea[3] * eb[3] + kTiny);
        const double r1k = pow(r, kexp);
        const double e = ea[2] * eb[2] * exp(-alpha * r1k) / r;
        c += -(alpha * r1k * kexp + 1.0) * e / (r * r);
      }
      gx += c * dx;
      gy += c * dy;
      gz += c * dz;
    }
    grad_out[3 * a + 0] = w.grad[3 * a + 0] + gx;
    grad_out[3 * a + 1] = w.grad[3 * a + 1] + gy;
    grad_out[3 * a + 2] = w.grad[3 * a + 2] + gz;
  }
}

}  // namespace

void launch_atoms(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                  bool, cudaStream_t s) {
  k_atoms<<<pl.nmol, 128, 0, s>>>(p, pl, w, pos);
}

void launch_shellpairs(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                       cudaStream_t s) {
  const int bs = 128;
  const int64_t nb = (pl.npair + bs - 1) / bs;
  if (nb > 0) k_shellpairs<<<(unsigned)nb, bs, 0, s>>>(p, pl, w, pos);
}

void launch_forces(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                   double *grad_out, cudaStream_t s) {
  cudaMemsetAsync(w.grad, 0, sizeof(double) * 3 * pl.natom, s);
  cudaMemsetAsync(w.dedh, 0, sizeof(double) * pl.nsh, s);
  const int bs = 128;
  const int64_t nb = (pl.npair + bs - 1) / bs;
  if (nb > 0) k_force_pairs<<<(unsigned)nb, bs, 0, s>>>(p, pl, w, pos);
  k_force_atoms<<<pl.nmol, 128, 0, s>>>(p, pl, w, pos, grad_out);
}

}  // namespace gbxtb
