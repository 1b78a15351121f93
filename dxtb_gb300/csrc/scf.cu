// SCF state update of GFN1-xTB on the device: Fermi-Dirac occupations,
// Mulliken charges, ES2/ES3 potential, potential mixing with the
// reference's convergence test, and the energy assembly.
//
// Reference behaviour reproduced (dxtb, src/dxtb/_src/...):
//   occupations   wavefunction/filling.py:201-366 (Newton on E_F from the
//                 HOMO/LUMO midpoint, |sum f - n| <= sqrt(eps), exp cut at 50,
//                 empty channels zero), called at scf/base.py:861-907
//   charges       scf/base.py:764-815: q = n0 - diag(P S)
//   potential     components/interactions/base.py:134-181,
//                 coulomb/secondorder.py:415-442, coulomb/thirdorder.py:304-332
//   convergence   scf/mixer/base.py:229-256 (L2 < x_atol and max < x_atol_max
//                 on the change of the orbital potential) and
//                 scf/unrolling/default.py:100-136 (the last unmixed output
//                 potential defines the final charges)
//   energies      scf/base.py:514-623 (E_H0 = tr(P H0), ES2 1/2 q gamma q,
//                 ES3 gam3 q^3/3, electronic free energy kT sum f ln f +
//                 (1-f) ln(1-f) over both spin channels with eps clamping),
//                 calculators/types/energy.py:148-325 (total = classical + SCF)
// Mixers (gbxtb_options.mixer), all on the shell-resolved potential with
// orbital-multiplicity weights, so that every norm and inner product equals
// that of the orbital-resolved vector the reference mixes (the orbital
// potential is the shell value repeated over the shell's 2l+1 orbitals, and
// every mixer forms linear combinations of such vectors):
//   Broyden    modified Broyden (Johnson, Phys. Rev. B 38, 12807 (1988)),
//              the engine's default;
//   Anderson   the reference's Anderson/Eyert mixer step for step
//              (scf/mixer/anderson.py:200-317: soft start with damp_init,
//              then `generations` differences, diagonal rescaling
//              1 + offset^2, x_bar + damp f_bar), the mixer the reference's
//              default full-mode SCF runs (scf/unrolling/base.py:81-99);
//   simple     x + damp (F(x) - x) (scf/mixer/simple.py).
// mix_guess = 0 takes the first output potential unmixed, and damp_dynamic
// switches the mixing parameter once the potential change drops below 0.1,
// as scf/unrolling/default.py:92-121 does.  The converged fixed point does
// not depend on the mixer; which of several fixed points an SCF reaches
// can.
#include "internal.cuh"

#include <cmath>
#include <math_constants.h>

namespace gbxtb {

namespace {

constexpr double kEps = 2.220446049250313e-16;

// ---------------------------------------------------------------------------
// Fermi occupations; also decides how many eigenvectors are needed (kvec).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_fermi(DevPlan pl, Work w, double kt, int maxiter, double thresh) {
  const int m = blockIdx.x;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const double *ev = w.eig + md.ao0;
  double *occ[2] = {w.occ + md.ao0, w.occ + pl.nao + md.ao0};
  __shared__ double red[32];
  __shared__ int s_conv;
  const double thr = thresh > 0.0 ? thresh : sqrt(kEps);
  double ef[2], target[2];
  bool nonempty[2];
  for (int s = 0; s < 2; ++s) {
    const double nel = md.nel[s];
    // index of the first orbital whose cumulative count reaches nel
    int homo = 0;
    while (homo < n - 1 && (double)(homo + 1) - nel < -5.0e-15) ++homo;
    nonempty[s] = (nel != 0.0);
    const int lumo = (n - 1 <= homo) ? homo : homo + 1;
    ef[s] = nonempty[s] ? 0.5 * (ev[homo] + ev[lumo]) : 0.0;
    target[s] = (double)homo + 1.0;
  }
  int it = 0;
  for (; it < maxiter; ++it) {
    double err[2];
    for (int s = 0; s < 2; ++s) {
      double sf = 0.0, sdf = 0.0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double e = nonempty[s] ? ev[i] : 0.0;
        const double x = (e - ef[s]) / kt;
        double f, df;
        if (x < 50.0) {
          const double et = exp(x);
          f = 1.0 / (et + 1.0);
          df = et / (kt * (et + 1.0) * (et + 1.0));
        } else {
          f = 0.0;
          df = kEps;
        }
        occ[s][i] = nonempty[s] ? f : 0.0;
        sf += f;
        sdf += df;
      }
      sf = block_sum(sf, red);
      sdf = block_sum(sdf, red);
      err[s] = target[s] - sf;
      ef[s] += err[s] / sdf;
    }
    if (threadIdx.x == 0) s_conv = (fabs(err[0]) <= thr && fabs(err[1]) <= thr);
    __syncthreads();
    const int conv = s_conv;
    __syncthreads();
    if (conv) break;
  }
  if (threadIdx.x == 0) {
    if (it >= maxiter) {
      w.status[m] |= GBXTB_MOL_FERMI_FAIL;
      w.phase[m] = kPhaseDone;
    }
    w.efermi[m] = ef[0];
    w.efermi[pl.nmol + m] = ef[1];
  }
  __syncthreads();
  // number of eigenvectors with non-zero occupation in either channel
  int kmax = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (occ[0][i] > 0.0 || occ[1][i] > 0.0) kmax = max(kmax, i + 1);
  const double km = block_max((double)kmax, red);
  if (threadIdx.x == 0) w.kvec[m] = (int)km;
}

// ---------------------------------------------------------------------------
// charges -> potential -> mixing (one block per molecule)
// ---------------------------------------------------------------------------
struct MixOpts {
  double x_atol, x_atol_max, alpha, w0, kt;
  double damp, damp_init, offset, damp_dyn;
  int maxiter, memory;
  int mixer, generations, soft_start, mix_guess, damp_dynamic, restart_at;
};

constexpr int kMixThreads = 256;
// mixed precision: potential change (orbital L2 norm) below which a molecule
// leaves the FP32 passes (FP32 noise in the potential is ~1e-6; switching at
// 1e-5 instead made the 512-molecule batch take 68 passes per molecule
// instead of 52, 22 of them FP64 instead of 13), and a cap on
// the FP32 passes far beyond the iteration counts seen (molecules that never
// converge keep iterating in FP32 until maxiter; their final pass is FP64)
constexpr double kLowpSwitch = 1e-4;
constexpr int kLowpMaxPasses = 1000;
// a molecule whose FP32 passes stop making progress close to convergence
// (potential change below kLowpStallBelow and not halved for kLowpStall
// passes: the FP32 noise floor) continues in FP64; molecules that do not
// converge at all oscillate far above it and stay in FP32
constexpr double kLowpStallBelow = 1e-3;
constexpr int kLowpStall = 8;
constexpr int kMaxMem = 30;
constexpr int kHistSlots = 29;  // hist_df / hist_u slots per shell (the workspace's kHistMax)

// Solve a x = b in place for a small system (n <= kMaxMem - 1, augmented
// column n) by Gaussian elimination with partial pivoting, as LAPACK's gesv
// (which torch.linalg.solve calls) does; one warp, result in a[.][n].
__device__ void warp_solve(double (*a)[kMaxMem + 1], int n) {
  const int lane = threadIdx.x & 31;
  for (int piv = 0; piv < n; ++piv) {
    int best = piv;
    for (int r = piv + 1; r < n; ++r)
      if (fabs(a[r][piv]) > fabs(a[best][piv])) best = r;
    __syncwarp();
    if (best != piv)
      for (int c = lane; c <= n; c += 32) {
        const double t = a[piv][c];
        a[piv][c] = a[best][c];
        a[best][c] = t;
      }
    __syncwarp();
    const double inv = 1.0 / a[piv][piv];
    for (int r = piv + 1; r < n; ++r) {
      const double fac = a[r][piv] * inv;
      __syncwarp();
      for (int c = lane + piv; c <= n; c += 32) a[r][c] -= fac * a[piv][c];
      __syncwarp();
    }
  }
  // back substitution (lane 0; n is small)
  if (lane == 0)
    for (int r = n - 1; r >= 0; --r) {
      double v = a[r][n];
      for (int c = r + 1; c < n; ++c) v -= a[r][c] * a[c][n];
      a[r][n] = v / a[r][r];
    }
  __syncwarp();
}

// Anderson/Eyert step of the reference (scf/mixer/anderson.py:200-317) for
// one molecule (one block).  History: rings of generations + 1 potentials x
// and differences F = F(x) - x in hist_u / hist_df; ring slot step % R holds
// the current x (= vin, the previous mixed potential or the guess) and F.
__device__ void anderson_step(const DevPlan &pl, const Work &w, const MolDesc &md, const MixOpts &o, int step,
                              double damp, double (*a)[kMaxMem + 1]) {
  const int nsh = md.nsh;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int32_t *lsh = pl.sh_l + md.sh0;
  double *vin = w.vin + md.sh0;
  const double *vout = w.vout + md.sh0;
  const int R = o.generations + 1;
  const int cur = step % R;
  auto X = [&](int slot) { return w.hist_u + (size_t)slot * pl.nsh + md.sh0; };
  auto F = [&](int slot) { return w.hist_df + (size_t)slot * pl.nsh + md.sh0; };
  double *x0 = X(cur), *f0 = F(cur);
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    x0[i] = vin[i];
    f0[i] = vout[i] - vin[i];
  }
  __syncthreads();
  const int it = step + 1;  // the reference's iter_step after its increment
  if (it > o.generations || (it > 1 && !o.soft_start)) {
    const int n = min(it - 1, o.generations);
    // a_ij = <F0 - F_i | F0 - F_j>, b_i = <F0 - F_i | F0>, i, j = 1..n
    for (int pidx = wid; pidx < n * (n + 1); pidx += nw) {
      const int ii = pidx / (n + 1), jj = pidx % (n + 1);
      const double *fi = F((cur - 1 - ii + R) % R);
      double s = 0.0;
      if (jj < n) {
        const double *fj = F((cur - 1 - jj + R) % R);
        for (int t = lane; t < nsh; t += 32) s += (2.0 * lsh[t] + 1.0) * (f0[t] - fi[t]) * (f0[t] - fj[t]);
      } else {
        for (int t = lane; t < nsh; t += 32) s += (2.0 * lsh[t] + 1.0) * (f0[t] - fi[t]) * f0[t];
      }
      s = warp_sum(s);
      if (lane == 0) a[ii][jj] = (ii == jj && o.offset >= 0.0) ? s * (1.0 + o.offset * o.offset) : s;
    }
    __syncthreads();
    if (wid == 0) warp_solve(a, n);
    __syncthreads();
    // x_bar = x0 + sum_i theta_i (x_i - x0), f_bar = F0 + sum_i theta_i (F_i - F0)
    double *xn = X((cur + 1) % R);
    for (int t = threadIdx.x; t < nsh; t += blockDim.x) {
      double xb = 0.0, fb = 0.0;
      for (int i = 0; i < n; ++i) {
        const int sl = (cur - 1 - i + R) % R;
        const double th = a[i][n];
        xb += th * (X(sl)[t] - x0[t]);
        fb += th * -(f0[t] - F(sl)[t]);
      }
      xb += x0[t];
      fb += f0[t];
      const double xm = xb + damp * fb;
      xn[t] = xm;
      vin[t] = xm;
    }
  } else {
    double *xn = X((cur + 1) % R);
    for (int t = threadIdx.x; t < nsh; t += blockDim.x) {
      const double xm = x0[t] + f0[t] * o.damp_init;
      xn[t] = xm;
      vin[t] = xm;
    }
  }
}

// Modified Broyden step (Johnson 1988) with step alpha, unit weights and
// w0: the engine's default mixer.  `step` counts earlier calls: the first
// call only records x and F.
__device__ void broyden_step(const DevPlan &pl, const Work &w, const MolDesc &md, int m, const MixOpts &o,
                             int step, double (*a)[kMaxMem + 1]) {
  const int nsh = md.nsh;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int32_t *lsh = pl.sh_l + md.sh0;
  double *vin = w.vin + md.sh0;
  const double *vout = w.vout + md.sh0;
  double *xprev = w.xprev + md.sh0, *fprev = w.fprev + md.sh0;
  __shared__ double red[32];
  const int mem = o.memory;
  if (step == 0) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
      const double f = vout[i] - vin[i];
      xprev[i] = vin[i];
      fprev[i] = f;
      vin[i] = vin[i] + o.alpha * f;
    }
    return;
  }
  const int nst = w.nhist[m];  // number of stored (dF, u) pairs ever pushed
  // new difference pair
  double nrm = 0.0;
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    const double df = (vout[i] - vin[i]) - fprev[i];
    nrm += (2.0 * lsh[i] + 1.0) * df * df;
  }
  nrm = sqrt(block_sum(nrm, red));
  const double inrm = (nrm > 0.0) ? 1.0 / nrm : 0.0;
  const int slot = nst % mem;
  double *DF = w.hist_df + (size_t)slot * pl.nsh + md.sh0;
  double *U = w.hist_u + (size_t)slot * pl.nsh + md.sh0;
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    const double f = vout[i] - vin[i];
    const double df = (f - fprev[i]) * inrm;
    DF[i] = df;
    U[i] = o.alpha * df + (vin[i] - xprev[i]) * inrm;
  }
  __syncthreads();
  const int k = min(nst + 1, mem);
  // Gram matrix a_ij = <dF_i, dF_j> + w0^2 delta_ij and rhs c_i = <dF_i, F>
  for (int pidx = wid; pidx < k * (k + 1); pidx += nw) {
    const int ii = pidx / (k + 1), jj = pidx % (k + 1);
    const double *x = w.hist_df + (size_t)ii * pl.nsh + md.sh0;
    double s = 0.0;
    if (jj < k) {
      const double *y = w.hist_df + (size_t)jj * pl.nsh + md.sh0;
      for (int t = lane; t < nsh; t += 32) s += (2.0 * lsh[t] + 1.0) * x[t] * y[t];
    } else {
      for (int t = lane; t < nsh; t += 32) s += (2.0 * lsh[t] + 1.0) * x[t] * (vout[t] - vin[t]);
    }
    s = warp_sum(s);
    if (lane == 0) a[ii][jj] = s + ((ii == jj && jj < k) ? o.w0 * o.w0 : 0.0);
  }
  __syncthreads();
  // Gauss-Jordan elimination (matrix is symmetric positive definite)
  if (wid == 0) {
    for (int piv = 0; piv < k; ++piv) {
      const double inv = 1.0 / a[piv][piv];
      __syncwarp();
      for (int c = lane; c <= k; c += 32) a[piv][c] *= inv;
      __syncwarp();
      for (int r = 0; r < k; ++r) {
        if (r == piv) continue;
        const double fac = a[r][piv];
        __syncwarp();
        for (int c = lane; c <= k; c += 32) a[r][c] -= fac * a[piv][c];
        __syncwarp();
      }
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    const double f = vout[i] - vin[i];
    double corr = 0.0;
    for (int t = 0; t < k; ++t) corr += a[t][k] * w.hist_u[(size_t)t * pl.nsh + md.sh0 + i];
    xprev[i] = vin[i];
    fprev[i] = f;
    vin[i] = vin[i] + o.alpha * f - corr;
  }
  if (threadIdx.x == 0) w.nhist[m] = nst + 1;
}

__global__ void __launch_bounds__(kMixThreads) k_charges_mix(DevParams p, DevPlan pl, Work w, MixOpts o) {
  const int m = blockIdx.x;
  const int phase = w.phase[m];
  if (phase == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao, nsh = md.nsh, nat = md.natom;
  const double *P = w.P + md.mat0, *S = w.S + md.mat0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __shared__ double red[32];
  __shared__ double a[kMaxMem][kMaxMem + 1];
  __shared__ int s_flag;

  // 1. orbital charges q = n0 - diag(P S)
  for (int i = wid; i < n; i += nw) {
    const double *pr = P + (int64_t)i * n, *sr = S + (int64_t)i * n;
    double s = 0.0;
    for (int j = lane; j < n; j += 32) s += pr[j] * sr[j];
    s = warp_sum(s);
    if (lane == 0) w.q[md.ao0 + i] = pl.ao_n0[md.ao0 + i] - s;
  }
  __syncthreads();
  // 2. shell and atom charges
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    const int sh = md.sh0 + i;
    const int o0 = pl.sh_ao[sh], no = 2 * pl.sh_l[sh] + 1;
    double s = 0.0;
    for (int k = 0; k < no; ++k) s += w.q[md.ao0 + o0 + k];
    w.qsh[sh] = s;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nat; i += blockDim.x) {
    const int at = md.atom0 + i;
    double s = 0.0;
    for (int k = 0; k < pl.atom_nsh[at]; ++k) s += w.qsh[pl.atom_sh0[at] + k];
    w.qat[at] = s;
  }
  __syncthreads();
  // 3. output potential v = gamma q_sh + gam3 q_at^2 (shell resolved)
  const double *G = w.gam + md.gam0;
  for (int i = wid; i < nsh; i += nw) {
    double s = 0.0;
    for (int j = lane; j < nsh; j += 32) s += G[(int64_t)i * nsh + j] * w.qsh[md.sh0 + j];
    s = warp_sum(s);
    if (lane == 0) {
      const int sh = md.sh0 + i;
      const int at = pl.sh_atom[sh];
      const double g3 = p.elem_data[(size_t)pl.atom_z[at] * GBXTB_ELEM_DOUBLES + 1];
      const double qa = w.qat[at];
      w.vout[sh] = s + g3 * qa * qa;
      w.vmix[sh] = s;  // ES2 part, kept for the energy
    }
  }
  __syncthreads();

  const int32_t *lsh = pl.sh_l + md.sh0;
  double *vin = w.vin + md.sh0, *vout = w.vout + md.sh0;

  if (phase == kPhaseFinal) {
    // energies of the final state
    double eh0 = 0.0;
    const double *H = w.H0 + md.mat0;
    for (int i = wid; i < n; i += nw) {
      const double *pr = P + (int64_t)i * n, *hr = H + (int64_t)i * n;
      double s = 0.0;
      for (int j = lane; j < n; j += 32) s += pr[j] * hr[j];
      eh0 += s;
    }
    eh0 = block_sum(eh0, red);
    double es2 = 0.0;
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) es2 += 0.5 * w.qsh[md.sh0 + i] * w.vmix[md.sh0 + i];
    es2 = block_sum(es2, red);
    double es3 = 0.0, erep = 0.0;
    for (int i = threadIdx.x; i < nat; i += blockDim.x) {
      const int at = md.atom0 + i;
      const double g3 = p.elem_data[(size_t)pl.atom_z[at] * GBXTB_ELEM_DOUBLES + 1];
      const double qa = w.qat[at];
      es3 += g3 * qa * qa * qa / 3.0;
      erep += w.erep[at];
    }
    es3 = block_sum(es3, red);
    erep = block_sum(erep, red);
    double g = 0.0;
    for (int s = 0; s < 2; ++s) {
      const double *oc = w.occ + (size_t)s * pl.nao + md.ao0;
      for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double f = fmax(oc[i], kEps), f1 = fmax(1.0 - oc[i], kEps);
        g += f * log(f) + f1 * log(f1);
      }
    }
    g = block_sum(g, red) * o.kt;
    if (threadIdx.x == 0) {
      double *en = w.energy + (size_t)m * 6;
      en[1] = erep;
      en[2] = eh0;
      en[3] = es2;
      en[4] = es3;
      en[5] = g;
      en[0] = erep + eh0 + es2 + es3 + g;
      if (!isfinite(en[0])) w.status[m] |= GBXTB_MOL_NONFINITE;
      w.phase[m] = pl.pool ? kPhaseFinished : kPhaseDone;
    }
    return;
  }

  // 4. convergence test on the change of the orbital potential
  double l2 = 0.0, mx = 0.0;
  for (int i = threadIdx.x; i < nsh; i += blockDim.x) {
    const double f = vout[i] - vin[i];
    l2 += (2.0 * lsh[i] + 1.0) * f * f;
    mx = fmax(mx, fabs(f));
  }
  l2 = sqrt(block_sum(l2, red));
  mx = block_max(mx, red);
  const int iter = w.iter[m];
  if (threadIdx.x == 0) {
    w.resid[2 * m] = l2;
    w.resid[2 * m + 1] = mx;
    // an FP32 pass never decides convergence: it hands the molecule to FP64
    // once the potential change is below kLowpSwitch (or after
    // kLowpMaxPasses FP32 passes), and before a final pass
    const bool lowp = (w.prec[m] == 0);
    int flag = 0;
    if (!isfinite(l2)) flag = 3;
    else if (!lowp && iter > 0 && l2 < o.x_atol && mx < o.x_atol_max) flag = 1;
    else if (iter >= o.maxiter) flag = 2;
    bool stalled = false;
    if (lowp) {
      if (l2 < 0.5 * w.best32[m]) {
        w.best32[m] = l2;
        w.stall32[m] = 0;
      } else {
        w.stall32[m] += 1;
      }
      stalled = l2 < kLowpStallBelow && w.stall32[m] >= kLowpStall;
    }
    if (lowp && (flag == 2 || l2 < kLowpSwitch || stalled || iter + 1 >= kLowpMaxPasses)) {
      w.prec[m] = 1;
      w.npass32[m] = iter + 1;
    }
    // restart_at: still iterating after that many passes with a mixer other
    // than Anderson, the molecule starts again from the guess with the
    // reference's Anderson mixer, every pass in FP64
    if (flag == 0 && o.restart_at > 0 && !w.mixsel[m] && o.mixer != GBXTB_MIXER_ANDERSON &&
        iter + 1 >= o.restart_at) {
      if (lowp) w.npass32[m] = iter + 1;
      flag = 4;
      w.mixsel[m] = 1;
      w.prec[m] = 1;
      w.mixstep[m] = 0;
      w.nhist[m] = 0;
      w.dampsw[m] = 0;
      w.status[m] |= GBXTB_MOL_RESTARTED;
    }
    s_flag = flag;
    if (flag == 3) {
      w.status[m] |= GBXTB_MOL_NONFINITE;
      w.phase[m] = kPhaseDone;
    } else if (flag == 1 || flag == 2) {
      if (flag == 2) w.status[m] |= GBXTB_MOL_NOT_CONVERGED;
      w.phase[m] = kPhaseFinal;
    }
    w.iter[m] = (flag == 4) ? 0 : iter + 1;
  }
  __syncthreads();
  const int flag = s_flag;
  if (flag == 3) return;
  if (flag == 4) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) vin[i] = 0.0;  // the guess (SAD)
    return;
  }
  if (flag) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) vin[i] = vout[i];
    return;
  }

  // 5. mixing.  The first output potential is taken unmixed without
  // mix_guess (scf/unrolling/default.py:92-96); the mixer starts at the
  // next pass.
  if (iter == 0 && !o.mix_guess) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) vin[i] = vout[i];
    return;
  }
  const int step = w.mixstep[m];  // mixer calls before this one
  const double damp = w.dampsw[m] ? o.damp_dyn : o.damp;
  const int mixer = w.mixsel[m] ? GBXTB_MIXER_ANDERSON : o.mixer;
  if (mixer == GBXTB_MIXER_ANDERSON) {
    anderson_step(pl, w, md, o, step, damp, a);
  } else if (mixer == GBXTB_MIXER_SIMPLE) {
    for (int i = threadIdx.x; i < nsh; i += blockDim.x) vin[i] = vin[i] + (vout[i] - vin[i]) * damp;
  } else {
    broyden_step(pl, w, md, m, o, step, a);
  }
  if (threadIdx.x == 0) {
    w.mixstep[m] = step + 1;
    // the reference switches after the step, for the steps that follow
    if (o.damp_dynamic && l2 < 0.1) w.dampsw[m] = 1;
  }
}

// Count and list (in index order) the molecules that still iterate, and
// among them those whose next pass tridiagonalises on a cluster.
__device__ __forceinline__ int block_compact(bool flag, int base, int32_t *list, int m, int *wsum) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int act = flag ? 1 : 0;
  int incl = act;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wsum[wid] = incl;
  __syncthreads();
  int off = 0, tot = 0;
  for (int k = 0; k < nw; ++k) {
    if (k < wid) off += wsum[k];
    tot += wsum[k];
  }
  if (act) list[base + off + incl - 1] = m;
  __syncthreads();
  return base + tot;
}

__global__ void k_count_active(DevPlan pl, Work w) {
  __shared__ int wsum[32];
  int base = 0, basecl = 0;
  for (int m0 = 0; m0 < pl.nmol; m0 += blockDim.x) {
    const int m = m0 + threadIdx.x;
    const bool act = m < pl.nmol && (w.phase[m] == kPhaseIterate || w.phase[m] == kPhaseFinal);
    const bool clus = act && cluster_pass(w.prec[m], pl.mol[m].nao);
    base = block_compact(act, base, w.active_list, m, wsum);
    basecl = block_compact(clus, basecl, w.cluster_list, m, wsum);
  }
  if (threadIdx.x == 0) {
    w.active[0] = base;
    w.active[1] = basecl;
  }
}

// Energies and atomic charges; those of failed molecules (kFailBits) are
// not a number.
__global__ void k_outputs(DevPlan pl, Work w, double *energy_out, double *charges_out) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < pl.nmol && energy_out) energy_out[t] = (w.status[t] & kFailBits) ? CUDART_NAN : w.energy[t * 6];
  if (t < pl.natom && charges_out)
    charges_out[t] = (w.status[pl.atom_mol[t]] & kFailBits) ? CUDART_NAN : w.qat[t];
}

}  // namespace

void launch_count_active(const DevPlan &pl, const Work &w, cudaStream_t s) {
  k_count_active<<<1, 256, 0, s>>>(pl, w);
}

void launch_fermi(const DevPlan &pl, const Work &w, double kt, int maxiter, double thresh, cudaStream_t s) {
  k_fermi<<<pl.nmol, 128, 0, s>>>(pl, w, kt, maxiter, thresh);
}

void launch_charges_mix(const DevParams &p, const DevPlan &pl, const Work &w,
                        const gbxtb_options &o, cudaStream_t s) {
  MixOpts mo;
  mo.x_atol = o.x_atol;
  mo.x_atol_max = o.x_atol_max;
  mo.alpha = o.broyden_alpha;
  mo.w0 = 0.01;
  mo.kt = o.kt;
  mo.maxiter = o.maxiter;
  mo.memory = o.broyden_memory < 1 ? 1 : (o.broyden_memory > kMaxMem - 1 ? kMaxMem - 1 : o.broyden_memory);
  mo.mixer = o.mixer;
  mo.generations = o.generations < 1 ? 1 : (o.generations > kHistSlots - 1 ? kHistSlots - 1 : o.generations);
  mo.damp = o.damp;
  mo.damp_init = o.damp_init;
  mo.offset = o.diagonal_offset;
  mo.damp_dyn = o.damp_dynamic_factor;
  mo.soft_start = o.soft_start;
  mo.mix_guess = o.mix_guess;
  mo.damp_dynamic = o.damp_dynamic;
  mo.restart_at = o.restart_at;
  k_charges_mix<<<pl.nmol, kMixThreads, 0, s>>>(p, pl, w, mo);
}

void launch_energies(const DevParams &, const DevPlan &pl, const Work &w, double,
                     double *energy_out, double *charges_out, cudaStream_t s) {
  const int64_t n = pl.nmol > pl.natom ? pl.nmol : pl.natom;
  k_outputs<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(pl, w, energy_out, charges_out);
}

}  // namespace gbxtb
