// Batched FP64 linear algebra of the SCF: generalised symmetric eigenproblem
// F C = S C e for hundreds of molecules of different sizes.
//
// Reference behaviour reproduced: dxtb's diagonalize()
// (scf/unrolling/base.py:141-175) calls tad_mctc's eighb, i.e. Cholesky
// reduction S = L L^T, F' = L^-1 F L^-T, eigh(F'), C = L^-T U, eigenvalues
// ascending; the density is P = C diag(f) C^T (scf/utils.py:29-52).
//
// GB300 design notes.  The FP64 pipe of a GB300 SM retires 2 DFMA per clock,
// so an FP64 warp instruction occupies it for 16 cycles: every FP64 stage
// here is written lane-parallel (no single-thread scalar chains):
//   * Cholesky and L^-1: one block per molecule, columns of L^-1 per thread;
//   * L^-1 F L^-T, C = L^-T Y, P = C f C^T and W = C (f e) C^T: one tiled
//     FP64 GEMM kernel (64x64 tiles, 4x4 register micro-tiles) over a flat
//     grid of (molecule, tile) pairs, skipping tiles outside triangular
//     factors and computing symmetric products as lower tiles plus mirror;
//   * tridiagonalisation: Householder, by size and precision one CTA per
//     molecule (FP32 in shared memory; FP64 up to 128 AOs), an 8-SM
//     cluster with the matrix in the cluster's shared memory (up to 400
//     AOs), or a blocked (panel) cluster kernel above;
//   * eigenvalues: Sturm-sequence multisection, eight lanes per eigenvalue,
//     FP64 Newton polish in FP64 passes;
//   * eigenvectors: inverse iteration on the tridiagonal matrix, one thread
//     per eigenvector (modified Gram-Schmidt inside clusters of close
//     eigenvalues), only for orbitals with non-zero Fermi occupation;
//   * back-transformation: one warp per eigenvector column with the column
//     in registers (above 384 AOs, blocks of columns with the reflector in
//     shared memory).
// In FP64 passes the on-chip cluster tridiagonalisation and its
// back-transformation compute in double-float pairs on the FP32 pipe
// (df64.cuh) in mixed-precision runs.
//
// Mixed precision.  GB300 retires 64 FP32 FMAs for every FP64 FMA, so the
// early SCF passes of a molecule (potential change above ~1e-5) run the
// per-pass linear algebra (Fock transform, tridiagonalisation, bisection,
// inverse iteration, back-transformation, density) in FP32; the passes that
// decide convergence, and the final pass that defines the energy, charges
// and forces, run in FP64.  Every kernel of that chain is a template on the
// scalar type; a molecule's w.prec flag selects the instantiation per block
// (block-uniform branch, one launch per stage).  FP32 operands live in the
// same per-molecule blocks as the FP64 ones (n x n floats at the start of
// the n x n double block); FP32 copies of L^-1 (with L^T above the
// diagonal) and of L^-1 H0 L^-T are made once per geometry in w.lo.
#include "internal.cuh"
#include "df64.cuh"

#include <cmath>
#include <algorithm>
#include <cooperative_groups.h>
#include <mutex>
#include <type_traits>

namespace cg = cooperative_groups;

namespace gbxtb {

namespace {

// Storage of an FP64 pass's Householder reflectors (row k of A, right of the
// diagonal): FP64 numbers, or double-float pairs (df64.cuh) when the on-chip
// cluster kernel ran the pass in double-float arithmetic and the plan's
// back-transformation is the one-warp kernel (at most 384 AOs), which then
// applies them in double-float arithmetic too.  tau[n-1], which no reflector
// uses, records it: kReflSplitFlag for pairs, 0 for FP64 numbers.
constexpr double kReflSplitFlag = 1.0;
// largest plan (AOs) whose back-transformation runs one warp per eigenvector
constexpr int kBtWarpMaxN = 384;

constexpr double kEps = 2.220446049250313e-16;
constexpr double kSafeMin = 2.2250738585072014e-308;

// Per-type constants of the templated kernels.
template <typename T> struct Num;
template <> struct Num<double> {
  static constexpr double eps = 2.220446049250313e-16;
  static constexpr double safemin = 2.2250738585072014e-308;
  static constexpr double ctol = 1e-4;   // relative width of an eigenvalue cluster
};
template <> struct Num<float> {
  static constexpr double eps = 1.1920928955078125e-07;
  static constexpr double safemin = 1.1754943508222875e-38;
  // a wider FP32 window chains whole valence bands into one cluster (the
  // MGS cost grows with its square); vectors of FP32 passes may be
  // non-orthogonal to ~1e-3, which the SCF tolerates until the FP64 passes
  static constexpr double ctol = 1e-4;
};

// FP32 or FP64 view of a per-molecule n x n work block.
template <typename T>
__device__ __forceinline__ T *mat_view(double *base, int64_t mat0) {
  return reinterpret_cast<T *>(base + mat0);
}
// L^-1 buffer (strict upper triangle: L^T) and L^-1 H0 L^-T in precision T.
template <typename T> __device__ __forceinline__ const T *linv_view(const Work &w, const MolDesc &md);
template <> __device__ __forceinline__ const double *linv_view<double>(const Work &w, const MolDesc &md) {
  return w.Linv + md.mat0;
}
template <> __device__ __forceinline__ const float *linv_view<float>(const Work &w, const MolDesc &md) {
  return reinterpret_cast<const float *>(w.lo + md.mat0);
}
template <typename T> __device__ __forceinline__ const T *h0p_view(const Work &w, const MolDesc &md);
template <> __device__ __forceinline__ const double *h0p_view<double>(const Work &w, const MolDesc &md) {
  return w.H0p + md.mat0;
}
template <> __device__ __forceinline__ const float *h0p_view<float>(const Work &w, const MolDesc &md) {
  return reinterpret_cast<const float *>(w.lo + md.mat0) + (int64_t)md.nao * md.nao;
}

__device__ __forceinline__ int find_mol_tile(const MolDesc *mol, const int64_t *tile0, int nmol,
                                             int64_t t) {
  int lo = 0, hi = nmol - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile0[mid] <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---------------------------------------------------------------------------
// Cholesky factorisation S = L L^T and L^-1 (lower triangular, zero upper)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512) k_cholesky(DevPlan pl, Work w) {
  const int m = blockIdx.x;
  if (!geom_due(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  if (n > kCholBlockMinN) return;  // launch_cholesky_blocked
  double *L = w.A + md.mat0;      // work copy of S -> L
  double *X = w.Linv + md.mat0;   // L^-1
  const double *S = w.S + md.mat0;
  __shared__ double diag;
  __shared__ int fail;
  if (threadIdx.x == 0) fail = 0;
  for (int64_t e = threadIdx.x; e < (int64_t)n * n; e += blockDim.x) {
    L[e] = S[e];
    X[e] = 0.0;
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    if (threadIdx.x == 0) {
      const double akk = L[(int64_t)k * n + k];
      if (!(akk > 0.0)) {
        fail = 1;
        diag = 1.0;
      } else {
        diag = sqrt(akk);
      }
      L[(int64_t)k * n + k] = diag;
    }
    __syncthreads();
    const double dk = diag;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) L[(int64_t)i * n + k] /= dk;
    __syncthreads();
    // trailing update of the lower triangle, warp per row
    {
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
      for (int i = k + 1 + wid; i < n; i += nw) {
        const double lik = L[(int64_t)i * n + k];
        for (int j = k + 1 + lane; j <= i; j += 32) L[(int64_t)i * n + j] -= lik * L[(int64_t)j * n + k];
      }
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && fail) {
    w.status[m] |= GBXTB_MOL_CHOLESKY_FAIL;
    w.phase[m] = kPhaseDone;
  }
  // X = L^-1: thread owns column j, forward substitution down the column
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    X[(int64_t)j * n + j] = 1.0 / L[(int64_t)j * n + j];
    for (int i = j + 1; i < n; ++i) {
      double s = 0.0;
      for (int k = j; k < i; ++k) s += L[(int64_t)i * n + k] * X[(int64_t)k * n + j];
      X[(int64_t)i * n + j] = -s / L[(int64_t)i * n + i];
    }
  }
  __syncthreads();
  // keep L itself: its transpose in the (unused) strict upper triangle of
  // the L^-1 buffer, its diagonal in ldiag
  for (int64_t t = threadIdx.x; t < (int64_t)n * n; t += blockDim.x) {
    const int r = (int)(t / n), c = (int)(t % n);
    if (c > r) X[t] = L[(int64_t)c * n + r];
  }
  for (int j = threadIdx.x; j < n; j += blockDim.x) w.ldiag[md.ao0 + j] = L[(int64_t)j * n + j];
}

// ---------------------------------------------------------------------------
// batched FP64 GEMM
//   mode 0: Z = Linv * F,  F = H0 - S o (v_i + v_j)/2 formed while loading
//   mode 1: A = Z * Linv^T  (symmetric: lower tiles + mirror)
//   mode 2: A = Linv^T * Y   (Y = Z, columns < kvec)
//   mode 3: P = A diag(f) A^T  (f = occupation, K = kvec; symmetric)
//   mode 4: Z = A diag(f e) A^T (energy-weighted density; symmetric)
//   mode 5: H0p = Z * Linv^T (as mode 1, once per geometry)
//   mode 6: A = H0p - (M + M^T)/2 with M = Linv diag(v) L (lower
//           triangular): the Fock matrix in the orthogonal basis.  Because
//           S = L L^T and S o (v_i + v_j) = diag(v) S + S diag(v),
//           L^-1 (H0 - S o V / 2) L^-T = H0p - (L^-1 diag(v) L + transpose)/2,
//           N^3/3 flops per SCF pass instead of 4 N^3/3.
//   The strict upper triangle of the Linv buffer holds L^T, ldiag diag(L).
// ---------------------------------------------------------------------------
constexpr int BM = 64, BN = 64, BK = 16;

// One 64 x 64 output tile of molecule md in precision T (modes 2, 3 and 6
// run in either precision; the others only in FP64).
template <typename T>
__device__ __forceinline__ void gemm_tile(const DevPlan &pl, const Work &w, const MolDesc &md, int mode,
                                          int i0, int j0, int kvec, T (*sa)[BM + 1], T (*sb)[BN + 1]) {
  const int n = md.nao;
  const bool sym = (mode == 1 || mode == 3 || mode == 4 || mode == 5 || mode == 6);
  const int ncol = (mode == 2) ? kvec : n;
  const int K = (mode == 3 || mode == 4) ? kvec : n;
  if (j0 >= ncol) return;
  if (sym && j0 > i0) return;
  int kmin = 0, kmax = K;
  if (mode == 0) kmax = min(K, i0 + BM);
  if (mode == 1 || mode == 5) kmax = min(K, j0 + BN);
  if (mode == 2) kmin = (i0 / BK) * BK;
  if (mode == 6) {
    kmin = (j0 / BK) * BK;
    kmax = min(K, i0 + BM);
  }

  const T *Lv = linv_view<T>(w, md);
  const double *S = w.S + md.mat0, *H = w.H0 + md.mat0;
  const T *Zs = mat_view<T>(w.Z, md.mat0), *As = mat_view<T>(w.A, md.mat0);
  const double *occa = w.occ + md.ao0, *occb = w.occ + pl.nao + md.ao0;
  const double *eig = w.eig + md.ao0;
  const int32_t *aosh = pl.ao_sh + md.ao0;
  const double *vin = w.vin;

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  T acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = T(0);

  for (int k0 = kmin; k0 < kmax; k0 += BK) {
    // A tile: sa[kk][ii] = A(i0+ii, k0+kk)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;
      int ii, kk;
      if (mode == 2) { kk = e >> 6; ii = e & 63; } else { ii = e >> 4; kk = e & 15; }
      const int i = i0 + ii, k = k0 + kk;
      T v = T(0);
      if (i < n && k < K) {
        switch (mode) {
          case 0: v = (k <= i) ? Lv[(int64_t)i * n + k] : T(0); break;
          case 1: case 5: v = Zs[(int64_t)i * n + k]; break;
          case 2: v = (k >= i) ? Lv[(int64_t)k * n + i] : T(0); break;
          case 6: v = (k <= i) ? Lv[(int64_t)i * n + k] * (T)vin[aosh[k]] : T(0); break;
          default: v = As[(int64_t)i * n + k]; break;
        }
      }
      sa[kk][ii] = v;
    }
    // B tile: sb[kk][jj] = B(k0+kk, j0+jj)
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + r * 256;
      int jj, kk;
      if (mode == 0 || mode == 2) { kk = e >> 6; jj = e & 63; } else { jj = e >> 4; kk = e & 15; }
      const int j = j0 + jj, k = k0 + kk;
      T v = T(0);
      if (j < ncol && k < K) {
        switch (mode) {
          case 0: {
            const int64_t idx = (int64_t)k * n + j;
            v = (T)(H[idx] - 0.5 * S[idx] * (vin[aosh[k]] + vin[aosh[j]]));
            break;
          }
          case 1: case 5: v = (k <= j) ? Lv[(int64_t)j * n + k] : T(0); break;
          case 2: v = Zs[(int64_t)k * n + j]; break;
          case 6:  // L(k, j): stored transposed above the diagonal
            v = (k > j) ? Lv[(int64_t)j * n + k] : ((k == j) ? (T)w.ldiag[md.ao0 + j] : T(0));
            break;
          case 3: v = As[(int64_t)j * n + k] * (T)(occa[k] + occb[k]); break;
          default: v = As[(int64_t)j * n + k] * (T)((occa[k] + occb[k]) * eig[k]); break;
        }
      }
      sb[kk][jj] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = sa[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = sb[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
  T *C = nullptr;
  double *Pd = w.P + md.mat0;  // the density is always stored in FP64
  switch (mode) {
    case 0: C = mat_view<T>(w.Z, md.mat0); break;
    case 1: C = mat_view<T>(w.A, md.mat0); break;
    case 2: C = mat_view<T>(w.A, md.mat0); break;
    case 3: break;
    case 5: C = mat_view<T>(w.H0p, md.mat0); break;
    case 6: C = mat_view<T>(w.A, md.mat0); break;
    default: C = mat_view<T>(w.Z, md.mat0); break;
  }
  const T *H0p = h0p_view<T>(w, md);
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty * 4 + r;
    if (i >= n) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = j0 + tx * 4 + c;
      if (j >= ncol) continue;
      if (sym) {
        if (j > i) continue;
        T val = acc[r][c];
        if (mode == 6) val = H0p[(int64_t)i * n + j] - ((i == j) ? val : T(0.5) * val);
        if (mode == 3) {
          Pd[(int64_t)i * n + j] = (double)val;
          Pd[(int64_t)j * n + i] = (double)val;
        } else {
          C[(int64_t)i * n + j] = val;
          C[(int64_t)j * n + i] = val;
        }
      } else {
        C[(int64_t)i * n + j] = acc[r][c];
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_gemm(DevPlan pl, Work w, const int64_t *tile0, int mode, int all) {
  const int64_t t = blockIdx.x;
  const int m = find_mol_tile(pl.mol, tile0, pl.nmol, t);
  if (mode == 0 || mode == 5) {
    if (!geom_due(pl, w, m)) return;
  } else if (mode == 4) {
    if (!force_due(pl, w, m)) return;
  }
  if (!all && w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const int nt = (n + BN - 1) / BN;
  const int local = (int)(t - tile0[m]);
  if (local >= nt * nt) return;  // pool slots reserve tiles for their capacity
  const int ti = local / nt, tj = local % nt;
  const int kvec = min(max(w.kvec[m], 0), n);
  __shared__ double sa[BK][BM + 1];
  __shared__ double sb[BK][BN + 1];
  const bool lowp = (mode == 2 || mode == 3 || mode == 6) && w.prec[m] == 0;
  if (lowp)
    gemm_tile<float>(pl, w, md, mode, ti * BM, tj * BN, kvec, reinterpret_cast<float (*)[BM + 1]>(&sa[0][0]),
                     reinterpret_cast<float (*)[BN + 1]>(&sb[0][0]));
  else
    gemm_tile<double>(pl, w, md, mode, ti * BM, tj * BN, kvec, sa, sb);
}

// FP32 copies of the L^-1 buffer (L^-1 below, L^T above the diagonal) and of
// L^-1 H0 L^-T, once per geometry (one block per molecule).
__global__ void __launch_bounds__(256) k_lowp_copies(DevPlan pl, Work w) {
  if (!geom_due(pl, w, blockIdx.x)) return;
  const MolDesc md = pl.mol[blockIdx.x];
  const int64_t nn = (int64_t)md.nao * md.nao;
  float *dst = reinterpret_cast<float *>(w.lo + md.mat0);
  const double *lv = w.Linv + md.mat0, *hp = w.H0p + md.mat0;
  for (int64_t e = threadIdx.x; e < nn; e += blockDim.x) {
    dst[e] = (float)lv[e];
    dst[nn + e] = (float)hp[e];
  }
}

// ---------------------------------------------------------------------------
// Householder tridiagonalisation of A (full symmetric storage, in place).
// Reflector k (v with v_0 = 1) is stored in column k below the diagonal,
// tau_k in w.tau, the tridiagonal in w.d / w.e.
// ---------------------------------------------------------------------------
constexpr int kTrdThreads = 512;

template <typename T>
__device__ __forceinline__ void tridiag_body(const MolDesc &md, const Work &w, T *sm, T *red) {
  const int n = md.nao;
  T *A = mat_view<T>(w.A, md.mat0);
  double *d = w.d + md.ao0, *e = w.e + md.ao0, *tau = w.tau + md.ao0;
  T *vs = sm;          // [n]
  T *ps = sm + n;      // [n]
  __shared__ T sc[4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k + 2 < n; ++k) {
    const int m1 = n - k - 1;  // length of x
    // column x = A[k+1.., k]
    T part = T(0);
    for (int t = 1 + threadIdx.x; t < m1; t += blockDim.x) {
      const T x = A[(int64_t)(k + 1 + t) * n + k];
      part += x * x;
    }
    const T xn2 = block_sum(part, red);
    if (threadIdx.x == 0) {
      const T alpha = A[(int64_t)(k + 1) * n + k];
      d[k] = A[(int64_t)k * n + k];
      if (xn2 == T(0)) {
        sc[0] = T(0);      // tau
        sc[1] = T(0);      // scale
        e[k] = alpha;
      } else {
        const T beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        sc[0] = (beta - alpha) / beta;
        sc[1] = T(1) / (alpha - beta);
        e[k] = beta;
      }
      tau[k] = sc[0];
    }
    __syncthreads();
    const T tk = sc[0], scale = sc[1];
    if (tk == T(0)) {
      // no reflection needed (tau = 0 makes the stored vector irrelevant)
      __syncthreads();
      continue;
    }
    for (int t = threadIdx.x; t < m1; t += blockDim.x) {
      T v = (t == 0) ? T(1) : A[(int64_t)(k + 1 + t) * n + k] * scale;
      vs[t] = v;
    }
    __syncthreads();
    // the reflector is kept in row k (contiguous), which the trailing
    // update never touches again
    for (int t = threadIdx.x; t < m1; t += blockDim.x) A[(int64_t)k * n + k + 1 + t] = vs[t];
    // p = tau * A22 v   (warp per row)
    for (int i = wid; i < m1; i += nw) {
      const T *row = A + (int64_t)(k + 1 + i) * n + (k + 1);
      T s = T(0);
      for (int j = lane; j < m1; j += 32) s += row[j] * vs[j];
      s = warp_sum(s);
      if (lane == 0) ps[i] = tk * s;
    }
    __syncthreads();
    T pv = T(0);
    for (int t = threadIdx.x; t < m1; t += blockDim.x) pv += ps[t] * vs[t];
    const T K = block_sum(pv, red);
    const T half = T(0.5) * tk * K;
    for (int t = threadIdx.x; t < m1; t += blockDim.x) ps[t] -= half * vs[t];  // w
    __syncthreads();
    // A22 -= v w^T + w v^T
    for (int i = wid; i < m1; i += nw) {
      T *row = A + (int64_t)(k + 1 + i) * n + (k + 1);
      const T vi = vs[i], wi = ps[i];
      for (int j = lane; j < m1; j += 32) row[j] -= vi * ps[j] + wi * vs[j];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (n >= 2) {
      d[n - 2] = A[(int64_t)(n - 2) * n + (n - 2)];
      d[n - 1] = A[(int64_t)(n - 1) * n + (n - 1)];
      e[n - 2] = A[(int64_t)(n - 1) * n + (n - 2)];
    } else {
      d[0] = A[0];
    }
  }
}

__global__ void __launch_bounds__(kTrdThreads) k_tridiag(DevPlan pl, Work w) {
  const int m = blockIdx.x;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  // FP32 passes run in k_tridiag_smem or (too large for shared memory) on a
  // cluster, like the FP64 passes of more than kClusterMinN AOs
  if (w.prec[m] == 0 || cluster_pass(w.prec[m], md.nao)) return;
  extern __shared__ double sm[];
  __shared__ double red[32];
  if (threadIdx.x == 0) w.tau[md.ao0 + md.nao - 1] = 0.0;  // reflectors as FP64 numbers
  tridiag_body<double>(md, w, sm, red);
}

// ---------------------------------------------------------------------------
// FP32 Householder tridiagonalisation with the matrix in shared memory
// (packed lower triangle, row i at i(i+1)/2), one CTA per molecule.  Every
// operand of a step is an on-chip access and a step needs five CTA
// barriers, instead of the L2 round trips and cluster barriers of the
// global-memory kernels; this is the kernel of the FP32 passes (most passes
// of every molecule, all passes of molecules that do not converge).
// A molecule with more than kSmemLocalMaxN AOs first runs its leading
// n - kSmemLocalMaxN steps on the FP32 view of A in global memory (the
// steps of tridiag_body), then loads the trailing matrix on chip.
// Output conventions as tridiag_body: reflector k in row k of the FP32 view
// of A (for the back-transformation), d, e, tau in FP64 arrays.
// Launched per size class (kSmemBins) over the plan's per-class molecule
// lists; molecules of an FP64 pass or already done return at once.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t poff(int i) { return (int64_t)i * (i + 1) / 2; }

// Sum over the CTA with one barrier: warp partials go to red[0..nw-1] and
// every thread adds them up.  Consecutive calls must alternate between two
// `red` buffers (the next write to a buffer comes after another barrier).
__device__ __forceinline__ float cta_sum(float v, float *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  float t = 0.f;
  for (int i = 0; i < nw; ++i) t += red[i];
  return t;
}

constexpr int kSmemCols = (kSmemLocalMaxN + 31) / 32;  // column slots per lane

// NW warps per CTA (the size class picks it: more warps for larger molecules)
template <int NW>
__global__ void __launch_bounds__(NW * 32) k_tridiag_smem(DevPlan pl, Work w, const int32_t *mol_list, int tail) {
  constexpr int kSmemWarps = NW;
  const int m = mol_list[blockIdx.x];
  if (w.phase[m] == kPhaseDone || w.prec[m] != 0) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  if (n > kSmemTridiagMaxN) return;          // on a cluster (k_tridiag_cluster_blocked)
  if (tail && n > kTailClusterMinN) return;  // on a cluster (k_tridiag_cluster)
  const int k0 = n > kSmemLocalMaxN ? n - kSmemLocalMaxN : 0;  // steps in global memory
  const int nl = n - k0;                                        // trailing size on chip
  extern __shared__ float smf[];
  float *Ap = smf;                          // packed lower triangle of A[k0.., k0..]
  float *vb = smf + poff(nl);               // [2][n] reflectors (current, previous)
  float *wb = vb + 2 * n;                   // [2][n] rank-2 partners
  float *prow = wb + 2 * n;                 // [n] row part of A v
  float *colpart = prow + n;                // [kSmemWarps][nl] column parts of A v
  __shared__ float red[4][32];
  float *Ag = mat_view<float>(w.A, md.mat0);
  double *d = w.d + md.ao0, *e = w.e + md.ao0, *tau = w.tau + md.ao0;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = NW;
  int rb = 0;  // alternating reduction buffer

  // leading steps on the full matrix in global memory
  {
    float *vs = vb, *ps = wb;
    for (int k = 0; k < k0; ++k) {
      const int m1 = n - k - 1;
      float part = 0.f;
      for (int t = 1 + threadIdx.x; t < m1; t += blockDim.x) {
        const float x = Ag[(int64_t)(k + 1 + t) * n + k];
        part += x * x;
      }
      const float xn2 = cta_sum(part, red[rb]);
      rb ^= 1;
      const float alpha = Ag[(int64_t)(k + 1) * n + k];
      float tk = 0.f, scale = 0.f, beta = alpha;
      if (xn2 != 0.f) {
        beta = -copysignf(sqrtf(alpha * alpha + xn2), alpha);
        tk = (beta - alpha) / beta;
        scale = 1.f / (alpha - beta);
      }
      if (threadIdx.x == 0) {
        d[k] = Ag[(int64_t)k * n + k];
        e[k] = beta;
        tau[k] = tk;
      }
      if (tk == 0.f) continue;  // uniform; nothing was written
      for (int t = threadIdx.x; t < m1; t += blockDim.x)
        vs[t] = (t == 0) ? 1.f : Ag[(int64_t)(k + 1 + t) * n + k] * scale;
      __syncthreads();
      for (int t = threadIdx.x; t < m1; t += blockDim.x) Ag[(int64_t)k * n + k + 1 + t] = vs[t];
      float pv = 0.f;
      for (int i = wid; i < m1; i += nw) {
        const float *row = Ag + (int64_t)(k + 1 + i) * n + (k + 1);
        float sacc = 0.f;
        for (int j = lane; j < m1; j += 32) sacc += row[j] * vs[j];
        sacc = warp_sum(sacc) * tk;
        if (lane == 0) {
          ps[i] = sacc;
          pv += sacc * vs[i];
        }
      }
      const float K = cta_sum(pv, red[rb]);
      rb ^= 1;
      const float half = 0.5f * tk * K;
      for (int i = wid; i < m1; i += nw) {
        float *row = Ag + (int64_t)(k + 1 + i) * n + (k + 1);
        const float vi = vs[i], wi = ps[i] - half * vs[i];
        for (int j = lane; j < m1; j += 32) row[j] -= vi * (ps[j] - half * vs[j]) + wi * vs[j];
      }
      __syncthreads();
    }
  }

  // The trailing matrix on chip (packed lower triangle, local indices).
  // One pass over it per step: the pending rank-2 update of the previous
  // step is applied to each element as it is read, and the updated element
  // enters this step's A v at once (row part in the warp, column part in
  // per-lane registers).  Column kl+1, which the next reflector needs, gets
  // this step's update right after the step.
  for (int i = wid; i < nl; i += nw)
    for (int j = lane; j <= i; j += 32) Ap[poff(i) + j] = Ag[(int64_t)(k0 + i) * n + k0 + j];
  for (int t = threadIdx.x; t < 2 * n; t += blockDim.x) {
    vb[t] = 0.f;
    wb[t] = 0.f;
  }
  __syncthreads();
  // squared norm of column 0 below the sub-diagonal (the first reflector)
  float part = 0.f;
  for (int t = 2 + threadIdx.x; t < nl; t += blockDim.x) {
    const float x = Ap[poff(t)];
    part += x * x;
  }
  float xn2 = cta_sum(part, red[rb]);
  rb ^= 1;
  int cur = 0;
  for (int kl = 0; kl + 2 < nl; ++kl) {
    const int k = k0 + kl;  // global step
    const int m1 = nl - kl - 1;
    float *vc = vb + cur * n, *wc = wb + cur * n;              // this step
    const float *vp = vb + (cur ^ 1) * n, *wp = wb + (cur ^ 1) * n;  // pending
    // reflector of column kl (already fully updated); every thread derives
    // the same parameters
    const float alpha = Ap[poff(kl + 1) + kl];
    float tk = 0.f, scale = 0.f, beta = alpha;
    if (xn2 != 0.f) {
      beta = -copysignf(sqrtf(alpha * alpha + xn2), alpha);
      tk = (beta - alpha) / beta;
      scale = 1.f / (alpha - beta);
    }
    if (threadIdx.x == 0) {
      d[k] = Ap[poff(kl) + kl];
      e[k] = beta;
      tau[k] = tk;
    }
    for (int t = threadIdx.x; t < m1; t += blockDim.x) {
      const float v = (tk == 0.f) ? 0.f : ((t == 0) ? 1.f : Ap[poff(kl + 1 + t) + kl] * scale);
      vc[kl + 1 + t] = v;
      Ag[(int64_t)k * n + k + 1 + t] = v;  // reflector for the back-transformation
    }
    __syncthreads();
    // fused pass over rows i > kl, columns kl < j <= i; a warp works on two
    // rows at once so that their reductions overlap
    float acc[kSmemCols];
#pragma unroll
    for (int c = 0; c < kSmemCols; ++c) acc[c] = 0.f;
    const int j0 = kl + 1;
    for (int i1 = j0 + wid; i1 < nl; i1 += 2 * nw) {
      const int i2 = i1 + nw;
      const bool has2 = i2 < nl;
      float *row1 = Ap + poff(i1);
      float *row2 = Ap + poff(has2 ? i2 : i1);
      const float vp1 = vp[i1], wp1 = wp[i1], vc1 = vc[i1];
      const float vp2 = has2 ? vp[i2] : 0.f, wp2 = has2 ? wp[i2] : 0.f, vc2 = has2 ? vc[i2] : 0.f;
      const int last = has2 ? i2 : i1;  // the longer row
      float s1 = 0.f, s2 = 0.f;
#pragma unroll
      for (int c = 0; c < kSmemCols; ++c) {
        const int j = j0 + lane + 32 * c;
        if (32 * c > last - j0) break;  // uniform over the warp
        if (j <= last) {
          const float wpj = wp[j], vpj = vp[j], vcj = vc[j];
          float add = 0.f;
          if (j <= i1) {
            const float a = row1[j] - (vp1 * wpj + wp1 * vpj);
            row1[j] = a;
            s1 += a * vcj;
            if (j < i1) add += a * vc1;
          }
          if (has2) {
            const float a = row2[j] - (vp2 * wpj + wp2 * vpj);
            row2[j] = a;
            s2 += a * vcj;
            if (j < i2) add += a * vc2;
          }
          acc[c] += add;
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
      }
      if (lane == 0) {
        prow[i1] = s1;
        if (has2) prow[i2] = s2;
      }
    }
#pragma unroll
    for (int c = 0; c < kSmemCols; ++c) {
      const int j = j0 + lane + 32 * c;
      if (j < nl) colpart[wid * nl + j] = acc[c];
    }
    __syncthreads();
    // p = tau A v, K = p.v, w = p - tau K v / 2
    float pv = 0.f;
    for (int i = j0 + threadIdx.x; i < nl; i += blockDim.x) {
      float sum = prow[i];
#pragma unroll
      for (int q = 0; q < kSmemWarps; ++q) sum += colpart[q * nl + i];
      const float pi = tk * sum;
      prow[i] = pi;
      pv += pi * vc[i];
    }
    const float K = cta_sum(pv, red[rb]);
    rb ^= 1;
    const float half = 0.5f * tk * K;
    for (int i = j0 + threadIdx.x; i < nl; i += blockDim.x) wc[i] = prow[i] - half * vc[i];
    __syncthreads();
    // this step's update of column kl+1 (rows i >= kl+1), and the squared
    // norm of its entries below the sub-diagonal (the next reflector)
    part = 0.f;
    {
      const float vj = vc[j0], wj = wc[j0];
      for (int i = j0 + threadIdx.x; i < nl; i += blockDim.x) {
        const float a = Ap[poff(i) + j0] - (vc[i] * wj + wc[i] * vj);
        Ap[poff(i) + j0] = a;
        if (i >= j0 + 2) part += a * a;
      }
    }
    xn2 = cta_sum(part, red[rb]);
    rb ^= 1;
    cur ^= 1;
  }
  // the last diagonal element still carries the final step's update
  if (threadIdx.x == 0) {
    if (nl >= 3) {
      const float *vp = vb + (cur ^ 1) * n, *wp = wb + (cur ^ 1) * n;
      Ap[poff(nl - 1) + nl - 1] -= 2.f * vp[nl - 1] * wp[nl - 1];
    }
    if (nl >= 2) {
      d[n - 2] = Ap[poff(nl - 2) + nl - 2];
      d[n - 1] = Ap[poff(nl - 1) + nl - 1];
      e[n - 2] = Ap[poff(nl - 1) + nl - 2];
    } else {
      d[n - 1] = Ap[0];
    }
  }
}

// ---------------------------------------------------------------------------
// Householder tridiagonalisation on a thread-block cluster (8 SMs per
// molecule), column by column, for molecules up to kClusterBlockedMinN AOs:
// FP64 passes above kClusterMinN AOs, and every pass in the tail of a batch,
// when one SM per molecule would leave the GPU idle.  The matrix lives in
// the cluster's shared memory for the whole reduction (rows owned
// cyclically, row i by CTA i mod 8; tridiag_cluster_onchip below).  Same
// arithmetic and storage conventions as k_tridiag.
// ---------------------------------------------------------------------------
constexpr int kClusterSize = 8;
constexpr int kTrdClThreads = 256;

template <typename T>
__device__ __forceinline__ T ld_cg(const T *p) {
  return __ldcg(p);
}

// The same reduction with the matrix held on chip: the 8 CTAs of the
// cluster keep their own rows (row i on CTA i mod 8, full length n) in
// shared memory for the whole tridiagonalisation, so that the matrix-vector
// product and the rank-2 update of a step touch only local shared memory.
//
// One exchange per step (one cluster barrier).  Step k starts with v_k in
// every CTA and the CTA's rows updated through step k-1:
//   (1) p_k = tau A22 v_k for its own rows: a warp takes four of its rows at
//       a time and sums their four dot products over the lanes together
//       (six adds by a transposed butterfly instead of twenty); p_k and the
//       per-warp partials of p.v are published;
//   (2) a copy of column k+1 of its rows, as it is before this step's
//       update, is published;  -- cluster barrier --
//   (3) every CTA gathers p and forms w_k = p - tau/2 (p.v) v for all rows;
//   (4) every CTA applies this step's update to the gathered copy of column
//       k+1 (the owners' expression, so bitwise their values), and
//   (5) the owners apply A22 -= v w^T + w v^T to their rows (two FMAs per
//       element), while
//   (6) every CTA forms reflector k+1 from that column: its squared norm by
//       a fixed-order block reduction, so tau and the scale are bitwise the
//       same everywhere and every branch on them is uniform over the
//       cluster.  A column with nothing to reduce gives tau = 0 and
//       v = e_1, an exact identity update, so every step passes the same
//       barriers.
// Publications are double-buffered by the parity of k: a CTA rewrites a
// buffer only after the barrier that follows every other CTA's last read.
// The FP64 pipe of this GPU retires two FMAs per clock per SM (1/64 of the
// FP32 rate), and an FP64 warp instruction holds it for 16 clocks whatever
// its active lanes: in FP64 and double-float, warp 0 alone forms the
// reflector's scalars and sums the cluster partials, which the other warps
// read from shared memory after a CTA barrier; in FP32 every warp forms
// them itself.
// Output conventions as tridiag_body (reflector k in row k of A in global
// memory, d, e, tau).
constexpr int kClWarps = kTrdClThreads / 32;  // warps per CTA of the cluster kernels

// Element arithmetic of tridiag_cluster_onchip.  T is the type the rows
// are held and updated in (FP32 passes: float; FP64 passes: double, or
// df64, double-float pairs on the FP32 pipe, in mixed-precision runs), G
// the type of the matrix in global memory.  The float and double forms are
// the plain expressions; the reflector's scalars of a df64 reduction are
// formed in double.
template <typename T>
struct ClOps;

template <typename R>
struct ClOpsNative {
  using G = R;
  using Acc = R;
  static __device__ __forceinline__ R zero() { return R(0); }
  static __device__ __forceinline__ R one() { return R(1); }
  static __device__ __forceinline__ R load(G x) { return x; }
  static __device__ __forceinline__ G store(R x) { return x; }
  static __device__ __forceinline__ double to_d(R x) { return (double)x; }
  static __device__ __forceinline__ R from_d(double x) { return (R)x; }
  static __device__ __forceinline__ bool is_zero(R x) { return x == R(0); }
  static __device__ __forceinline__ R add(R a, R b) { return a + b; }
  static __device__ __forceinline__ R mul(R a, R b) { return a * b; }
  static __device__ __forceinline__ R half_prod(R tk, R K) { return R(0.5) * tk * K; }
  static __device__ __forceinline__ R axpy_neg(R p, R h, R v) { return p - h * v; }  // p - h v
  static __device__ __forceinline__ R rank2(R a, R vi, R wj, R wi, R vj) { return fma(-vi, wj, fma(-wi, vj, a)); }
  static __device__ __forceinline__ Acc acc0() { return R(0); }
  static __device__ __forceinline__ void dot(Acc &acc, R a, R b) { acc += a * b; }
  static __device__ __forceinline__ R fin(Acc acc) { return acc; }
  static __device__ __forceinline__ R shfl_xor(R a, int off) { return __shfl_xor_sync(0xffffffffu, a, off); }
  static __device__ __forceinline__ R shfl(R a, int src) { return __shfl_sync(0xffffffffu, a, src); }
  // Householder scalars from the squared norm below alpha and alpha
  static __device__ __forceinline__ void reflector(R xn2, R alpha, R &tk, R &scale, double &beta_out) {
    R beta = alpha;
    tk = R(0);
    scale = R(0);
    if (xn2 != R(0)) {
      beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
      tk = (beta - alpha) / beta;
      scale = R(1) / (alpha - beta);
    }
    beta_out = (double)beta;
  }
};
template <>
struct ClOps<float> : ClOpsNative<float> {};
template <>
struct ClOps<double> : ClOpsNative<double> {};

template <>
struct ClOps<df64> {
  using G = double;
  using Acc = DfAcc;
  static __device__ __forceinline__ df64 zero() { return df64(0.f); }
  static __device__ __forceinline__ df64 one() { return df64(1.f); }
  static __device__ __forceinline__ df64 load(G x) { return df_from_double(x); }
  static __device__ __forceinline__ G store(df64 x) { return df_to_double(x); }
  static __device__ __forceinline__ double to_d(df64 x) { return df_to_double(x); }
  static __device__ __forceinline__ df64 from_d(double x) { return df_from_double(x); }
  static __device__ __forceinline__ bool is_zero(df64 x) { return x.hi == 0.f; }
  static __device__ __forceinline__ df64 add(df64 a, df64 b) { return df_add(a, b); }
  static __device__ __forceinline__ df64 mul(df64 a, df64 b) { return df_mul(a, b); }
  static __device__ __forceinline__ df64 half_prod(df64 tk, df64 K) {
    return df_mul(df64(0.5f * tk.hi, 0.5f * tk.lo), K);  // exact halving
  }
  static __device__ __forceinline__ df64 axpy_neg(df64 p, df64 h, df64 v) { return df_add(p, df_neg(df_mul(h, v))); }
  static __device__ __forceinline__ df64 rank2(df64 a, df64 vi, df64 wj, df64 wi, df64 vj) {
    return df_rank2(a, vi, wj, wi, vj);
  }
  static __device__ __forceinline__ Acc acc0() { return DfAcc{}; }
  static __device__ __forceinline__ void dot(Acc &acc, df64 a, df64 b) { df_dot_add(acc, a, b); }
  static __device__ __forceinline__ df64 fin(Acc acc) { return df_dot_final(acc); }
  static __device__ __forceinline__ df64 shfl_xor(df64 a, int off) { return df_shfl_xor(a, off); }
  static __device__ __forceinline__ df64 shfl(df64 a, int src) { return df_shfl(a, src); }
  static __device__ __forceinline__ void reflector(df64 xn2, df64 alpha, df64 &tk, df64 &scale, double &beta_out) {
    double t, sc;
    ClOpsNative<double>::reflector(df_to_double(xn2), df_to_double(alpha), t, sc, beta_out);
    tk = df_from_double(t);
    scale = df_from_double(sc);
  }
};

template <typename T>
__device__ __forceinline__ T cl_warp_sum(T v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = ClOps<T>::add(v, ClOps<T>::shfl_xor(v, off));
  return v;
}

// Sum over the cluster of the per-warp partials part[buf][0..kClWarps)
// published by every CTA; every lane of the calling warp gets the sum.
template <typename T>
__device__ __forceinline__ T cluster_partial_sum(cg::cluster_group &cluster, T (*part)[kClWarps], int buf) {
  static_assert(kClusterSize * kClWarps == 64, "two partials per lane");
  const int lane = threadIdx.x & 31;
  const T v0 = cluster.map_shared_rank(&part[buf][0], lane / kClWarps)[lane % kClWarps];
  const T v1 = cluster.map_shared_rank(&part[buf][0], (lane + 32) / kClWarps)[(lane + 32) % kClWarps];
  return cl_warp_sum(ClOps<T>::add(ClOps<T>::add(ClOps<T>::zero(), v0), v1));
}

// Sums of four per-lane values a0..a3 over the warp by a transposed
// butterfly: after it, lane 8 q holds the sum of a_q (q = 0..3).
template <typename T>
__device__ __forceinline__ T warp_sum4(T a0, T a1, T a2, T a3) {
  using O = ClOps<T>;
  const int lane = threadIdx.x & 31;
  const bool h4 = lane & 16, h3 = lane & 8;
  // offset 16: the lower half keeps rows 0, 1, the upper half rows 2, 3
  const T s0 = h4 ? a0 : a2, s1 = h4 ? a1 : a3;
  const T k0 = h4 ? a2 : a0, k1 = h4 ? a3 : a1;
  const T b0 = O::add(k0, O::shfl_xor(s0, 16));
  const T b1 = O::add(k1, O::shfl_xor(s1, 16));
  // offset 8: bit 3 picks the first or the second row of the pair
  T c = O::add(h3 ? b1 : b0, O::shfl_xor(h3 ? b0 : b1, 8));
#pragma unroll
  for (int off = 4; off > 0; off >>= 1) c = O::add(c, O::shfl_xor(c, off));
  return c;
}

template <typename T>
__device__ __forceinline__ void tridiag_cluster_onchip(cg::cluster_group &cluster, const MolDesc &md,
                                                       const Work &w, T *sm, T (*nrmw)[kClWarps],
                                                       T (*kpw)[kClWarps], T *scal, bool refl_split) {
  using O = ClOps<T>;
  using G = typename O::G;
  using Acc = typename O::Acc;
  // double-float reflectors stay pairs in A (kReflSplitFlag)
  const bool split_store = std::is_same<T, df64>::value && refl_split;
  // FP32: every warp forms the scalars it needs itself (no CTA barrier);
  // FP64 and double-float: warp 0 alone (the FP64 pipe is scarce)
  constexpr bool kOneWarp = !std::is_same<T, float>::value;
  const int rank = (int)cluster.block_rank();
  const int n = md.nao;
  const int nloc = (n - rank + kClusterSize - 1) / kClusterSize;  // rows rank, rank + 8, ...
  G *Ag = mat_view<G>(w.A, md.mat0);
  double *d = w.d + md.ao0, *e = w.e + md.ao0, *tau = w.tau + md.ao0;
  const int nloc_max = (n + kClusterSize - 1) / kClusterSize;
  T *rows = sm;                                   // [nloc_max][n]
  T *vsb = rows + (size_t)nloc_max * n;           // [2][n] reflector v_k by row k+1+t, by parity of k
  T *wv = vsb + 2 * (size_t)n;                    // [n] w_k by row k+1+t
  T *psb = wv + n;                                // [2][nloc_max] p_k of own rows (read by all)
  T *colb = psb + 2 * (size_t)nloc_max;           // [2][nloc_max] column k+1 of own rows before step k's update
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  auto own = [&](int i, int j) -> T & { return rows[(size_t)(i / kClusterSize) * n + j]; };
  // first own local row index with row >= r
  auto first_local = [&](int r) {
    const int f = (r - rank + kClusterSize - 1) / kClusterSize;
    return f > 0 ? f : 0;
  };
  // Reflector k from X[0..m1) = column k of rows k+1..n-1 (identical in every
  // CTA): squared norm of X[1..) by a fixed-order block reduction, scalars,
  // then X becomes v_k in place (v_k[0] = 1).  Without reflection (zero
  // norm) tau_k = 0 and v_k = e_1: the step's update is then exactly the
  // identity, so the step keeps the same barriers.
  auto make_reflector = [&](int k, T *X) -> T {
    const int m1 = n - k - 1;
    const T alpha = X[0];  // read by every thread before the barrier below, X[0] is rewritten after it
    Acc part = O::acc0();
    for (int t = 1 + threadIdx.x; t < m1; t += blockDim.x) O::dot(part, X[t], X[t]);
    const T ws = cl_warp_sum(O::fin(part));
    if (lane == 0) nrmw[0][wid] = ws;
    __syncthreads();
    T tk = O::zero(), scale = O::zero();
    if (!kOneWarp || wid == 0) {
      T xn2 = O::zero();
      for (int q = 0; q < kClWarps; ++q) xn2 = O::add(xn2, nrmw[0][q]);
      double beta;
      O::reflector(xn2, alpha, tk, scale, beta);
      if (threadIdx.x == 0) {
        scal[0] = tk;
        scal[1] = scale;
        if (rank == 0) {
          e[k] = beta;
          tau[k] = O::to_d(tk);
        }
      }
    }
    if (kOneWarp) {
      __syncthreads();
      tk = scal[0];
      scale = scal[1];
    }
    for (int t = threadIdx.x; t < m1; t += blockDim.x) X[t] = (t == 0) ? O::one() : O::mul(X[t], scale);
    return tk;
  };
  // load own rows
  for (int li = wid; li < nloc; li += nw) {
    const G *src = Ag + (int64_t)(rank + li * kClusterSize) * n;
    T *dst = rows + (size_t)li * n;
    for (int j = lane; j < n; j += 32) dst[j] = O::load(src[j]);
  }
  if (rank == 0 && threadIdx.x == 0) tau[n - 1] = split_store ? kReflSplitFlag : 0.0;
  cluster.sync();
  if (n < 3) {
    if (threadIdx.x == 0) {
      if (n == 2) {
        if (rank == 0) d[0] = O::to_d(own(0, 0));
        if (rank == 1) {
          d[1] = O::to_d(own(1, 1));
          e[0] = O::to_d(own(1, 0));
        }
      } else if (rank == 0) {
        d[0] = O::to_d(own(0, 0));
      }
    }
    return;
  }
  // reflector 0 from column 0, gathered from the owners
  for (int t = threadIdx.x; t < n - 1; t += blockDim.x) {
    const int i = 1 + t;
    vsb[t] = cluster.map_shared_rank(rows, i % kClusterSize)[(size_t)(i / kClusterSize) * n];
  }
  __syncthreads();
  if (threadIdx.x == 0 && rank == 0) d[0] = O::to_d(own(0, 0));
  T tk = make_reflector(0, vsb);
  __syncthreads();
  for (int k = 0; k + 2 < n; ++k) {
    const int m1 = n - k - 1;
    const int buf = k & 1;
    T *vs = vsb + (size_t)buf * n;
    T *ps = psb + (size_t)buf * nloc_max;
    T *colbuf = colb + (size_t)buf * nloc_max;
    const int lfirst = first_local(k + 1);
    if (rank == 0) {
      if (split_store)
        for (int t = threadIdx.x; t < m1; t += blockDim.x)
          reinterpret_cast<T *>(Ag)[(int64_t)k * n + k + 1 + t] = vs[t];
      else
        for (int t = threadIdx.x; t < m1; t += blockDim.x) Ag[(int64_t)k * n + k + 1 + t] = O::store(vs[t]);
    }
    if (threadIdx.x == 32 && k > 0 && rank == k % kClusterSize) d[k] = O::to_d(own(k, k));
    // (1) p_k = tau A22 v for own rows (warp w takes the local rows li = w mod
    // nw, four at a time; the same rows it updates below), per-warp partial p.v
    Acc pv = O::acc0();
    const int l00 = lfirst + ((wid - lfirst) % nw + nw) % nw;  // first local row >= lfirst with li = wid mod nw
    for (int l0 = l00; l0 < nloc; l0 += 4 * nw) {
      const int l1 = l0 + nw < nloc ? l0 + nw : l0, l2 = l0 + 2 * nw < nloc ? l0 + 2 * nw : l0,
                l3 = l0 + 3 * nw < nloc ? l0 + 3 * nw : l0;
      const T *r0 = rows + (size_t)l0 * n + (k + 1), *r1 = rows + (size_t)l1 * n + (k + 1),
              *r2 = rows + (size_t)l2 * n + (k + 1), *r3 = rows + (size_t)l3 * n + (k + 1);
      Acc a0 = O::acc0(), a1 = O::acc0(), a2 = O::acc0(), a3 = O::acc0();
      for (int j = lane; j < m1; j += 32) {
        const T vj = vs[j];
        O::dot(a0, r0[j], vj);
        O::dot(a1, r1[j], vj);
        O::dot(a2, r2[j], vj);
        O::dot(a3, r3[j], vj);
      }
      const T c = O::mul(warp_sum4(O::fin(a0), O::fin(a1), O::fin(a2), O::fin(a3)), tk);
      T pq[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) pq[q] = O::shfl(c, 8 * q);
      if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int li = l0 + q * nw;
          if (li < nloc) {
            ps[li] = pq[q];
            O::dot(pv, pq[q], vs[rank + li * kClusterSize - (k + 1)]);
          }
        }
      }
    }
    if (lane == 0) kpw[buf][wid] = O::fin(pv);
    // (2) column k+1 of own rows k+2.. before this step's update, for every CTA
    for (int li = first_local(k + 2) + threadIdx.x; li < nloc; li += blockDim.x)
      colbuf[li] = rows[(size_t)li * n + (k + 1)];
    cluster.sync();
    // (3) p.v and w_k for all rows (p gathered from the owners); the
    // column k+1 copies gathered alongside
    const bool next = k + 3 < n;  // a reflector k+1 follows
    T *X = vsb + (size_t)(buf ^ 1) * n;  // column k+1 of rows k+2.., then v_{k+1}
    T half;
    if (!kOneWarp || wid == 0) {
      const T K = cluster_partial_sum(cluster, kpw, buf);
      half = O::half_prod(tk, K);
      if (kOneWarp && lane == 0) scal[2] = half;
    }
    if (kOneWarp) {
      __syncthreads();
      half = scal[2];
    }
    for (int t = threadIdx.x; t < m1; t += blockDim.x) {
      const int i = k + 1 + t;
      const int r = i % kClusterSize, li = i / kClusterSize;
      const T p = cluster.map_shared_rank(psb, r)[(size_t)buf * nloc_max + li];
      wv[t] = O::axpy_neg(p, half, vs[t]);
      if (next && t >= 1) X[t - 1] = cluster.map_shared_rank(colb, r)[(size_t)buf * nloc_max + li];
    }
    __syncthreads();
    // (4) column k+1 after this step's update, for rows k+2.. (the same
    // expression the owners evaluate below, so bitwise their values)
    if (next)
      for (int t = 1 + threadIdx.x; t < m1; t += blockDim.x)
        X[t - 1] = O::rank2(X[t - 1], vs[t], wv[0], wv[t], vs[0]);
    // (5) A22 -= v w^T + w v^T on own rows
    for (int li = l00; li < nloc; li += nw) {
      const int t = rank + li * kClusterSize - (k + 1);
      T *row = rows + (size_t)li * n + (k + 1);
      const T vi = vs[t], wi = wv[t];
      for (int j = lane; j < m1; j += 32) row[j] = O::rank2(row[j], vi, wv[j], wi, vs[j]);
    }
    // (6) reflector k+1
    if (next) {
      __syncthreads();
      tk = make_reflector(k + 1, X);
    }
    __syncthreads();
  }
  // the last 2 x 2 block, from the owners' rows after the last update
  if (threadIdx.x == 0) {
    if (rank == (n - 2) % kClusterSize) d[n - 2] = O::to_d(own(n - 2, n - 2));
    if (rank == (n - 1) % kClusterSize) {
      d[n - 1] = O::to_d(own(n - 1, n - 1));
      e[n - 2] = O::to_d(own(n - 1, n - 2));
    }
  }
}

// Shared memory of tridiag_cluster_onchip for n AOs.
template <typename T>
__host__ __device__ constexpr size_t onchip_smem_bytes(int n) {
  return sizeof(T) * ((size_t)((n + kClusterSize - 1) / kClusterSize) * (n + 4) + 3 * (size_t)n);
}
// Molecules whose rows need at most this much shared memory per CTA run in
// a launch sized for it, which lets two CTAs share an SM (FP64 up to 320
// AOs, every FP32 pass up to 400); the others in a launch with one CTA per
// SM.  The SCF's tridiagonalisation is latency-bound, so two clusters per
// set of SMs keep the pipes busier.
constexpr size_t kOnchipSmallBytes = 110 * 1024;

__global__ void __cluster_dims__(kClusterSize, 1, 1) __launch_bounds__(kTrdClThreads)
    k_tridiag_cluster(DevPlan pl, Work w, const int32_t *mol_list, int tail, int big, int df64_mode) {
  cg::cluster_group cluster = cg::this_cluster();
  const int m = list_mol(w, mol_list, blockIdx.x / kClusterSize);
  if (m < 0) return;  // the whole cluster
  const MolDesc md = pl.mol[m];
  extern __shared__ double sm[];
  __shared__ double nrmw[2][kClWarps], kpw[2][kClWarps], scal[4];
  // uniform over the cluster; FP32 passes of molecules that fit in shared
  // memory run in k_tridiag_smem (in the tail of a batch only those up to
  // kTailClusterMinN AOs), molecules above kClusterBlockedMinN AOs in
  // k_tridiag_cluster_blocked
  const bool smem32 = w.prec[m] == 0 && md.nao <= kSmemTridiagMaxN && !(tail && md.nao > kTailClusterMinN);
  // the launch for small or for large shared-memory needs
  const size_t need = w.prec[m] ? onchip_smem_bytes<double>(md.nao) : onchip_smem_bytes<float>(md.nao);
  const bool other_launch = big ? need <= kOnchipSmallBytes : need > kOnchipSmallBytes;
  const bool done = (w.phase[m] == kPhaseDone) || smem32 || md.nao > kClusterBlockedMinN || other_launch;
  if (!done) {
    // df64_mode: 0 native FP64; 1 double-float, reflectors stored as FP64;
    // 2 double-float, reflectors stored as pairs
    if (w.prec[m] && df64_mode)
      tridiag_cluster_onchip<df64>(cluster, md, w, reinterpret_cast<df64 *>(sm),
                                   reinterpret_cast<df64(*)[kClWarps]>(nrmw),
                                   reinterpret_cast<df64(*)[kClWarps]>(kpw), reinterpret_cast<df64 *>(scal),
                                   df64_mode == 2);
    else if (w.prec[m])
      tridiag_cluster_onchip<double>(cluster, md, w, sm, nrmw, kpw, scal, false);
    else
      tridiag_cluster_onchip<float>(cluster, md, w, reinterpret_cast<float *>(sm),
                                    reinterpret_cast<float(*)[kClWarps]>(nrmw),
                                    reinterpret_cast<float(*)[kClWarps]>(kpw), reinterpret_cast<float *>(scal), false);
  }
  // no CTA leaves while others may still read its shared memory
  cluster.sync();
}

// ---------------------------------------------------------------------------
// Blocked Householder tridiagonalisation on a thread-block cluster (8 SMs
// per molecule) for molecules above kClusterBlockedMinN AOs.
//
// Rows are owned cyclically (row i by CTA i mod 8).  Columns are reduced in
// panels of kPanel (LAPACK's dlatrd/dsytrd split): within a panel the
// trailing matrix is left as it was at the panel start, and column c's
// reflector and its vector w come from it plus the panel's earlier pairs
// (v_l, w_l):
//   a   = A[:, c] - sum_l (v_l w_l[c] + w_l v_l[c])
//   p   = tau (A22 v - V (W^T v) - W (V^T v)),   w = p - tau/2 (p.v) v
// and the rank-2 updates of the panel are applied to the trailing matrix at
// its end in one pass (A22 -= V W^T + W V^T).  The matrix is therefore read
// once per column (A22 v) and read and written once per panel, instead of
// read twice and written once per column.
//
// Per column two cluster barriers: after the own rows' corrected column
// entries are published (every CTA gathers the whole column from
// distributed shared memory and builds the reflector), and after the
// partial sums of A22 v, V^T v, W^T v are published.  The w of the next
// row (c + 1), which the next column's correction needs before any
// barrier, is computed identically by every CTA.
//
// Storage: v of column c goes to row c right of the diagonal (the
// back-transformation reads it there); the panel's w vectors go to the
// eigenvector matrix Z, free until the inverse iteration, as W[l][i]
// (row-major, l < kPanel).  Same outputs d, e, tau as k_tridiag.
// ---------------------------------------------------------------------------
constexpr int kTrdBlkThreads = 512;
constexpr int kPanel = 32;    // columns per panel
constexpr int kUpdRows = 64;  // own rows per trailing-update tile
constexpr int kUpdCols = 64;  // columns per trailing-update tile

// dynamic shared memory of k_tridiag_cluster_blocked for molecules up to maxn AOs
// (laid out in 8-byte slots for both precisions)
inline size_t tridiag_cluster_smem_bytes(int maxn) {
  const size_t slots = 2 * (size_t)maxn + (size_t)maxn / kClusterSize + 2 + 6 * kPanel + 4 +
                       2 * (size_t)kPanel * (kUpdRows + kUpdCols);
  return sizeof(double) * slots;
}

// row . v over m1 entries, lanes strided, four loads in flight per lane;
// the warp sum is returned in every lane
template <typename T, bool CG>
__device__ __forceinline__ T row_dot(const T *row, const T *v, int m1, int lane) {
  T a0 = T(0), a1 = T(0), a2 = T(0), a3 = T(0);
  int t = lane;
  for (; t + 96 < m1; t += 128) {
    a0 += (CG ? ld_cg(row + t) : row[t]) * v[t];
    a1 += (CG ? ld_cg(row + t + 32) : row[t + 32]) * v[t + 32];
    a2 += (CG ? ld_cg(row + t + 64) : row[t + 64]) * v[t + 64];
    a3 += (CG ? ld_cg(row + t + 96) : row[t + 96]) * v[t + 96];
  }
  for (; t < m1; t += 32) a0 += (CG ? ld_cg(row + t) : row[t]) * v[t];
  return warp_sum((a0 + a1) + (a2 + a3));
}

template <typename T>
__device__ __forceinline__ void tridiag_cluster_blocked(cg::cluster_group &cluster, const MolDesc &md,
                                                        const Work &w, T *sm, T *red) {
  const int rank = (int)cluster.block_rank();
  const int n = md.nao;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int NW = kTrdBlkThreads / 32;
  T *A = mat_view<T>(w.A, md.mat0);
  T *W = mat_view<T>(w.Z, md.mat0);  // W[l * n + i], l < kPanel
  double *d = w.d + md.ao0, *e = w.e + md.ao0, *tau = w.tau + md.ao0;
  // shared memory (8-byte slots, see tridiag_cluster_smem_bytes)
  T *vs = sm;                                              // [n] reflector of the current column
  T *xs = sm + n;                                          // [n] own corrected column entries (DSMEM)
  T *ys = sm + 2 * n;                                      // [n / 8 + 1] own rows' A22 v
  T *part = ys + n / kClusterSize + 2;                     // [2 kPanel + 2] own partial sums (DSMEM)
  T *x12 = part + 2 * kPanel + 2;                          // [2 kPanel] totals of W^T v, V^T v
  T *coef = x12 + 2 * kPanel;                              // [2 kPanel + 2] row c's W, V entries; scalars
  T *tile = coef + 2 * kPanel + 2;                         // trailing-update tiles
  constexpr int kNorm = 2 * kPanel, kVav = 2 * kPanel + 1;
  T wnext = T(0);  // w of row c + 1 (identical in every CTA)
  // own rows are i = rank + 8 g
  auto first_own = [&](int lo) {  // smallest own row >= lo
    return lo + ((rank - lo) % kClusterSize + kClusterSize) % kClusterSize;
  };
  for (int p0 = 0; p0 + 2 < n; p0 += kPanel) {
    const int pw = min(kPanel, n - 2 - p0);
    for (int jj = 0; jj < pw; ++jj) {
      const int c = p0 + jj;
      const int m1 = n - c - 1;
      // --- A: corrected entries of column c in the own rows i > c ---------
      // coefficients of row c: W[l][c], V[l][c] = A[p0 + l][c]; the previous
      // column's pair is not yet in global memory for other CTAs: its w(c)
      // is wnext, its v(c) = 1, and its v in the own rows is still in vs
      if (tid < jj) {
        coef[tid] = (tid == jj - 1) ? wnext : ld_cg(W + (int64_t)tid * n + c);
        coef[kPanel + tid] = (tid == jj - 1) ? T(1) : ld_cg(A + (int64_t)(p0 + tid) * n + c);
      }
      __syncthreads();
      T nrm = T(0);
      for (int i = first_own(c + 1) + kClusterSize * tid; i < n; i += kClusterSize * kTrdBlkThreads) {
        T x = A[(int64_t)i * n + c];
        int l = 0;
        for (; l + 8 < jj; l += 8) {  // eight pairs of loads in flight
          T va[8], wa[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            va[u] = ld_cg(A + (int64_t)(p0 + l + u) * n + i);
            wa[u] = W[(int64_t)(l + u) * n + i];
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) x -= va[u] * coef[l + u] + wa[u] * coef[kPanel + l + u];
        }
        for (; l + 1 < jj; ++l)
          x -= ld_cg(A + (int64_t)(p0 + l) * n + i) * coef[l] + W[(int64_t)l * n + i] * coef[kPanel + l];
        if (jj > 0) x -= vs[i - c] * coef[jj - 1] + W[(int64_t)(jj - 1) * n + i] * coef[kPanel + jj - 1];
        xs[i - c - 1] = x;
        if (i > c + 1) nrm += x * x;
      }
      nrm = block_sum(nrm, red);
      if (tid == 0) part[kNorm] = nrm;
      cluster.sync();
      // --- B: reflector, A22 v and the partial sums -------------------------
      T xn2 = T(0);
      {
        T pr[kClusterSize];
#pragma unroll
        for (int r = 0; r < kClusterSize; ++r) pr[r] = *cluster.map_shared_rank(part + kNorm, r);
#pragma unroll
        for (int r = 0; r < kClusterSize; ++r) xn2 += pr[r];
      }
      for (int t = tid; t < m1; t += kTrdBlkThreads)
        vs[t] = *cluster.map_shared_rank(xs + t, (c + 1 + t) % kClusterSize);
      __syncthreads();
      const T alpha = vs[0];
      T tk = T(0), scale = T(0), beta = alpha;
      if (xn2 != T(0)) {
        beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
        tk = (beta - alpha) / beta;
        scale = T(1) / (alpha - beta);
      }
      if (rank == 0 && tid == 0) {
        T dc = ld_cg(A + (int64_t)c * n + c);
        for (int l = 0; l < jj; ++l) dc -= T(2) * coef[l] * coef[kPanel + l];
        d[c] = dc;
        e[c] = beta;
        tau[c] = tk;
      }
      __syncthreads();  // every thread has read alpha
      for (int t = tid; t < m1; t += kTrdBlkThreads) vs[t] = (t == 0) ? T(1) : vs[t] * scale;
      __syncthreads();
      // y = A22 v for the own rows, four rows per warp at a time (two
      // loads of each in flight per lane), and for row c + 1 in every CTA
      // (by warp 0, in the same order everywhere)
      T s1 = T(0), s2 = T(0), svav = T(0);  // lane l: partial W^T v, V^T v
      {
        constexpr int kRows = 4;
        constexpr int kStride = kClusterSize * NW;  // between a warp's rows
        const int own0 = first_own(c + 1);
        for (int i0 = own0 + kClusterSize * wid; i0 < n; i0 += kRows * kStride) {
          const T *row[kRows];
          bool ok[kRows];
#pragma unroll
          for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * kStride;
            ok[u] = i < n && i != c + 1;  // row c + 1 is taken below
            row[u] = A + (int64_t)(ok[u] ? i : i0) * n + (c + 1);
          }
          // the W and V entries of these rows (lane l < jj), loaded ahead
          T wl[kRows], vl[kRows];
#pragma unroll
          for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * kStride;
            const bool use = ok[u] && lane < jj;
            wl[u] = use ? W[(int64_t)lane * n + i] : T(0);
            vl[u] = use ? ld_cg(A + (int64_t)(p0 + lane) * n + i) : T(0);
          }
          T acc[kRows] = {};
          int t = lane;
          for (; t + 32 < m1; t += 64) {
            const T v0 = vs[t], v1 = vs[t + 32];
            T r0[kRows], r1[kRows];
#pragma unroll
            for (int u = 0; u < kRows; ++u) {
              r0[u] = row[u][t];
              r1[u] = row[u][t + 32];
            }
#pragma unroll
            for (int u = 0; u < kRows; ++u) acc[u] += r0[u] * v0 + r1[u] * v1;
          }
          if (t < m1) {
            const T v0 = vs[t];
#pragma unroll
            for (int u = 0; u < kRows; ++u) acc[u] += row[u][t] * v0;
          }
#pragma unroll
          for (int u = 0; u < kRows; ++u) {
            const int i = i0 + u * kStride;
            if (!ok[u]) continue;  // uniform over the warp
            const T y = warp_sum(acc[u]);
            const T vi = vs[i - c - 1];
            if (lane == 0) ys[i / kClusterSize] = y;
            svav += vi * y;  // identical in every lane
            s1 += wl[u] * vi;
            s2 += vl[u] * vi;
          }
        }
      }
      if (wid == 0) {
        const T acc = row_dot<T, true>(A + (int64_t)(c + 1) * n + (c + 1), vs, m1, lane);
        if (lane == 0) coef[2 * kPanel] = acc;  // y(c + 1)
        if ((c + 1) % kClusterSize == rank) {
          svav += acc;  // v(c + 1) = 1
          if (lane < jj) {
            s1 += ld_cg(W + (int64_t)lane * n + c + 1);
            s2 += ld_cg(A + (int64_t)(p0 + lane) * n + c + 1);
          }
        }
      }
      // reduce the per-lane partials over the warps: tile[wid][0..2 kPanel]
      {
        T *pw_part = tile + wid * (2 * kPanel + 1);
        pw_part[lane] = s1;
        pw_part[kPanel + lane] = s2;
        if (lane == 0) pw_part[2 * kPanel] = svav;
        __syncthreads();
        if (tid < 2 * kPanel + 1) {
          T s = T(0);
          for (int q = 0; q < NW; ++q) s += tile[q * (2 * kPanel + 1) + tid];
          if (tid < 2 * kPanel) part[tid] = s;
          else part[kVav] = s;
        }
      }
      cluster.sync();
      // --- C: w for the own rows and for row c + 1 ---------------------------
      if (tid <= 2 * kPanel) {
        const int slot = (tid < 2 * kPanel) ? tid : kVav;
        T pr[kClusterSize];
#pragma unroll
        for (int r = 0; r < kClusterSize; ++r) pr[r] = *cluster.map_shared_rank(part + slot, r);
        T s = T(0);
#pragma unroll
        for (int r = 0; r < kClusterSize; ++r) s += pr[r];
        if (tid < 2 * kPanel) x12[tid] = s;
        else coef[2 * kPanel + 1] = s;  // v^T A22 v
      }
      __syncthreads();
      T x1x2 = T(0);
      for (int l = 0; l < jj; ++l) x1x2 += x12[l] * x12[kPanel + l];
      const T K = tk * (coef[2 * kPanel + 1] - T(2) * x1x2);
      const T half = T(0.5) * tk * K;
      // own rows: w_i = tk (y_i - sum_l V[l][i] x1_l - W[l][i] x2_l) - half v_i
      // (four rows per warp at a time, their loads in flight together)
      for (int i0 = first_own(c + 2) + kClusterSize * wid; i0 < n; i0 += 4 * kClusterSize * NW) {
        T corr[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u * kClusterSize * NW;
          corr[u] = (i < n && lane < jj) ? ld_cg(A + (int64_t)(p0 + lane) * n + i) * x12[lane] +
                                               W[(int64_t)lane * n + i] * x12[kPanel + lane]
                                         : T(0);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int i = i0 + u * kClusterSize * NW;
          const T cu = warp_sum(corr[u]);
          if (lane == 0 && i < n) W[(int64_t)jj * n + i] = tk * (ys[i / kClusterSize] - cu) - half * vs[i - c - 1];
        }
      }
      // row c + 1, in every CTA (warp 0, the same order everywhere)
      if (wid == 0) {
        T corr = T(0);
        if (lane < jj)
          corr = ld_cg(A + (int64_t)(p0 + lane) * n + c + 1) * x12[lane] +
                 ld_cg(W + (int64_t)lane * n + c + 1) * x12[kPanel + lane];
        corr = warp_sum(corr);
        const T wn = tk * (coef[2 * kPanel] - corr) - half;  // v(c + 1) = 1
        if (lane == 0) {
          coef[2 * kPanel] = wn;
          if ((c + 1) % kClusterSize == rank) W[(int64_t)jj * n + c + 1] = wn;
        }
      }
      // v into row c (read by other CTAs only after the next barrier)
      if (rank == 0)
        for (int t = tid; t < m1; t += kTrdBlkThreads) A[(int64_t)c * n + c + 1 + t] = vs[t];
      __syncthreads();
      wnext = coef[2 * kPanel];
    }
    // --- trailing update of the own rows i >= pe, columns j >= pe -----------
    cluster.sync();  // every w and v of the panel is visible
    const int pe = p0 + pw;
    T *Vr = tile, *Wr = tile + kPanel * kUpdRows;  // [l][q]
    T *Vc = Wr + kPanel * kUpdRows, *Wc = Vc + kPanel * kUpdCols;  // [l][jc]
    const int ty = tid / 16, tx = tid % 16;  // 2 rows x 4 columns per thread
    for (int rb = first_own(pe); rb < n; rb += kClusterSize * kUpdRows) {
      for (int k = tid; k < pw * kUpdRows; k += kTrdBlkThreads) {
        const int l = k / kUpdRows, q = k % kUpdRows;
        const int i = rb + kClusterSize * q;
        Vr[k] = (i < n) ? ld_cg(A + (int64_t)(p0 + l) * n + i) : T(0);
        Wr[k] = (i < n) ? ld_cg(W + (int64_t)l * n + i) : T(0);
      }
      for (int cb = pe; cb < n; cb += kUpdCols) {
        __syncthreads();
        for (int k = tid; k < pw * kUpdCols; k += kTrdBlkThreads) {
          const int l = k / kUpdCols, jc = k % kUpdCols;
          const int j = cb + jc;
          Vc[k] = (j < n) ? ld_cg(A + (int64_t)(p0 + l) * n + j) : T(0);
          Wc[k] = (j < n) ? ld_cg(W + (int64_t)l * n + j) : T(0);
        }
        __syncthreads();
        T acc[2][4] = {};
        for (int l = 0; l < pw; ++l) {
          T vr[2], wr[2], vc[4], wc[4];
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            vr[a] = Vr[l * kUpdRows + 2 * ty + a];
            wr[a] = Wr[l * kUpdRows + 2 * ty + a];
          }
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            vc[b] = Vc[l * kUpdCols + 4 * tx + b];
            wc[b] = Wc[l * kUpdCols + 4 * tx + b];
          }
#pragma unroll
          for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) acc[a][b] += vr[a] * wc[b] + wr[a] * vc[b];
        }
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          const int i = rb + kClusterSize * (2 * ty + a);
          if (i >= n) continue;
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int j = cb + 4 * tx + b;
            if (j < n) A[(int64_t)i * n + j] -= acc[a][b];
          }
        }
      }
      __syncthreads();
    }
    cluster.sync();  // updated rows visible before the next panel
  }
  if (rank == 0 && tid == 0) {
    if (n >= 2) {
      d[n - 2] = ld_cg(A + (int64_t)(n - 2) * n + (n - 2));
      d[n - 1] = ld_cg(A + (int64_t)(n - 1) * n + (n - 1));
      e[n - 2] = ld_cg(A + (int64_t)(n - 1) * n + (n - 2));
    } else {
      d[0] = ld_cg(A);
    }
  }
}

__global__ void __cluster_dims__(kClusterSize, 1, 1) __launch_bounds__(kTrdBlkThreads, 1)
    k_tridiag_cluster_blocked(DevPlan pl, Work w, const int32_t *mol_list) {
  cg::cluster_group cluster = cg::this_cluster();
  const int m = list_mol(w, mol_list, blockIdx.x / kClusterSize);
  if (m < 0) return;  // the whole cluster
  const MolDesc md = pl.mol[m];
  extern __shared__ double sm[];
  __shared__ double red[32];
  // uniform over the cluster; smaller molecules run in k_tridiag_cluster
  if (w.phase[m] == kPhaseDone || md.nao <= kClusterBlockedMinN) return;
  if (w.prec[m])
    tridiag_cluster_blocked<double>(cluster, md, w, sm, red);
  else
    tridiag_cluster_blocked<float>(cluster, md, w, reinterpret_cast<float *>(sm), reinterpret_cast<float *>(red));
  cluster.sync();
}

// ---------------------------------------------------------------------------
// eigenvalues of the tridiagonal matrix by Sturm bisection
//
// The count of eigenvalues below x is the number of sign changes of the
// leading principal minors p_j of T - x I (p_{j+1} = (d_j - x) p_j -
// e_{j-1}^2 p_{j-1}); the recurrence needs no division (3 FP64 operations
// per step instead of ~11 for the pivot form), is rescaled by exact powers
// of two against overflow/underflow, and its signs are read as integer bits.
// A zero minor is replaced by a tiny value of the opposite sign of its
// predecessor (the pivot form's choice of a negative pivot).
// All eigenvalues are bracketed to 1e-4 Eh first; only those that can carry
// occupation (below the LUMO bracket + 60 kT + 0.01 Eh) are refined to full
// precision: for the rest (E - E_F)/kT >= 50, where the occupation is
// exactly zero and only their count enters the Fermi iteration.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int sturm_count(const double *ds, const double *e2, int n, double x,
                                           double pivmin) {
  double pm = 1.0;           // p_{j-1}
  double pc = ds[0] - x;     // p_j
  if (pc == 0.0) pc = -pivmin;
  int cnt = (int)((unsigned long long)__double_as_longlong(pc) >> 63);
  for (int j = 1; j < n; ++j) {
    double pn = fma(ds[j] - x, pc, -e2[j - 1] * pm);
    const long long bits = __double_as_longlong(pn);
    const long long bc = __double_as_longlong(pc);
    // zero test on the bits (an integer instruction, not an FP64 compare)
    if ((bits << 1) == 0) pn = (bc < 0) ? pivmin : -pivmin;
    const long long bn = __double_as_longlong(pn);
    cnt += (int)((unsigned long long)(bn ^ bc) >> 63);
    const int ex = (int)((bits >> 52) & 0x7ff);
    pm = pc;
    pc = pn;
    if (ex > 1023 + 400) {         // |p| > 2^400: scale both down by 2^-400
      pm *= 0x1p-400;
      pc *= 0x1p-400;
    } else if (ex < 1023 - 400) {  // |p| < 2^-400 (or zero): scale up
      const int exm = (int)((__double_as_longlong(pm) >> 52) & 0x7ff);
      if (exm < 1023 - 200) {
        pm *= 0x1p+400;
        pc *= 0x1p+400;
      }
    }
  }
  return cnt;
}

// FP32 form of the same recurrence (FP32 passes): |d - x| and e^2 stay
// below 2^20 for xTB Hamiltonians in Hartree, so rescaling by 2^+-40 keeps
// every minor inside the FP32 range.
__device__ __forceinline__ int sturm_count(const float *ds, const float *e2, int n, float x,
                                           float pivmin) {
  float pm = 1.0f;
  float pc = ds[0] - x;
  if (pc == 0.0f) pc = -pivmin;
  int cnt = (int)((unsigned)__float_as_int(pc) >> 31);
  for (int j = 1; j < n; ++j) {
    float pn = fmaf(ds[j] - x, pc, -e2[j - 1] * pm);
    const int bits = __float_as_int(pn);
    const int bc = __float_as_int(pc);
    if (pn == 0.0f) pn = (bc < 0) ? pivmin : -pivmin;
    const int bn = __float_as_int(pn);
    cnt += (int)((unsigned)(bn ^ bc) >> 31);
    const int ex = (bits >> 23) & 0xff;
    pm = pc;
    pc = pn;
    if (ex > 127 + 40) {
      pm *= 0x1p-40f;
      pc *= 0x1p-40f;
    } else if (ex < 127 - 40) {
      const int exm = (__float_as_int(pm) >> 23) & 0xff;
      if (exm < 127 - 20) {
        pm *= 0x1p+40f;
        pc *= 0x1p+40f;
      }
    }
  }
  return cnt;
}


constexpr int kBisectGroup = 8;  // lanes per eigenvalue in the multisection

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
// biased binary exponent field of x (0 for zero and subnormals)
__device__ __forceinline__ int dexp(double x) { return (int)((dbits(x) >> 52) & 0x7ff); }

// Newton correction -p_n(x) / p_n'(x) of the characteristic polynomial
// p_n(x) = det(T - x I) of the tridiagonal (ds, e2 = e^2):
//   p_{j+1} = (d_j - x) p_j - e_{j-1}^2 p_{j-1},
//   p'_{j+1} = (d_j - x) p'_j - p_j - e_{j-1}^2 p'_{j-1},
// all four running values rescaled together by powers of two.
__device__ __forceinline__ double newton_correction(const double *ds, const double *e2, int n, double x) {
  double pm = 1.0, pc = ds[0] - x;  // p_{j-1}, p_j
  double qm = 0.0, qc = -1.0;       // p'_{j-1}, p'_j
  for (int j = 1; j < n; ++j) {
    const double a = ds[j] - x, b = e2[j - 1];
    const double pn = fma(a, pc, -b * pm);
    const double qn = fma(a, qc, -fma(b, qm, pc));
    pm = pc;
    pc = pn;
    qm = qc;
    qc = qn;
    // largest binary exponent of the four running values, from their bits
    // (integer instructions; FP64 max/abs would hold the FP64 pipe)
    const int ex = max(max(dexp(pc), dexp(qc)), max(dexp(pm), dexp(qm)));
    if (ex > 1023 + 400) {
      pm *= 0x1p-400; pc *= 0x1p-400; qm *= 0x1p-400; qc *= 0x1p-400;
    } else if (ex < 1023 - 400 && ((dbits(pc) | dbits(qc) | dbits(pm) | dbits(qm)) << 1) != 0) {
      pm *= 0x1p+400; pc *= 0x1p+400; qm *= 0x1p+400; qc *= 0x1p+400;
    }
  }
  return (qc != 0.0 && isfinite(pc) && isfinite(qc)) ? -pc / qc : 0.0;
}

// Eigenvalues of one molecule's tridiagonal matrix.
//
// Only eigenvalues that can carry occupation are computed: those below the
// cut = (LUMO bracket) + 60 kT + 0.01 Eh.  Above it (E - E_F)/kT >= 50, where
// the occupation is exactly zero, so those eigenvalues only enter the Fermi
// iteration through their count; they get placeholder values above the cut
// (ascending), which gives the same occupations.
//
// FP32 pass: bisection of the FP32 copy of the matrix to FP32 resolution.
// FP64 pass: the same FP32 bisection as the start value, then Newton on the
// FP64 characteristic polynomial (quadratic convergence from ~1e-7), then a
// check with two FP64 Sturm counts that the result is the eigenvalue of this
// index; on failure (a near-degenerate cluster) full FP64 bisection.  This
// needs ~8 FP64 count-equivalents per eigenvalue instead of ~55.
// (Every loop is bounded: a non-finite matrix ends with a garbage value,
// which the SCF status check turns into an error, never in a hang.)
template <typename T>
__device__ __forceinline__ void bisect_body(const MolDesc &md, const Work &w, int part, int nsplit,
                                            double kt, double *sm, double *red) {
  const int n = md.nao;
  double *ds = sm, *e2 = sm + n;                                  // FP64 pass only
  float *ds32 = reinterpret_cast<float *>(sm + 2 * n), *e2_32 = ds32 + n;
  __shared__ double s_cut;
  __shared__ int s_ncut;
  const double *d = w.d + md.ao0, *e = w.e + md.ao0;
  double *ev = w.eig + md.ao0;
  constexpr bool kFp64 = sizeof(T) == 8;
  double glo = 1e300, ghi = -1e300, emax = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double ee = (i < n - 1) ? e[i] * e[i] : 0.0;
    if (kFp64) {
      ds[i] = d[i];
      e2[i] = ee;
    }
    ds32[i] = (float)d[i];
    e2_32[i] = (float)ee;
    const double el = (i > 0) ? fabs(e[i - 1]) : 0.0;
    const double er = (i < n - 1) ? fabs(e[i]) : 0.0;
    glo = fmin(glo, d[i] - el - er);
    ghi = fmax(ghi, d[i] + el + er);
    emax = fmax(emax, ee);
  }
  glo = block_min(glo, red);
  ghi = block_max(ghi, red);
  emax = block_max(emax, red);
  const double tnorm = fmax(fabs(glo), fabs(ghi));
  // the FP32 copy differs from the matrix by <= eps32 |T| per entry
  const double glo32 = glo - 4.0 * Num<float>::eps * tnorm * n - 1e-30;
  const double ghi32 = ghi + 4.0 * Num<float>::eps * tnorm * n + 1e-30;
  const float piv32 = (float)(Num<float>::safemin * fmax(1.0, emax));
  const double piv64 = Num<double>::safemin * fmax(1.0, emax);
  // index of the lowest eigenvalue of the alpha channel that is empty at T=0
  const int lumo = min(n - 1, (int)ceil(md.nel[0] - 5.0e-15));
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 32) {
    // LUMO bracket to 1e-4 by 33-section: the warp's 32 points per round
    float lo = (float)glo32, hi = (float)ghi32;
    for (int it = 0; it < 24 && hi - lo > 1.0e-4f; ++it) {
      const float x = lo + (hi - lo) * (float)(lane + 1) / 33.0f;
      const unsigned below = __ballot_sync(0xffffffffu, sturm_count(ds32, e2_32, n, x, piv32) <= lumo);
      const int p = __popc(below);
      const float nlo = (p > 0) ? lo + (hi - lo) * (float)p / 33.0f : lo;
      const float nhi = (p < 32) ? lo + (hi - lo) * (float)(p + 1) / 33.0f : hi;
      if (nlo == lo && nhi == hi) break;
      lo = nlo;
      hi = nhi;
    }
    if (lane == 0) {
      const double cut = (double)hi + 60.0 * kt + 0.01;
      s_cut = cut;
      s_ncut = max(lumo + 1, min(n, sturm_count(ds32, e2_32, n, (float)cut, piv32)));
    }
  }
  __syncthreads();
  const double cut = s_cut;
  const int ncut = s_ncut;
  // eigenvalue idx is located by a group of kBisectGroup lanes: each round
  // evaluates kBisectGroup Sturm counts at once and shrinks the bracket by
  // kBisectGroup + 1 (3.2 bits per round instead of 1)
  const int r = threadIdx.x % kBisectGroup, grp = threadIdx.x / kBisectGroup;
  const unsigned gmask = ((1u << kBisectGroup) - 1u) << (lane & ~(kBisectGroup - 1));
  const int per_block = blockDim.x / kBisectGroup;
  const int stride = per_block * nsplit;
  for (int idx = part * per_block + grp; idx < n; idx += stride) {
    if (idx >= ncut) {
      if (r == 0) ev[idx] = cut + 1.0 + 1.0e-3 * (idx - ncut);  // empty orbital (placeholder)
      continue;
    }
    // FP32 multisection to the resolution of the FP32 copy (eps32 |T|)
    const float ftol = (float)(2.0 * Num<float>::eps * tnorm);
    float lo = (float)glo32, hi = (float)fmax(cut, ghi32);
    constexpr float kInv = 1.0f / (kBisectGroup + 1);
    for (int it = 0; it < 40 && hi - lo > ftol; ++it) {
      const float x = lo + (hi - lo) * ((float)(r + 1) * kInv);
      const unsigned below = __ballot_sync(gmask, sturm_count(ds32, e2_32, n, x, piv32) <= idx) & gmask;
      const int p = __popc(below);
      const float nlo = (p > 0) ? lo + (hi - lo) * ((float)p * kInv) : lo;
      const float nhi = (p < kBisectGroup) ? lo + (hi - lo) * ((float)(p + 1) * kInv) : hi;
      if (nlo == lo && nhi == hi) break;
      lo = nlo;
      hi = nhi;
    }
    if (r != 0) continue;
    ev[idx] = 0.5 * ((double)lo + (double)hi);
  }
  if (!kFp64) return;
  // FP64 pass: Newton polish of every start value of this block, one
  // eigenvalue per thread (all lanes busy: an FP64 warp instruction holds
  // the FP64 pipe for 16 clocks whatever its active lanes), after the
  // start values of the whole block are written
  __syncthreads();
  const double tol = 4.0 * Num<double>::eps * tnorm;
  const double delta = 64.0 * Num<double>::eps * tnorm + 1e-300;
  for (int l = threadIdx.x;; l += blockDim.x) {
    // the block's indices in the order of the loop above
    const int idx = part * per_block + (l % per_block) + (l / per_block) * stride;
    if (idx >= ncut || idx >= n) break;
    double x = ev[idx];
    for (int it = 0; it < 6; ++it) {
      const double dx = newton_correction(ds, e2, n, x);
      x += dx;
      if (!(fabs(dx) > tol)) break;
    }
    const bool ok = isfinite(x) && sturm_count(ds, e2, n, x - delta, piv64) <= idx &&
                    sturm_count(ds, e2, n, x + delta, piv64) > idx;
    if (!ok) {
      double blo = glo - 2.0 * Num<double>::eps * tnorm * n - 1e-300;
      double bhi = fmax(cut, ghi) + 2.0 * Num<double>::eps * tnorm * n + 1e-300;
      for (int it = 0; it < 128; ++it) {
        const double mid = 0.5 * (blo + bhi);
        if (mid <= blo || mid >= bhi) break;
        if (sturm_count(ds, e2, n, mid, piv64) <= idx) blo = mid; else bhi = mid;
      }
      x = 0.5 * (blo + bhi);
    }
    ev[idx] = x;
  }
}

// grid (molecules, parts): block (x, y) handles eigenvalue indices
// y*g + t/8 + j*g*parts (g = threads/8) of molecule mol_list[x] (all
// molecules if mol_list is null)
__global__ void __launch_bounds__(256) k_bisect(DevPlan pl, Work w, double kt, const int32_t *mol_list) {
  const int m = mol_list ? list_mol(w, mol_list, blockIdx.x) : (int)blockIdx.x;
  if (m < 0) return;
  const int part = blockIdx.y;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  if (part * (int)(blockDim.x / kBisectGroup) >= md.nao) return;  // no index of this part (uniform)
  extern __shared__ double sm[];
  __shared__ double red[32];
  if (w.prec[m])
    bisect_body<double>(md, w, part, gridDim.y, kt, sm, red);
  else
    bisect_body<float>(md, w, part, gridDim.y, kt, sm, red);
}



// ---------------------------------------------------------------------------
// eigenvectors of the tridiagonal matrix by inverse iteration
//   output Y[j][i] (component j of eigenvector i) in w.Z, i < kvec
// ---------------------------------------------------------------------------
__device__ __forceinline__ double start_value(int i, int j) {
  const uint32_t h = (uint32_t)i * 2654435761u ^ ((uint32_t)j * 2246822519u + 0x9e3779b9u);
  uint32_t x = h;
  x ^= x >> 15; x *= 0x2c1b3c6du; x ^= x >> 12; x *= 0x297a2d39u; x ^= x >> 15;
  return ((double)(x & 0xffffff) / 16777216.0) - 0.5;
}

constexpr int kInvitThreads = 256;

// One thread per eigenvector: LU factorisation with partial pivoting of
// T - lambda I (factors kept in global scratch, interleaved over eigenvectors
// so that the sequential sweeps of neighbouring threads are coalesced) and
// one inverse-iteration solve.  U1 holds the reciprocals of the pivots, so
// that each element costs one division in the factorisation and none in the
// two solves (a division is ~10 FP64 instructions).
// |a| >= |b|: in FP64 from the bits (an integer compare; an FP64 compare
// holds the FP64 pipe), the same result for every non-NaN pair
template <typename T>
__device__ __forceinline__ bool mag_ge(T a, T b) { return fabs(a) >= fabs(b); }
template <>
__device__ __forceinline__ bool mag_ge<double>(double a, double b) { return (dbits(a) << 1) >= (dbits(b) << 1); }

template <typename T>
__device__ __forceinline__ void invit_factor(int n, int i, T lam, const T *d, const T *e, T pert, T *U1,
                                             T *U2, T *U3, T *LM, T *PV) {
  T u1 = d[0] - lam;
  T u2n = (n > 1) ? e[0] : T(0);
  for (int j = 0; j < n - 1; ++j) {
    const T sub = e[j];
    const T dn = d[j + 1] - lam;
    const T sup2 = (j + 1 < n - 1) ? e[j + 1] : T(0);
    const int64_t o = (int64_t)j * n + i;
    if (mag_ge(u1, sub)) {
      const bool tiny = !mag_ge(u1, pert);
      const T rinv = T(1) / (tiny ? ((u1 < T(0)) ? -pert : pert) : u1);
      const T mult = (u1 == T(0)) ? T(0) : (tiny ? sub / u1 : sub * rinv);
      U1[o] = rinv;
      U2[o] = u2n;
      U3[o] = T(0);
      LM[o] = mult;
      PV[o] = T(0);
      u1 = dn - mult * u2n;
      u2n = sup2;
    } else {
      const T rinv = T(1) / sub;
      const T mult = u1 * rinv;
      U1[o] = rinv;
      U2[o] = dn;
      U3[o] = sup2;
      LM[o] = mult;
      PV[o] = T(1);
      u1 = u2n - mult * dn;
      u2n = -mult * sup2;
    }
  }
  const int64_t o = (int64_t)(n - 1) * n + i;
  U1[o] = T(1) / (!mag_ge(u1, pert) ? ((u1 < T(0)) ? -pert : pert) : u1);
  U2[o] = T(0);
  U3[o] = T(0);
}

template <typename T>
__device__ __forceinline__ void invit_solve(int n, int i, const T *U1, const T *U2, const T *U3, const T *LM,
                                            const T *PV, T *Y) {
  // The sweeps are sequential recurrences; their operands are read in
  // chunks of kChunk rows ahead of the arithmetic, so that one L2 round trip
  // serves kChunk steps instead of one.
  constexpr int kChunk = 8;
  // forward sweep with the running component in a register
  T carry = Y[i];
  for (int j0 = 0; j0 < n - 1; j0 += kChunk) {
    T yn[kChunk], ln[kChunk], pn[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
      const int j = j0 + c;
      if (j < n - 1) {
        const int64_t o = (int64_t)j * n + i;
        yn[c] = Y[o + n];
        ln[c] = LM[o];
        pn[c] = PV[o];
      }
    }
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
      const int j = j0 + c;
      if (j < n - 1) {
        const int64_t o = (int64_t)j * n + i;
        if (pn[c] != T(0)) {
          Y[o] = yn[c];
          carry = carry - ln[c] * yn[c];
        } else {
          Y[o] = carry;
          carry = yn[c] - ln[c] * carry;
        }
      }
    }
  }
  Y[(int64_t)(n - 1) * n + i] = carry;
  // back substitution
  T x1 = T(0), x2 = T(0), nrm = T(0);
  for (int j0 = n - 1; j0 >= 0; j0 -= kChunk) {
    T yv[kChunk], u1[kChunk], u2[kChunk], u3[kChunk];
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
      const int j = j0 - c;
      if (j >= 0) {
        const int64_t o = (int64_t)j * n + i;
        yv[c] = Y[o];
        u1[c] = U1[o];
        u2[c] = U2[o];
        u3[c] = U3[o];
      }
    }
#pragma unroll
    for (int c = 0; c < kChunk; ++c) {
      const int j = j0 - c;
      if (j >= 0) {
        const T sv = (yv[c] - u2[c] * x1 - u3[c] * x2) * u1[c];
        Y[(int64_t)j * n + i] = sv;
        x2 = x1;
        x1 = sv;
        nrm = fmax(nrm, fabs(sv));
      }
    }
  }
  const T inv = (nrm > T(0)) ? T(1) / nrm : T(1);
  T s2 = T(0);
  for (int j = 0; j < n; ++j) {
    const T y = Y[(int64_t)j * n + i] * inv;
    s2 += y * y;
  }
  const T in2 = T(1) / sqrt(s2);
  for (int j = 0; j < n; ++j) {
    const int64_t o = (int64_t)j * n + i;
    Y[o] = (Y[o] * inv) * in2;
  }
}

// Modified Gram-Schmidt inside every cluster of close eigenvalues, one warp
// per cluster, lanes over vector components.
template <typename T>
__device__ __forceinline__ void invit_cluster_mgs(int n, int kvec, const double *ev, double ctol, T *Y) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int c = wid; c < kvec; c += nw) {
    if (c > 0 && ev[c] - ev[c - 1] <= ctol) continue;  // not a cluster start
    int cend = c + 1;
    while (cend < kvec && ev[cend] - ev[cend - 1] <= ctol) ++cend;
    for (int i = c + 1; i < cend; ++i) {
      for (int p = c; p < i; ++p) {
        T dot = T(0);
        for (int j = lane; j < n; j += 32) dot += Y[(int64_t)j * n + p] * Y[(int64_t)j * n + i];
        dot = warp_sum(dot);
        for (int j = lane; j < n; j += 32) Y[(int64_t)j * n + i] -= dot * Y[(int64_t)j * n + p];
      }
      T s2 = T(0);
      for (int j = lane; j < n; j += 32) {
        const T y = Y[(int64_t)j * n + i];
        s2 += y * y;
      }
      s2 = warp_sum(s2);
      const T in2 = T(1) / sqrt(s2);
      for (int j = lane; j < n; j += 32) Y[(int64_t)j * n + i] *= in2;
    }
  }
}

template <typename T>
__device__ __forceinline__ void invit_body(const MolDesc &md, const Work &w, T *sm, double *red) {
  const int n = md.nao;
  const int m = blockIdx.x;
  const int kvec = min(max(w.kvec[m], 0), n);
  T *d = sm, *e = sm + n;
  const double *ev = w.eig + md.ao0;
  T *Y = mat_view<T>(w.Z, md.mat0);
  T *U1 = reinterpret_cast<T *>(w.invit + md.mat0 * 5);
  T *U2 = U1 + (int64_t)n * n;
  T *U3 = U2 + (int64_t)n * n;
  T *LM = U3 + (int64_t)n * n;
  T *PV = LM + (int64_t)n * n;
  double tl = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    d[i] = (T)w.d[md.ao0 + i];
    e[i] = (i < n - 1) ? (T)w.e[md.ao0 + i] : T(0);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double el = (i > 0) ? fabs((double)e[i - 1]) : 0.0;
    const double er = (i < n - 1) ? fabs((double)e[i]) : 0.0;
    tl = fmax(tl, fabs((double)d[i]) + el + er);
  }
  const double tnorm = block_max(tl, red);
  // eigenvalues closer than ctol |T| are orthogonalised explicitly; others
  // come out orthogonal to eps |T| / gap from inverse iteration
  // (FP64: <= 2e-12; FP32: <= 1e-3, enough for the early SCF passes)
  const double ctol = Num<T>::ctol * tnorm;
  const T pert = (T)(Num<T>::eps * tnorm);
  for (int i = threadIdx.x; i < kvec; i += blockDim.x) {
    invit_factor<T>(n, i, (T)ev[i], d, e, pert, U1, U2, U3, LM, PV);
    for (int j = 0; j < n; ++j) Y[(int64_t)j * n + i] = (T)start_value(i, j);
    invit_solve<T>(n, i, U1, U2, U3, LM, PV, Y);
  }
  __syncthreads();
  invit_cluster_mgs<T>(n, kvec, ev, ctol, Y);
  __syncthreads();
  for (int i = threadIdx.x; i < kvec; i += blockDim.x) invit_solve<T>(n, i, U1, U2, U3, LM, PV, Y);
  __syncthreads();
  invit_cluster_mgs<T>(n, kvec, ev, ctol, Y);
}

__global__ void __launch_bounds__(kInvitThreads) k_invit(DevPlan pl, Work w) {
  const int m = blockIdx.x;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  extern __shared__ double sm[];
  __shared__ double red[32];
  if (w.prec[m])
    invit_body<double>(md, w, sm, red);
  else
    invit_body<float>(md, w, reinterpret_cast<float *>(sm), red);
}

// ---------------------------------------------------------------------------
// back-transformation Y <- Q Y, Q = H_0 ... H_{n-3}
// A block owns 32 eigenvector columns and splits the rows over 8 warps:
// per reflector, partial dot products per warp, one reduction in shared
// memory, then every warp updates its rows (coalesced rows of Y).
// ---------------------------------------------------------------------------
constexpr int kBtThreads = 256;

// COLS eigenvector columns per block, kBtThreads / COLS row groups.
template <typename T, int COLS>
__device__ __forceinline__ void backtransform_body(const MolDesc &md, const Work &w, int kvec, int c0, T *vsm,
                                                   T *part, T *sfac) {
  constexpr int kGroups = kBtThreads / COLS;
  const int n = md.nao;
  const T *A = mat_view<T>(w.A, md.mat0);
  const double *tau = w.tau + md.ao0;
  T *Y = mat_view<T>(w.Z, md.mat0);
  const int col = threadIdx.x % COLS, rg = threadIdx.x / COLS;
  const int c = c0 + col;
  const bool active = c < kvec;
  for (int k = n - 3; k >= 0; --k) {
    const T tk = (T)tau[k];
    if (tk == T(0)) continue;  // uniform across the block
    const int m1 = n - k - 1;
    for (int t = threadIdx.x; t < m1; t += blockDim.x) vsm[t] = A[(int64_t)k * n + k + 1 + t];
    __syncthreads();
    T s = T(0);
    if (active)
      for (int r = rg; r < m1; r += kGroups) s += vsm[r] * Y[(int64_t)(k + 1 + r) * n + c];
    part[rg * COLS + col] = s;
    __syncthreads();
    if (rg == 0) {
      T t = T(0);
#pragma unroll
      for (int g = 0; g < kGroups; ++g) t += part[g * COLS + col];
      sfac[col] = t * tk;
    }
    __syncthreads();
    if (active) {
      const T f = sfac[col];
      for (int r = rg; r < m1; r += kGroups) Y[(int64_t)(k + 1 + r) * n + c] -= f * vsm[r];
    }
    __syncthreads();
  }
}

// grid (column groups, molecules): molecule mol_list[y] (all if null)
template <int COLS>
__global__ void __launch_bounds__(kBtThreads) k_backtransform(DevPlan pl, Work w, const int32_t *mol_list) {
  const int m = mol_list ? list_mol(w, mol_list, blockIdx.y) : (int)blockIdx.y;
  if (m < 0) return;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const int kvec = min(max(w.kvec[m], 0), n);
  const int c0 = blockIdx.x * COLS;
  if (c0 >= kvec) return;
  extern __shared__ double vsm[];
  __shared__ double part[kBtThreads];
  __shared__ double sfac[COLS];
  if (w.prec[m])
    backtransform_body<double, COLS>(md, w, kvec, c0, vsm, part, sfac);
  else
    backtransform_body<float, COLS>(md, w, kvec, c0, reinterpret_cast<float *>(vsm),
                                    reinterpret_cast<float *>(part), reinterpret_cast<float *>(sfac));
}

// Back-transformation with one warp per eigenvector: the column lives in
// registers (row r in lane r % 32, slot r / 32), so applying a reflector is a
// warp reduction and a register update, with no CTA barrier; the reflector
// rows are read through L1, shared by the eight warps of a CTA.
// Reflector k is zero in rows r <= k, so slots below (k + 1) / 32 take no
// part: the reflectors are applied in ranges of 32 with the first slot QS a
// compile-time constant (every load of a reflector still in flight at once),
// which halves the FP64 work on average.
template <typename T, int NQ, int QS>
__device__ __forceinline__ void bt_apply_range(T (&y)[NQ], const T *A, const double *tau, int n, int lane,
                                               int khi, int klo) {
  using O = ClOps<T>;
  for (int k = khi; k >= klo; --k) {
    const double tk64 = tau[k];
    if (tk64 == 0.0) continue;
    const T tk = O::from_d(tk64);
    const T *v = A + (int64_t)k * n;  // reflector k: v[r] = A[k][r] multiplies row r > k
    T vq[NQ - QS];
    typename O::Acc acc = O::acc0();
#pragma unroll
    for (int q = QS; q < NQ; ++q) {
      const int r = lane + 32 * q;
      vq[q - QS] = (r > k && r < n) ? v[r] : O::zero();
      O::dot(acc, vq[q - QS], y[q]);
    }
    const T dot = O::mul(cl_warp_sum(O::fin(acc)), tk);
#pragma unroll
    for (int q = QS; q < NQ; ++q) y[q] = O::axpy_neg(y[q], dot, vq[q - QS]);
  }
}

// reflectors kstart, kstart - 1, ..., 0 in the ranges (k + 1) / 32 = QS, QS - 1, ..., 0
template <typename T, int NQ, int QS>
__device__ __forceinline__ void bt_apply_from(T (&y)[NQ], const T *A, const double *tau, int n, int lane,
                                              int kstart) {
  const int klo = 32 * QS - 1 > 0 ? 32 * QS - 1 : 0;
  const int khi = kstart < 32 * QS + 30 ? kstart : 32 * QS + 30;
  if (khi >= klo) bt_apply_range<T, NQ, QS>(y, A, tau, n, lane, khi, klo);
  if constexpr (QS > 0) bt_apply_from<T, NQ, QS - 1>(y, A, tau, n, lane, kstart);
}

// T: the arithmetic (float in FP32 passes; double, or df64 where the
// reflectors are double-float pairs, in FP64 passes); the eigenvector
// matrix is FP32 or FP64 in memory (ClOps<T>::G)
template <typename T, int NQ>
__device__ __forceinline__ void backtransform_column(const MolDesc &md, const Work &w, int c) {
  using O = ClOps<T>;
  using G = typename O::G;
  const int n = md.nao;
  const int lane = threadIdx.x & 31;
  const T *A = reinterpret_cast<const T *>(mat_view<G>(w.A, md.mat0));
  const double *tau = w.tau + md.ao0;
  G *Y = mat_view<G>(w.Z, md.mat0);
  T y[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int r = lane + 32 * q;
    y[q] = (r < n) ? O::load(Y[(int64_t)r * n + c]) : O::zero();
  }
  bt_apply_from<T, NQ, NQ - 1>(y, A, tau, n, lane, n - 3);
#pragma unroll
  for (int q = 0; q < NQ; ++q) {
    const int r = lane + 32 * q;
    if (r < n) Y[(int64_t)r * n + c] = O::store(y[q]);
  }
}

// grid (column groups of 8, molecules): molecule mol_list[y] (all if null);
// every molecule has at most 32 * NQ AOs
template <int NQ>
__global__ void __launch_bounds__(256, 2) k_backtransform_warp(DevPlan pl, Work w, const int32_t *mol_list) {
  const int m = mol_list ? list_mol(w, mol_list, blockIdx.y) : (int)blockIdx.y;
  if (m < 0) return;
  if (w.phase[m] == kPhaseDone) return;
  const MolDesc md = pl.mol[m];
  const int kvec = min(max(w.kvec[m], 0), md.nao);
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (c >= kvec) return;  // whole warp
  if (w.prec[m] && w.tau[md.ao0 + md.nao - 1] == kReflSplitFlag)
    backtransform_column<df64, NQ>(md, w, c);
  else if (w.prec[m])
    backtransform_column<double, NQ>(md, w, c);
  else
    backtransform_column<float, NQ>(md, w, c);
}

}  // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
int launch_cholesky(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s) {
  k_cholesky<<<pl.nmol, 512, 0, s>>>(pl, w);
  return 1 + launch_cholesky_blocked(pl, w, maxn, s);
}

void launch_gemm(const DevPlan &pl, const Work &w, const int64_t *tile0, int64_t ntile, int mode,
                 int all, cudaStream_t s) {
  if (ntile > 0) k_gemm<<<(unsigned)ntile, 256, 0, s>>>(pl, w, tile0, mode, all);
}

void launch_lowp_copies(const DevPlan &pl, const Work &w, cudaStream_t s) {
  k_lowp_copies<<<pl.nmol, 256, 0, s>>>(pl, w);
}

void launch_tridiag(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s) {
  const size_t smem = sizeof(double) * 2 * (size_t)maxn;
  k_tridiag<<<pl.nmol, kTrdThreads, smem, s>>>(pl, w);
}

// FP32 passes of molecules with at most kSmemTridiagMaxN AOs, one launch
// per size class.
size_t tridiag_smem_bytes(int nmax, int nwarps) {
  const int nloc = nmax < kSmemLocalMaxN ? nmax : kSmemLocalMaxN;
  return sizeof(float) * ((size_t)nloc * (nloc + 1) / 2 + 5 * (size_t)nmax + (size_t)nwarps * nloc);
}

void launch_tridiag_smem(const DevPlan &pl, const Work &w, cudaStream_t s, bool tail) {
  for (int c = 0; c < kSmemBins; ++c) {
    if (pl.bin_count[c] <= 0) continue;
    const int nw = pl.bin_warps[c] ? pl.bin_warps[c] : kSmemBinWarps[c];
    const size_t smem = tridiag_smem_bytes(pl.bin_maxn[c], nw);
    if (nw == 8)
      k_tridiag_smem<8><<<pl.bin_count[c], 256, smem, s>>>(pl, w, pl.bin_mols[c], tail ? 1 : 0);
    else if (nw == 16)
      k_tridiag_smem<16><<<pl.bin_count[c], 512, smem, s>>>(pl, w, pl.bin_mols[c], tail ? 1 : 0);
    else
      k_tridiag_smem<32><<<pl.bin_count[c], 1024, smem, s>>>(pl, w, pl.bin_mols[c], tail ? 1 : 0);
  }
}


// Cluster tridiagonalisation for the molecules listed in mol_list (device).
// Returns the number of launches.
int launch_tridiag_cluster(const DevPlan &pl, const Work &w, const int32_t *mol_list, int count, int maxn,
                           cudaStream_t s, bool tail, bool df64_passes) {
  if (count <= 0) return 0;
  // two size classes of shared memory (kOnchipSmallBytes)
  const size_t need = onchip_smem_bytes<double>(min(maxn, kClusterBlockedMinN));
  const size_t small = need < kOnchipSmallBytes ? need : kOnchipSmallBytes;
  // double-float reflectors stay pairs when the one-warp back-transformation
  // (plans of at most 384 AOs) applies them
  const int t = tail ? 1 : 0, sp = df64_passes ? (maxn <= kBtWarpMaxN ? 2 : 1) : 0;
  k_tridiag_cluster<<<count * kClusterSize, kTrdClThreads, small, s>>>(pl, w, mol_list, t, 0, sp);
  int launches = 1;
  if (need > kOnchipSmallBytes) {
    k_tridiag_cluster<<<count * kClusterSize, kTrdClThreads, need, s>>>(pl, w, mol_list, t, 1, sp);
    ++launches;
  }
  if (maxn <= kClusterBlockedMinN) return launches;
  k_tridiag_cluster_blocked<<<count * kClusterSize, kTrdBlkThreads, tridiag_cluster_smem_bytes(maxn), s>>>(
      pl, w, mol_list);
  return launches + 1;
}

// All molecules (mol_list null, count = nmol) with 256 threads per block,
// or the listed ones with `threads` per block and as many blocks as the
// largest molecule needs (more SMs per molecule for a short list).
void launch_bisect(const DevPlan &pl, const Work &w, int maxn, double kt, const int32_t *mol_list, int count,
                   int threads, cudaStream_t s) {
  if (count <= 0) return;
  const size_t smem = sizeof(double) * 3 * (size_t)maxn;
  const int per_block = threads / kBisectGroup;
  dim3 grid(count, (maxn + per_block - 1) / per_block);
  k_bisect<<<grid, threads, smem, s>>>(pl, w, kt, mol_list);
}



void launch_invit(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s) {
  k_invit<<<pl.nmol, kInvitThreads, sizeof(double) * 2 * (size_t)maxn, s>>>(pl, w);
}

// Warp-per-eigenvector kernel up to 384 AOs; beyond that 32 columns per
// block for the whole batch and 8 per block (4x the blocks per molecule) for
// a short list of molecules.
void launch_backtransform(const DevPlan &pl, const Work &w, int maxn, const int32_t *mol_list, int count,
                          cudaStream_t s) {
  if (count <= 0) return;
  if (maxn <= kBtWarpMaxN) {
    dim3 grid((maxn + 7) / 8, count);
    if (maxn <= 128)
      k_backtransform_warp<4><<<grid, 256, 0, s>>>(pl, w, mol_list);
    else if (maxn <= 256)
      k_backtransform_warp<8><<<grid, 256, 0, s>>>(pl, w, mol_list);
    else
      k_backtransform_warp<12><<<grid, 256, 0, s>>>(pl, w, mol_list);
    return;
  }
  const size_t smem = sizeof(double) * (size_t)maxn;
  if (mol_list) {
    dim3 grid((maxn + 7) / 8, count);
    k_backtransform<8><<<grid, kBtThreads, smem, s>>>(pl, w, mol_list);
  } else {
    dim3 grid((maxn + 31) / 32, count);
    k_backtransform<32><<<grid, kBtThreads, smem, s>>>(pl, w, mol_list);
  }
}



// Dynamic shared-memory limits of the kernels whose footprint grows with the
// largest molecule of a plan.  The attribute is per function and process
// wide, and plans created earlier keep launching, so it only ever grows.
cudaError_t set_linalg_smem_limits(int maxn) {
  static std::mutex mu;
  static size_t cur_smem = 0, cur1 = 0, cur2 = 0, cur3 = 0, cur_c = 0;
  std::lock_guard<std::mutex> lock(mu);
  // every warp count of k_tridiag_smem may serve any size class (autotuning)
  const size_t need_s = tridiag_smem_bytes(maxn < kSmemTridiagMaxN ? maxn : kSmemTridiagMaxN, 32);
  const size_t need1 = sizeof(double) * (size_t)maxn;
  const size_t need2 = sizeof(double) * 2 * (size_t)maxn;
  const size_t need3 = sizeof(double) * 3 * (size_t)maxn;
  const size_t need_c = tridiag_cluster_smem_bytes(maxn);
  // above 48 KB of dynamic plus static shared memory a kernel needs the
  // attribute; the kernels' static arrays take at most 4 KB
  const size_t opt_in = 44 * 1024;
  cudaError_t e = cudaSuccess;
  if (need_s > opt_in && need_s > cur_smem) {
    e = cudaFuncSetAttribute(k_tridiag_smem<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need_s);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_tridiag_smem<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need_s);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_tridiag_smem<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need_s);
    if (e != cudaSuccess) return e;
    cur_smem = need_s;
  }
  if (need1 > opt_in && need1 > cur1) {
    e = cudaFuncSetAttribute(k_backtransform<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need1);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_backtransform<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need1);
    if (e != cudaSuccess) return e;
    cur1 = need1;
  }
  if (need2 > opt_in && need2 > cur2) {
    e = cudaFuncSetAttribute(k_tridiag, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need2);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_invit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need2);
    if (e != cudaSuccess) return e;
    cur2 = need2;
  }
  if (need3 > opt_in && need3 > cur3) {
    e = cudaFuncSetAttribute(k_bisect, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need3);
    if (e != cudaSuccess) return e;
    cur3 = need3;
  }
  // the on-chip cluster tridiagonalisation (up to kClusterBlockedMinN AOs)
  static size_t cur_o = 0;
  const size_t need_o = onchip_smem_bytes<double>(maxn < kClusterBlockedMinN ? maxn : kClusterBlockedMinN);
  if (need_o > opt_in && need_o > cur_o) {
    e = cudaFuncSetAttribute(k_tridiag_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need_o);
    if (e != cudaSuccess) return e;
    cur_o = need_o;
  }
  if (maxn > kClusterBlockedMinN && need_c > cur_c) {
    e = cudaFuncSetAttribute(k_tridiag_cluster_blocked, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)need_c);
    if (e != cudaSuccess) return e;
    cur_c = need_c;
  }
  return e;
}

}  // namespace gbxtb
