// Blocked FP64 Cholesky factorisation S = L L^T and inverse L^-1 for large
// molecules, spread over the whole GPU.
//
// The one-CTA kernel (k_cholesky in linalg.cu) keeps a molecule on one SM,
// whose FP64 pipe needs ~N^3 / 3 clocks for the two triangular O(N^3 / 3)
// stages: 0.7 s at N = 1600, 18 s at N = 6000.  Here a molecule with more
// than kCholBlockMinN AOs is factorised right-looking in 64-column panels:
// per panel one CTA factors the diagonal block on chip, row blocks solve
// against it in parallel, and the trailing lower triangle is updated as a
// set of independent 64 x 64 tiles.  L^-1 is then formed block row by block
// row: the diagonal blocks are inverted in parallel, and block (i, j) is
// -inv(L_ii) sum_{k=j}^{i-1} L_ik X_kj, independent over j.  Output as
// k_cholesky: L^-1 in the lower triangle of w.Linv, L^T in its strict upper
// triangle, diag(L) in w.ldiag.
//
// Reference: scf/unrolling/base.py:141-175 (tad_mctc eighb: Cholesky
// reduction of the generalised eigenproblem).
#include "internal.cuh"

namespace gbxtb {

namespace {

constexpr int kB = 64;  // panel / tile width

__device__ __forceinline__ bool big_mol(const DevPlan &pl, const Work &w, int m) {
  return pl.mol[m].nao > kCholBlockMinN && geom_due(pl, w, m) && w.phase[m] != kPhaseDone;
}

// A = lower triangle of S (row-major), Linv = 0.
__global__ void k_chol_copy(DevPlan pl, Work w) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const int64_t nn = (int64_t)n * n;
  const double *S = w.S + md.mat0;
  double *A = w.A + md.mat0, *X = w.Linv + md.mat0;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nn; e += (int64_t)gridDim.x * blockDim.x) {
    A[e] = S[e];
    X[e] = 0.0;
  }
}

// Panel p, step 1: factor the diagonal block on chip (one CTA per molecule).
__global__ void __launch_bounds__(256) k_chol_diag(DevPlan pl, Work w, int p) {
  const int m = blockIdx.x;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao, k = p * kB;
  if (k >= n) return;
  const int b = min(kB, n - k);
  double *A = w.A + md.mat0;
  __shared__ double T[kB][kB + 1];
  __shared__ int fail;
  if (threadIdx.x == 0) fail = 0;
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int r = e / b, c = e % b;
    T[r][c] = (c <= r) ? A[(int64_t)(k + r) * n + k + c] : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < b; ++c) {
    if (threadIdx.x == 0) {
      const double t = T[c][c];
      if (!(t > 0.0)) {
        fail = 1;
        T[c][c] = 1.0;
      } else {
        T[c][c] = sqrt(t);
      }
    }
    __syncthreads();
    const double dc = T[c][c];
    for (int r = c + 1 + threadIdx.x; r < b; r += blockDim.x) T[r][c] /= dc;
    __syncthreads();
    for (int e = threadIdx.x; e < (b - c - 1) * (b - c - 1); e += blockDim.x) {
      const int r = c + 1 + e / (b - c - 1), q = c + 1 + e % (b - c - 1);
      if (q <= r) T[r][q] -= T[r][c] * T[q][c];
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < b * b; e += blockDim.x) {
    const int r = e / b, c = e % b;
    if (c <= r) A[(int64_t)(k + r) * n + k + c] = T[r][c];
  }
  if (threadIdx.x == 0 && fail) {
    w.status[m] |= GBXTB_MOL_CHOLESKY_FAIL;
    w.phase[m] = kPhaseDone;
  }
}

// Panel p, step 2: rows below the diagonal block, A_ik <- A_ik L_kk^-T.
// grid (row blocks, molecules); one thread per row.
__global__ void __launch_bounds__(kB) k_chol_panel(DevPlan pl, Work w, int p) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao, k = p * kB;
  const int r0 = k + kB + blockIdx.x * kB;
  if (k + kB >= n || r0 >= n) return;
  double *A = w.A + md.mat0;
  __shared__ double Lk[kB][kB + 1];
  for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
    const int r = e / kB, c = e % kB;
    Lk[r][c] = (c <= r) ? A[(int64_t)(k + r) * n + k + c] : 0.0;
  }
  __syncthreads();
  const int r = r0 + threadIdx.x;
  if (r >= n) return;
  double x[kB];
  double *row = A + (int64_t)r * n + k;
#pragma unroll
  for (int c = 0; c < kB; ++c) x[c] = row[c];
  // x L_kk^T = a: forward substitution over the columns
#pragma unroll
  for (int c = 0; c < kB; ++c) {
    double t = x[c];
#pragma unroll
    for (int q = 0; q < c; ++q) t -= x[q] * Lk[c][q];
    x[c] = t / Lk[c][c];
  }
#pragma unroll
  for (int c = 0; c < kB; ++c) row[c] = x[c];
}

// 64 x 64 tile C -= P_i P_j^T (or accumulate into registers) with K = 64:
// 256 threads, 4 x 4 per thread, operands staged in shared memory.
struct TileAcc {
  double v[4][4];
};

__device__ __forceinline__ void tile_mma(const double *Ai, int lda_i, const double *Bj, int ldb_j, int kk,
                                         int rows_i, int rows_j, TileAcc &acc, double (*sa)[kB + 1],
                                         double (*sb)[kB + 1]) {
  // sa[q][r] = Ai[r][q], sb[q][c] = Bj[c][q] for q < kk (kk <= 64)
  for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
    const int r = e / kB, q = e % kB;
    sa[q][r] = (r < rows_i && q < kk) ? Ai[(int64_t)r * lda_i + q] : 0.0;
    sb[q][r] = (r < rows_j && q < kk) ? Bj[(int64_t)r * ldb_j + q] : 0.0;
  }
  __syncthreads();
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int q = 0; q < kk; ++q) {
    double a[4], bb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = sa[q][ty * 4 + u];
      bb[u] = sb[q][tx * 4 + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) acc.v[u][v] = fma(a[u], bb[v], acc.v[u][v]);
  }
  __syncthreads();
}

// Panel p, step 3: trailing lower tiles (ti >= tj > p) -= P_ti P_tj^T.
// grid (tile pairs of the largest molecule, molecules).
__global__ void __launch_bounds__(256) k_chol_update(DevPlan pl, Work w, int p) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao, k = p * kB;
  const int nt = (n + kB - 1) / kB;
  const int rem = nt - p - 1;  // trailing tile rows
  if (rem <= 0 || (int)blockIdx.x >= rem * (rem + 1) / 2) return;
  // decode the lower tile (ti >= tj) of the trailing block
  int ti = 0;
  while ((ti + 1) * (ti + 2) / 2 <= (int)blockIdx.x) ++ti;
  const int tj = blockIdx.x - ti * (ti + 1) / 2;
  const int i0 = (p + 1 + ti) * kB, j0 = (p + 1 + tj) * kB;
  double *A = w.A + md.mat0;
  __shared__ double sa[kB][kB + 1], sb[kB][kB + 1];
  TileAcc acc;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc.v[u][v] = 0.0;
  tile_mma(A + (int64_t)i0 * n + k, n, A + (int64_t)j0 * n + k, n, kB, min(kB, n - i0), min(kB, n - j0), acc,
           sa, sb);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = i0 + ty * 4 + u, c = j0 + tx * 4 + v;
      if (r < n && c < n && c <= r) A[(int64_t)r * n + c] -= acc.v[u][v];
    }
}

// Inverse, step 0: X_jj = inv(L_jj) for every diagonal block (grid (blocks,
// molecules)); column c of X_jj by forward substitution in one thread.
__global__ void __launch_bounds__(kB) k_trinv_diag(DevPlan pl, Work w) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao, k = blockIdx.x * kB;
  if (k >= n) return;
  const int b = min(kB, n - k);
  const double *A = w.A + md.mat0;
  double *X = w.Linv + md.mat0;
  __shared__ double Lk[kB][kB + 1];
  for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
    const int r = e / kB, c = e % kB;
    Lk[r][c] = (r < b && c < b && c <= r) ? A[(int64_t)(k + r) * n + k + c] : 0.0;
  }
  __syncthreads();
  const int c = threadIdx.x;
  if (c >= b) return;
  double x[kB];
#pragma unroll
  for (int r = 0; r < kB; ++r) x[r] = 0.0;
  x[c] = 1.0 / Lk[c][c];
#pragma unroll
  for (int r = 0; r < kB; ++r) {
    if (r <= c || r >= b) continue;
    double t = 0.0;
#pragma unroll
    for (int q = 0; q < kB; ++q)
      if (q >= c && q < r) t += Lk[r][q] * x[q];
    x[r] = -t / Lk[r][r];
  }
#pragma unroll
  for (int r = 0; r < kB; ++r)
    if (r >= c && r < b) X[(int64_t)(k + r) * n + k + c] = x[r];
}

// Inverse, block row i: X_ij = -X_ii sum_{k=j}^{i-1} L_ik X_kj for j < i.
// grid (j, molecules).
__global__ void __launch_bounds__(256) k_trinv_row(DevPlan pl, Work w, int bi) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const int nt = (n + kB - 1) / kB;
  const int bj = blockIdx.x;
  if (bi >= nt || bj >= bi) return;
  const double *A = w.A + md.mat0;
  double *X = w.Linv + md.mat0;
  const int i0 = bi * kB, j0 = bj * kB;
  const int rows_i = min(kB, n - i0);
  __shared__ double sa[kB][kB + 1], sb[kB][kB + 1];
  TileAcc acc;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) acc.v[u][v] = 0.0;
  // T = sum_k L_ik X_kj: sa from L rows i, sb from X^T (columns j of X rows k)
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int bk = bj; bk < bi; ++bk) {
    const int k0 = bk * kB;
    for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
      const int r = e / kB, q = e % kB;
      sa[q][r] = (r < rows_i) ? A[(int64_t)(i0 + r) * n + k0 + q] : 0.0;
      sb[q][r] = X[(int64_t)(k0 + q) * n + j0 + r];  // X_kj(q, r), full blocks below the diagonal
    }
    __syncthreads();
    for (int q = 0; q < kB; ++q) {
      double a[4], bb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        a[u] = sa[q][ty * 4 + u];
        bb[u] = sb[q][tx * 4 + u];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc.v[u][v] = fma(a[u], bb[v], acc.v[u][v]);
    }
    __syncthreads();
  }
  // X_ij = -X_ii T: sa[q][r] = X_ii(r, q), sb[q][c] = T(q, c) staged through
  // shared memory
  for (int e = threadIdx.x; e < kB * kB; e += blockDim.x) {
    const int r = e / kB, q = e % kB;
    sa[q][r] = (r < rows_i && q < rows_i && q <= r) ? X[(int64_t)(i0 + r) * n + i0 + q] : 0.0;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) sb[ty * 4 + u][tx * 4 + v] = acc.v[u][v];
  __syncthreads();
  TileAcc out;
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) out.v[u][v] = 0.0;
  for (int q = 0; q < kB; ++q) {
    double a[4], bb[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      a[u] = sa[q][ty * 4 + u];
      bb[u] = sb[q][tx * 4 + u];
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int v = 0; v < 4; ++v) out.v[u][v] = fma(a[u], bb[v], out.v[u][v]);
  }
#pragma unroll
  for (int u = 0; u < 4; ++u)
#pragma unroll
    for (int v = 0; v < 4; ++v) {
      const int r = i0 + ty * 4 + u, c = j0 + tx * 4 + v;
      if (r < n) X[(int64_t)r * n + c] = -out.v[u][v];
    }
}

// L^T into the strict upper triangle of the L^-1 buffer, diag(L) into ldiag.
__global__ void k_chol_finish(DevPlan pl, Work w) {
  const int m = blockIdx.y;
  if (!big_mol(pl, w, m)) return;
  const MolDesc md = pl.mol[m];
  const int n = md.nao;
  const int64_t nn = (int64_t)n * n;
  const double *A = w.A + md.mat0;
  double *X = w.Linv + md.mat0;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn; t += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(t / n), c = (int)(t % n);
    if (c > r) X[t] = A[(int64_t)c * n + r];
    if (c == r) w.ldiag[md.ao0 + r] = A[t];
  }
}

}  // namespace

// Blocked factorisation of every molecule with more than kCholBlockMinN
// AOs (maxn: largest molecule of the plan); k_cholesky skips those.
int launch_cholesky_blocked(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s) {
  if (maxn <= kCholBlockMinN) return 0;
  const int nt = (maxn + kB - 1) / kB;
  int launches = 0;
  k_chol_copy<<<dim3(64, pl.nmol), 256, 0, s>>>(pl, w);
  ++launches;
  for (int p = 0; p < nt; ++p) {
    k_chol_diag<<<pl.nmol, 256, 0, s>>>(pl, w, p);
    ++launches;
    const int rem = nt - p - 1;
    if (rem > 0) {
      k_chol_panel<<<dim3(rem, pl.nmol), kB, 0, s>>>(pl, w, p);
      k_chol_update<<<dim3(rem * (rem + 1) / 2, pl.nmol), 256, 0, s>>>(pl, w, p);
      launches += 2;
    }
  }
  k_trinv_diag<<<dim3(nt, pl.nmol), kB, 0, s>>>(pl, w);
  for (int bi = 1; bi < nt; ++bi) k_trinv_row<<<dim3(bi, pl.nmol), 256, 0, s>>>(pl, w, bi);
  k_chol_finish<<<dim3(64, pl.nmol), 256, 0, s>>>(pl, w);
  return launches + nt + 1;
}

}  // namespace gbxtb
