// Internal definitions shared by the gbxtb CUDA translation units.
//
// Data layout in HBM (ragged, no padding):
//   * molecules m = 0..nmol-1 own contiguous ranges of atoms, shells and
//     atomic orbitals (AOs); every per-molecule dense matrix (overlap S, core
//     Hamiltonian H0, inverse Cholesky factor, Fock/eigenvector work arrays,
//     density P) is a row-major nao x nao block at offset MolDesc::mat0 of a
//     buffer that packs all molecules back to back;
//   * the shell-resolved Coulomb matrix is an nsh x nsh block at MolDesc::gam0.
#pragma once

#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "../../include/gbxtb.h"

namespace gbxtb {

constexpr int kMaxPrim = GBXTB_MAX_PRIM;
constexpr int kMaxL = 2;

// FP32 passes tridiagonalise in shared memory (packed lower triangle, one
// CTA per molecule, kSmemBinWarps[c] warps for size class c).  On chip fit
// kSmemLocalMaxN AOs: 300 * 301 / 2 + 5 * 400 + 32 * 300 floats = 227 KB,
// all a CTA can have; molecules up to kSmemTridiagMaxN AOs first run their
// leading steps in global memory.  Molecules are launched in size classes
// n <= kSmemBinN[c] (the shared memory of a launch follows its largest).
constexpr int kSmemLocalMaxN = 300;
constexpr int kSmemTridiagMaxN = 400;
constexpr int kSmemBins = 3;
constexpr int kSmemBinN[kSmemBins] = {96, 192, kSmemTridiagMaxN};
constexpr int kSmemBinWarps[kSmemBins] = {8, 16, 32};
// Molecules with more AOs than this are Cholesky-factorised block-wise over
// the whole GPU (cholesky.cu) instead of in one CTA.
constexpr int kCholBlockMinN = 192;

// FP64 passes of molecules with more AOs than this tridiagonalise on an
// 8-SM cluster (the FP64 pipe of one SM needs ~N^3 / 2 clocks)
constexpr int kClusterMinN = 128;
// Cluster passes of molecules with more AOs than this use the blocked
// (panel) cluster tridiagonalisation; smaller ones the column-by-column one.
constexpr int kClusterBlockedMinN = 400;
// In the tail of a batch (fewer molecules than SMs), FP32 passes of
// molecules with more AOs than this tridiagonalise on an 8-SM cluster with
// the matrix in the cluster's shared memory instead of on one SM (120
// measured best with the one-exchange cluster step: 2.62 s per
// 512-molecule call against 2.73 s at 160).
constexpr int kTailClusterMinN = 120;

// Passes that tridiagonalise on an 8-SM cluster in every pass (not only in
// the tail of a batch): FP64 passes above kClusterMinN AOs and FP32 passes
// too large for the shared-memory kernel.
__host__ __device__ __forceinline__ bool cluster_pass(int prec, int nao) {
  return prec ? nao > kClusterMinN : nao > kSmemTridiagMaxN;
}

// FP64 passes of the on-chip cluster tridiagonalisation in double-float
// arithmetic (gbxtb_options.fp64_split)
inline bool split64(const gbxtb_options &o) {
  return o.fp64_split == 2 || (o.fp64_split == 0 && o.mixed_precision != 0);
}

// molecule phases of the SCF state machine
constexpr int kPhaseIterate = 0;  // mixing iterations
constexpr int kPhaseFinal = 1;    // one more V -> Q pass with the unmixed potential
constexpr int kPhaseDone = 2;     // finished (batch), or free slot (pool)
constexpr int kPhaseSetup = 3;    // pool: admitted, geometry terms pending
constexpr int kPhaseFinished = 4; // pool: converged in this step, forces pending

struct MolDesc {
  int32_t atom0, natom;
  int32_t sh0, nsh;
  int32_t ao0, nao;
  int64_t mat0;   // offset of this molecule's nao*nao blocks
  int64_t gam0;   // offset of its nsh*nsh block
  int64_t pair0;  // first unordered shell pair (i <= j) of this molecule
  double nel[2];  // alpha / beta electrons
};

// Parameter tables on the device.
struct DevParams {
  int max_z;
  const int32_t *elem_shell0;
  const int32_t *elem_nshell;
  const double *elem_data;   // [z][GBXTB_ELEM_DOUBLES]
  const int32_t *shell_int;  // [rec][GBXTB_SHELL_INTS]
  const double *shell_data;  // [rec][GBXTB_SHELL_DOUBLES]
  const double *kpair;       // [z][z]
  double g[GBXTB_GLOBALS];
};

// Index maps of a planned batch (device arrays).
struct DevPlan {
  int nmol, natom, nsh, nao;
  int pool;  // 0: a batch solved in one call; 1: a slot pool (continuous batching)
  int64_t nmat, ngam, npair;
  const MolDesc *mol;
  const int32_t *atom_z, *atom_mol, *atom_sh0, *atom_nsh;
  const int32_t *sh_atom, *sh_rec, *sh_ao, *sh_l, *sh_mol;  // sh_ao: AO offset inside the molecule
  const int32_t *ao_sh;                                       // global shell of each AO
  const double *ao_n0;                                        // reference occupation per AO
  const int32_t *bin_mols[kSmemBins];  // molecules of each shared-memory size class
  int bin_count[kSmemBins];
  int bin_maxn[kSmemBins];             // largest molecule of each class
  int bin_warps[kSmemBins];            // warps per CTA of each class (autotuned)
  int bisect_threads;                  // threads per CTA of the batch-wide bisection (autotuned)
};

// Device scratch of one singlepoint call.
struct Work {
  // nao*nao blocks
  double *S, *H0, *Linv, *A, *Z, *P;
  double *H0p;    // L^-1 H0 L^-T (orthogonal-basis core Hamiltonian), per geometry
  double *lo;     // per molecule: FP32 copies of the L^-1 buffer and of H0p
                  // (2 n^2 floats inside the n^2-double block)
  double *ldiag;  // diagonal of the Cholesky factor L (per AO)
  double *invit;  // 5 * nmat: inverse-iteration LU factors
  // per AO
  double *eig, *d, *e, *tau, *occ, *q;  // occ: [2][nao_total]
  // per shell
  double *qsh, *vin, *vout, *vmix, *fprev, *xprev;  // potentials are shell resolved
  double *hist_df, *hist_u;                          // [mem][nsh_total]
  double *gam;                                       // nsh*nsh blocks
  double *dedh;                                      // dE/dh per shell (forces)
  // per atom
  double *cn, *erep, *qat, *grad, *dedcn;  // grad: [natom][3]
  // per molecule
  int32_t *status, *phase, *iter, *kvec, *nhist;
  int32_t *mixstep; // mixer calls made (the reference mixer's iter_step)
  int32_t *dampsw;  // 1: damp_dynamic has switched the mixing parameter
  int32_t *mixsel;  // 1: restarted with the reference's Anderson mixer (restart_at)
  int32_t *prec;    // 0: the next pass runs in FP32, 1: in FP64
  int32_t *npass32; // number of FP32 passes the molecule made
  int32_t *stall32; // FP32 passes since the potential change last halved
  double *best32;   // smallest potential change of the FP32 passes
  double *efermi;   // [2][nmol]
  double *energy;   // [nmol][6]: total, rep, h0, es2, es3, fermi
  double *resid;    // [nmol][2]: L2, max norm of the last potential change
  int32_t *active;  // [2]: molecules not yet done; of those, FP64 passes with more than kClusterMinN AOs
  int32_t *active_list;  // [nmol]: indices of the molecules not yet done
  int32_t *cluster_list;  // [nmol]: molecules whose next pass tridiagonalises on a cluster (cluster_pass)
};

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int warp_sum_int(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; `red` must hold at least blockDim.x/32 doubles.  All threads
// get the result.
__device__ __forceinline__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

// Block-wide FP32 sum (same contract as the FP64 one).
__device__ __forceinline__ float block_sum(float v, float *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  float t = (threadIdx.x < nw) ? red[threadIdx.x] : 0.0f;
  if (wid == 0) t = warp_sum(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  float r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_max(double v, double *red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_max(v);
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double t = (threadIdx.x < nw) ? red[threadIdx.x] : -1.0e308;
  if (wid == 0) t = warp_max(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  double r = red[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_min(double v, double *red) {
  return -block_max(-v, red);
}

__device__ __forceinline__ bool mol_running(const Work &w, int m) {
  return w.phase[m] != kPhaseDone;
}

// Molecule of entry `idx` of a device-side molecule list, or -1 past the
// list's current length (launches over the lists of iterating molecules may
// be sized by an upper bound of that length).
__device__ __forceinline__ int list_mol(const Work &w, const int32_t *list, int idx) {
  if (list == w.active_list && idx >= w.active[0]) return -1;
  if (list == w.cluster_list && idx >= w.active[1]) return -1;
  return list[idx];
}

// Geometry kernels work on every molecule of a batch that has not failed
// (non-finite positions, overlap not positive definite), and in a pool only
// on the molecules admitted since the last step.
__device__ __forceinline__ bool geom_due(const DevPlan &pl, const Work &w, int m) {
  return pl.pool ? w.phase[m] == kPhaseSetup : w.phase[m] != kPhaseDone;
}

// Status bits of a molecule whose result is not a number: Fermi level not
// found, overlap not positive definite, non-finite input or values.
constexpr int kFailBits = GBXTB_MOL_FERMI_FAIL | GBXTB_MOL_CHOLESKY_FAIL | GBXTB_MOL_NONFINITE;

// Force kernels work on every molecule of a batch that has not failed, and
// in a pool only on the molecules that converged in this step.
__device__ __forceinline__ bool force_due(const DevPlan &pl, const Work &w, int m) {
  return pl.pool ? w.phase[m] == kPhaseFinished : (w.status[m] & kFailBits) == 0;
}

// Parameters of one call: the context's tables with the call's switches in
// the spare global slot (g[15] = 1: no halogen-bond term).
inline DevParams call_params(const DevParams &p, const gbxtb_options &o) {
  DevParams c = p;
  c.g[15] = o.no_halogen ? 1.0 : 0.0;
  return c;
}

// ---------------------------------------------------------------------------
// host-side launch helpers (defined in the .cu files)
// ---------------------------------------------------------------------------
void launch_atoms(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                  bool forces, cudaStream_t s);
void launch_shellpairs(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                       cudaStream_t s);
// both return the number of kernel launches they made
int launch_cholesky(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
int launch_cholesky_blocked(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
void launch_fock(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_eigensolve_tridiag(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_fermi(const DevPlan &pl, const Work &w, double kt, int maxiter, double thresh, cudaStream_t s);
void launch_eigenvectors(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_density(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_charges_mix(const DevParams &p, const DevPlan &pl, const Work &w,
                        const gbxtb_options &o, cudaStream_t s);
void launch_energies(const DevParams &p, const DevPlan &pl, const Work &w, double kt,
                     double *energy_out, double *charges_out, cudaStream_t s);
void launch_forces(const DevParams &p, const DevPlan &pl, const Work &w, const double *pos,
                   double *grad_out, cudaStream_t s);

// C-ABI helpers shared by the entry-point translation units (capi.cu):
// record the message of a failure for gbxtb_last_error and return `code`;
// the device scratch a plan's gbxtb_singlepoint needs.
int set_error(int code, const std::string &msg);
size_t plan_workspace_bytes(const gbxtb_plan *plan);
// CUDA device the plan's buffers live on.
int plan_device(const gbxtb_plan *plan);
// GBXTB_OK, or GBXTB_ERR_ARG with a message when an SCF option is out of range.
int check_options(const gbxtb_options *opts);

}  // namespace gbxtb
