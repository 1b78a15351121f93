// Host-side internals of the engine shared by the C-ABI translation units:
// the parameter context and plan objects, the workspace layout, error
// reporting and the kernel launchers.
#pragma once

#include "internal.cuh"

#include <string>
#include <vector>

namespace gbxtb {
void launch_gemm(const DevPlan &pl, const Work &w, const int64_t *tile0, int64_t ntile, int mode,
                 int all, cudaStream_t s);
void launch_tridiag(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
void launch_lowp_copies(const DevPlan &pl, const Work &w, cudaStream_t s);
// tail: the launch shapes of the tail of a batch (FP32 passes above
// kTailClusterMinN AOs move from k_tridiag_smem to the cluster kernel)
void launch_tridiag_smem(const DevPlan &pl, const Work &w, cudaStream_t s, bool tail = false);
// df64_passes: FP64 passes of the on-chip kernel in double-float arithmetic
// (df64.cuh) on the FP32 pipe
int launch_tridiag_cluster(const DevPlan &pl, const Work &w, const int32_t *mol_list, int count, int maxn,
                           cudaStream_t s, bool tail = false, bool df64_passes = false);
void launch_bisect(const DevPlan &pl, const Work &w, int maxn, double kt, const int32_t *mol_list, int count,
                   int threads, cudaStream_t s);
void launch_invit(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
void launch_backtransform(const DevPlan &pl, const Work &w, int maxn, const int32_t *mol_list, int count,
                          cudaStream_t s);
cudaError_t set_linalg_smem_limits(int maxn);
void launch_count_active(const DevPlan &pl, const Work &w, cudaStream_t s);
}  // namespace gbxtb

namespace gbxtb {
// record the message of a failure for gbxtb_last_error and return `code`
int fail(int code, const std::string &msg);
int cuda_fail(cudaError_t e, const char *what);
}  // namespace gbxtb

#define CK(call)                                  \
  do {                                            \
    cudaError_t e__ = (call);                     \
    if (e__ != cudaSuccess) return gbxtb::cuda_fail(e__, #call); \
  } while (0)

namespace gbxtb {
// Index maps of one molecule with molecule-local atom/shell/AO indices
// (basis/indexhelper.py:283-491) and its alpha/beta electron counts
// (scf/iterator.py:147-189, wavefunction/filling.py:41-113).
struct MolMaps {
  int natom = 0, nsh = 0, nao = 0;
  double nel[2] = {0.0, 0.0};
  std::vector<int32_t> atom_z, atom_sh0, atom_nsh;
  std::vector<int32_t> sh_atom, sh_rec, sh_ao, sh_l;
  std::vector<int32_t> ao_sh;
  std::vector<double> ao_n0;
};
// uhf < 0: unpaired electrons from the parity of the electron count.
int describe_molecule(const gbxtb_ctx *ctx, const int32_t *numbers, int natoms, double charge, int uhf,
                      MolMaps &out);
}  // namespace gbxtb

namespace gbxtb {
inline size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr int kHistMax = 29;  // longest mixer history (Broyden pairs; Anderson generations + 1)
}  // namespace gbxtb

struct gbxtb_ctx {
  int device = 0;
  gbxtb::DevParams p{};
  void *dbuf = nullptr;
  std::vector<int32_t> elem_shell0, elem_nshell, shell_int;
  std::vector<double> shell_data, elem_data;
};

struct gbxtb_plan {
  gbxtb_ctx *ctx = nullptr;
  gbxtb::DevPlan pl{};
  int64_t *tile0 = nullptr;
  int64_t ntile = 0;
  int maxn = 0;
  void *dbuf = nullptr;
  size_t ws_bytes = 0;
  std::vector<gbxtb::MolDesc> mol;
  // state of the last singlepoint
  cudaStream_t last_stream = nullptr;
  gbxtb::Work last_work{};
  void *last_ws = nullptr;  // workspace of the last singlepoint (its final SCF state)
  gbxtb_options last_opts{};  // options of the last singlepoint
  bool has_run = false;
  int32_t *h_active = nullptr;  // pinned
  int num_sms = 0;
  int smem_launches = 0;  // size classes with molecules (k_tridiag_smem launches per pass)
  int nbig = 0;           // molecules with more than kClusterMinN AOs (cluster passes at most)
  // CUDA graphs of one SCF pass ([0]: launch shapes over all molecules, [1]:
  // the tail shapes), with the workspace and options they were captured for
  cudaGraphExec_t pass_graph[2] = {nullptr, nullptr};
  int pass_graph_launches[2] = {0, 0};
  void *graph_ws = nullptr;
  gbxtb_options graph_opts{};
  cudaStream_t capture_stream = nullptr;  // non-blocking, for capturing the pass graphs
  // profiling
  cudaEvent_t ev[GBXTB_PROF_CLASSES][2] = {};
  bool ev_ready = false;
  double prof_ms[GBXTB_PROF_CLASSES] = {};
  int64_t prof_launches[GBXTB_PROF_CLASSES] = {};
  int64_t total_launches = 0;
};

namespace gbxtb {

// Workspace layout of a plan.
struct Layout {
  size_t off[64];
  int n = 0;
  size_t total = 0;
  size_t add(size_t bytes) {
    off[n] = total;
    total += align256(bytes);
    return off[n++];
  }
};

inline Layout make_layout(const DevPlan &pl) {
  Layout L;
  const size_t d = sizeof(double), i4 = sizeof(int32_t);
  for (int k = 0; k < 8; ++k) L.add(d * pl.nmat);          // S H0 Linv A Z P H0p lo
  L.add(d * 5 * pl.nmat);                                   // invit
  for (int k = 0; k < 6; ++k) L.add(d * pl.nao);            // eig d e tau q ldiag
  L.add(d * 2 * pl.nao);                                    // occ
  for (int k = 0; k < 7; ++k) L.add(d * pl.nsh);            // qsh vin vout vmix fprev xprev dedh
  L.add(d * kHistMax * pl.nsh);                             // hist_df
  L.add(d * kHistMax * pl.nsh);                             // hist_u
  L.add(d * pl.ngam);                                       // gam
  for (int k = 0; k < 4; ++k) L.add(d * pl.natom);          // cn erep qat dedcn
  L.add(d * 3 * pl.natom);                                  // grad
  for (int k = 0; k < 11; ++k) L.add(i4 * pl.nmol);  // status phase iter kvec nhist prec npass32 stall32 mixstep dampsw mixsel
  L.add(d * 2 * pl.nmol);                                   // efermi
  L.add(d * 6 * pl.nmol);                                   // energy
  L.add(d * 2 * pl.nmol);                                   // resid
  L.add(d * pl.nmol);                                       // best32
  L.add(i4 * 4);                                            // active
  L.add(i4 * pl.nmol);                                      // active_list
  L.add(i4 * pl.nmol);                                      // cluster_list
  return L;
}

inline Work make_work(const DevPlan &pl, void *base) {
  Layout L = make_layout(pl);
  char *b = static_cast<char *>(base);
  int k = 0;
  auto D = [&]() { return reinterpret_cast<double *>(b + L.off[k++]); };
  auto I = [&]() { return reinterpret_cast<int32_t *>(b + L.off[k++]); };
  Work w{};
  w.S = D(); w.H0 = D(); w.Linv = D(); w.A = D(); w.Z = D(); w.P = D(); w.H0p = D(); w.lo = D();
  w.invit = D();
  w.eig = D(); w.d = D(); w.e = D(); w.tau = D(); w.q = D(); w.ldiag = D();
  w.occ = D();
  w.qsh = D(); w.vin = D(); w.vout = D(); w.vmix = D(); w.fprev = D(); w.xprev = D(); w.dedh = D();
  w.hist_df = D(); w.hist_u = D();
  w.gam = D();
  w.cn = D(); w.erep = D(); w.qat = D(); w.dedcn = D();
  w.grad = D();
  w.status = I(); w.phase = I(); w.iter = I(); w.kvec = I(); w.nhist = I(); w.prec = I();
  w.npass32 = I();
  w.stall32 = I();
  w.mixstep = I();
  w.dampsw = I();
  w.mixsel = I();
  w.efermi = D(); w.energy = D(); w.resid = D(); w.best32 = D();
  w.active = I();
  w.active_list = I();
  w.cluster_list = I();
  return w;
}

}  // namespace gbxtb
