// C ABI of libgbxtb.so: parameter context, batch planning (atom/shell/AO
// maps built on the host, uploaded once), workspace layout and the SCF
// driver loop that launches the device kernels on the caller's stream.
//
// Reference behaviour reproduced (dxtb, src/dxtb/_src/...):
//   planning      basis/indexhelper.py:283-491 (index maps),
//                 scf/iterator.py:147-189 (n0 = refocc / (2l+1), nel = sum n0 - charge),
//                 wavefunction/filling.py:41-113 (alpha/beta split by parity or uhf)
//   SCF driver    scf/unrolling/default.py:71-136 (iterate potential,
//                 mix, stop on convergence or maxiter, final charges from the
//                 last unmixed potential), calculators/types/energy.py:78-402
#include "internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

namespace gbxtb {
void launch_gemm(const DevPlan &pl, const Work &w, const int64_t *tile0, int64_t ntile, int mode,
                 int all, cudaStream_t s);
void launch_tridiag(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
void launch_lowp_copies(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_tridiag_smem(const DevPlan &pl, const Work &w, cudaStream_t s);
void launch_tridiag_cluster(const DevPlan &pl, const Work &w, const int32_t *mol_list, int count,
                            int maxn, cudaStream_t s);
void launch_bisect(const DevPlan &pl, const Work &w, int maxn, double kt, const int32_t *mol_list, int count,
                   int threads, cudaStream_t s);
void launch_invit(const DevPlan &pl, const Work &w, int maxn, cudaStream_t s);
void launch_backtransform(const DevPlan &pl, const Work &w, int maxn, const int32_t *mol_list, int count,
                          cudaStream_t s);
cudaError_t set_linalg_smem_limits(int maxn);
void launch_count_active(const DevPlan &pl, const Work &w, cudaStream_t s);
}  // namespace gbxtb

using namespace gbxtb;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return GBXTB_ERR_CUDA;
}

#define CK(call)                                  \
  do {                                            \
    cudaError_t e__ = (call);                     \
    if (e__ != cudaSuccess) return cuda_fail(e__, #call); \
  } while (0)

size_t align256(size_t x) { return (x + 255) / 256 * 256; }

constexpr int kHistMax = 29;

}  // namespace

struct gbxtb_ctx {
  int device = 0;
  DevParams p{};
  void *dbuf = nullptr;
  std::vector<int32_t> elem_shell0, elem_nshell, shell_int;
  std::vector<double> shell_data, elem_data;
};

struct gbxtb_plan {
  gbxtb_ctx *ctx = nullptr;
  DevPlan pl{};
  int64_t *tile0 = nullptr;
  int64_t ntile = 0;
  int maxn = 0;
  void *dbuf = nullptr;
  size_t ws_bytes = 0;
  std::vector<MolDesc> mol;
  // state of the last singlepoint
  cudaStream_t last_stream = nullptr;
  Work last_work{};
  bool has_run = false;
  int32_t *h_active = nullptr;  // pinned
  int num_sms = 0;
  int smem_launches = 0;  // size classes with molecules (k_tridiag_smem launches per pass)
  // profiling
  cudaEvent_t ev[GBXTB_PROF_CLASSES][2] = {};
  bool ev_ready = false;
  double prof_ms[GBXTB_PROF_CLASSES] = {};
  int64_t prof_launches[GBXTB_PROF_CLASSES] = {};
  int64_t total_launches = 0;
};

namespace {

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

Layout make_layout(const DevPlan &pl) {
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
  for (int k = 0; k < 8; ++k) L.add(i4 * pl.nmol);          // status phase iter kvec nhist prec npass32 stall32
  L.add(d * 2 * pl.nmol);                                   // efermi
  L.add(d * 6 * pl.nmol);                                   // energy
  L.add(d * 2 * pl.nmol);                                   // resid
  L.add(d * pl.nmol);                                       // best32
  L.add(i4 * 4);                                            // active
  L.add(i4 * pl.nmol);                                      // active_list
  return L;
}

Work make_work(const DevPlan &pl, void *base) {
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
  w.efermi = D(); w.energy = D(); w.resid = D(); w.best32 = D();
  w.active = I();
  w.active_list = I();
  return w;
}

}  // namespace

namespace gbxtb {
int set_error(int code, const std::string &msg) { return fail(code, msg); }
size_t plan_workspace_bytes(const gbxtb_plan *plan) { return plan ? plan->ws_bytes : 0; }
}  // namespace gbxtb

extern "C" {

int gbxtb_version(void) { return GBXTB_VERSION; }

const char *gbxtb_last_error(void) { return g_err.c_str(); }

int gbxtb_ctx_create(const gbxtb_params *params, gbxtb_ctx **out) {
  if (!params || !out) return fail(GBXTB_ERR_ARG, "null argument");
  if (params->max_z < 1 || params->n_shell_records < 1 || !params->elem_shell0 ||
      !params->elem_nshell || !params->elem_data || !params->shell_int || !params->shell_data ||
      !params->kpair || !params->globals)
    return fail(GBXTB_ERR_ARG, "incomplete parameter tables");
  if (params->globals[11] != 2.0) return fail(GBXTB_ERR_ARG, "only gexp = 2 is supported");
  const int nz = params->max_z + 1, ns = params->n_shell_records;
  for (int r = 0; r < ns; ++r) {
    const int l = params->shell_int[r * GBXTB_SHELL_INTS], np = params->shell_int[r * GBXTB_SHELL_INTS + 1];
    if (l < 0 || l > kMaxL) return fail(GBXTB_ERR_ARG, "angular momentum > 2 not supported");
    if (np < 1 || np > kMaxPrim) return fail(GBXTB_ERR_ARG, "bad primitive count");
  }
  auto *c = new (std::nothrow) gbxtb_ctx();
  if (!c) return fail(GBXTB_ERR_NOMEM, "host allocation failed");
  cudaGetDevice(&c->device);
  c->elem_shell0.assign(params->elem_shell0, params->elem_shell0 + nz);
  c->elem_nshell.assign(params->elem_nshell, params->elem_nshell + nz);
  c->shell_int.assign(params->shell_int, params->shell_int + (size_t)ns * GBXTB_SHELL_INTS);
  c->shell_data.assign(params->shell_data, params->shell_data + (size_t)ns * GBXTB_SHELL_DOUBLES);
  c->elem_data.assign(params->elem_data, params->elem_data + (size_t)nz * GBXTB_ELEM_DOUBLES);
  size_t b_es0 = align256(sizeof(int32_t) * nz), b_ens = align256(sizeof(int32_t) * nz);
  size_t b_ed = align256(sizeof(double) * nz * GBXTB_ELEM_DOUBLES);
  size_t b_si = align256(sizeof(int32_t) * ns * GBXTB_SHELL_INTS);
  size_t b_sd = align256(sizeof(double) * ns * GBXTB_SHELL_DOUBLES);
  size_t b_kp = align256(sizeof(double) * nz * nz);
  size_t total = b_es0 + b_ens + b_ed + b_si + b_sd + b_kp;
  cudaError_t e = cudaMalloc(&c->dbuf, total);
  if (e != cudaSuccess) {
    delete c;
    return cuda_fail(e, "cudaMalloc(params)");
  }
  char *b = static_cast<char *>(c->dbuf);
  size_t o = 0;
  auto up = [&](const void *src, size_t bytes, size_t span) -> void * {
    void *dst = b + o;
    cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice);
    o += span;
    return dst;
  };
  c->p.max_z = params->max_z;
  c->p.elem_shell0 = (const int32_t *)up(params->elem_shell0, sizeof(int32_t) * nz, b_es0);
  c->p.elem_nshell = (const int32_t *)up(params->elem_nshell, sizeof(int32_t) * nz, b_ens);
  c->p.elem_data = (const double *)up(params->elem_data, sizeof(double) * nz * GBXTB_ELEM_DOUBLES, b_ed);
  c->p.shell_int = (const int32_t *)up(params->shell_int, sizeof(int32_t) * ns * GBXTB_SHELL_INTS, b_si);
  c->p.shell_data = (const double *)up(params->shell_data, sizeof(double) * ns * GBXTB_SHELL_DOUBLES, b_sd);
  c->p.kpair = (const double *)up(params->kpair, sizeof(double) * nz * nz, b_kp);
  for (int k = 0; k < GBXTB_GLOBALS; ++k) c->p.g[k] = params->globals[k];
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    cudaFree(c->dbuf);
    delete c;
    return cuda_fail(e, "upload parameters");
  }
  *out = c;
  return GBXTB_OK;
}

void gbxtb_ctx_destroy(gbxtb_ctx *ctx) {
  if (!ctx) return;
  if (ctx->dbuf) cudaFree(ctx->dbuf);
  delete ctx;
}

int gbxtb_plan_create(gbxtb_ctx *ctx, int32_t nmol, const int32_t *numbers,
                      const int64_t *atom_offsets, const double *charge, const int32_t *uhf,
                      gbxtb_plan **out, size_t *workspace_bytes) {
  if (!ctx || !numbers || !atom_offsets || !out || !workspace_bytes || nmol < 1)
    return fail(GBXTB_ERR_ARG, "null argument or empty batch");
  std::vector<MolDesc> mol(nmol);
  std::vector<int32_t> atom_z, atom_mol, atom_sh0, atom_nsh;
  std::vector<int32_t> sh_atom, sh_rec, sh_ao, sh_l, sh_mol, ao_sh;
  std::vector<double> ao_n0;
  std::vector<int64_t> tile0(nmol + 1);
  int64_t nmat = 0, ngam = 0, npair = 0, ntile = 0;
  int maxn = 0;
  if (atom_offsets[0] != 0) return fail(GBXTB_ERR_ARG, "atom_offsets[0] must be 0");
  for (int m = 0; m < nmol; ++m) {
    const int64_t a0 = atom_offsets[m], a1 = atom_offsets[m + 1];
    if (a1 <= a0) return fail(GBXTB_ERR_ARG, "molecule without atoms");
    MolDesc &md = mol[m];
    md.atom0 = (int32_t)atom_z.size();
    md.natom = (int32_t)(a1 - a0);
    md.sh0 = (int32_t)sh_atom.size();
    md.ao0 = (int32_t)ao_sh.size();
    int nao = 0;
    double n0sum = 0.0;
    for (int64_t a = a0; a < a1; ++a) {
      const int z = numbers[a];
      if (z < 1 || z > ctx->p.max_z || ctx->elem_nshell[z] < 1)
        return fail(GBXTB_ERR_ELEMENT, "atomic number " + std::to_string(z) + " has no GFN1 parameters");
      const int ga = (int32_t)atom_z.size();
      atom_z.push_back(z);
      atom_mol.push_back(m);
      atom_sh0.push_back((int32_t)sh_atom.size());
      atom_nsh.push_back(ctx->elem_nshell[z]);
      for (int s = 0; s < ctx->elem_nshell[z]; ++s) {
        const int rec = ctx->elem_shell0[z] + s;
        const int l = ctx->shell_int[(size_t)rec * GBXTB_SHELL_INTS];
        const double refocc = ctx->shell_data[(size_t)rec * GBXTB_SHELL_DOUBLES + 19];
        const int gs = (int32_t)sh_atom.size();
        sh_atom.push_back(ga);
        sh_rec.push_back(rec);
        sh_ao.push_back(nao);
        sh_l.push_back(l);
        sh_mol.push_back(m);
        for (int k = 0; k < 2 * l + 1; ++k) {
          ao_sh.push_back(gs);
          ao_n0.push_back(refocc / (2 * l + 1));
          n0sum += refocc / (2 * l + 1);
        }
        nao += 2 * l + 1;
      }
    }
    md.nsh = (int32_t)sh_atom.size() - md.sh0;
    md.nao = nao;
    md.mat0 = nmat;
    md.gam0 = ngam;
    md.pair0 = npair;
    nmat += (int64_t)nao * nao;
    ngam += (int64_t)md.nsh * md.nsh;
    npair += (int64_t)md.nsh * (md.nsh + 1) / 2;
    tile0[m] = ntile;
    const int64_t nt = (nao + 63) / 64;
    ntile += nt * nt;
    maxn = std::max(maxn, nao);
    // electrons (scf/iterator.py:183-187, filling.py:41-113)
    const double chg = charge ? charge[m] : 0.0;
    const double nel = std::nearbyint(n0sum - chg);
    if (nel < 0.0) return fail(GBXTB_ERR_ARG, "negative number of electrons");
    const int nel_i = (int)nel;
    int u;
    if (uhf && uhf[m] >= 0) {
      u = uhf[m];
      if (u > nel_i) return fail(GBXTB_ERR_ARG, "more unpaired electrons than electrons");
      if ((u % 2) != (nel_i % 2))
        return fail(GBXTB_ERR_ARG, "parity of unpaired electrons and electrons differs");
    } else {
      u = nel_i % 2;
    }
    const double nb = (nel - u) / 2.0;
    md.nel[0] = nb + u;
    md.nel[1] = nb;
  }
  tile0[nmol] = ntile;
  // shared-memory size classes of the FP32 tridiagonalisation
  std::vector<int32_t> bins[kSmemBins];
  int bin_maxn[kSmemBins] = {};
  for (int m = 0; m < nmol; ++m)
    for (int c = 0; c < kSmemBins; ++c)
      if (mol[m].nao <= kSmemBinN[c]) {
        bins[c].push_back(m);
        bin_maxn[c] = std::max(bin_maxn[c], mol[m].nao);
        break;
      }
  auto *pl = new (std::nothrow) gbxtb_plan();
  if (!pl) return fail(GBXTB_ERR_NOMEM, "host allocation failed");
  pl->ctx = ctx;
  pl->mol = mol;
  pl->maxn = maxn;
  pl->ntile = ntile;
  DevPlan &d = pl->pl;
  d.nmol = nmol;
  d.natom = (int)atom_z.size();
  d.nsh = (int)sh_atom.size();
  d.nao = (int)ao_sh.size();
  d.nmat = nmat;
  d.ngam = ngam;
  d.npair = npair;
  // one device block for all index arrays
  Layout L;
  const size_t o_mol = L.add(sizeof(MolDesc) * nmol);
  const size_t o_tile = L.add(sizeof(int64_t) * (nmol + 1));
  const size_t o_az = L.add(4 * atom_z.size()), o_am = L.add(4 * atom_z.size());
  const size_t o_as0 = L.add(4 * atom_z.size()), o_ans = L.add(4 * atom_z.size());
  const size_t o_sa = L.add(4 * sh_atom.size()), o_sr = L.add(4 * sh_atom.size());
  const size_t o_so = L.add(4 * sh_atom.size()), o_sl = L.add(4 * sh_atom.size());
  const size_t o_sm = L.add(4 * sh_atom.size());
  const size_t o_aos = L.add(4 * ao_sh.size());
  const size_t o_n0 = L.add(8 * ao_n0.size());
  size_t o_bin[kSmemBins];
  for (int c = 0; c < kSmemBins; ++c) o_bin[c] = L.add(4 * std::max<size_t>(1, bins[c].size()));
  cudaError_t e = cudaMalloc(&pl->dbuf, L.total);
  if (e != cudaSuccess) {
    delete pl;
    return cuda_fail(e, "cudaMalloc(plan)");
  }
  char *b = static_cast<char *>(pl->dbuf);
  auto up = [&](size_t off, const void *src, size_t bytes) {
    return cudaMemcpy(b + off, src, bytes, cudaMemcpyHostToDevice);
  };
  up(o_mol, mol.data(), sizeof(MolDesc) * nmol);
  up(o_tile, tile0.data(), sizeof(int64_t) * (nmol + 1));
  up(o_az, atom_z.data(), 4 * atom_z.size());
  up(o_am, atom_mol.data(), 4 * atom_z.size());
  up(o_as0, atom_sh0.data(), 4 * atom_z.size());
  up(o_ans, atom_nsh.data(), 4 * atom_z.size());
  up(o_sa, sh_atom.data(), 4 * sh_atom.size());
  up(o_sr, sh_rec.data(), 4 * sh_atom.size());
  up(o_so, sh_ao.data(), 4 * sh_atom.size());
  up(o_sl, sh_l.data(), 4 * sh_atom.size());
  up(o_sm, sh_mol.data(), 4 * sh_atom.size());
  up(o_aos, ao_sh.data(), 4 * ao_sh.size());
  for (int c = 0; c < kSmemBins; ++c)
    if (!bins[c].empty()) up(o_bin[c], bins[c].data(), 4 * bins[c].size());
  e = up(o_n0, ao_n0.data(), 8 * ao_n0.size());
  if (e != cudaSuccess) {
    cudaFree(pl->dbuf);
    delete pl;
    return cuda_fail(e, "upload plan");
  }
  d.mol = (const MolDesc *)(b + o_mol);
  pl->tile0 = (int64_t *)(b + o_tile);
  d.atom_z = (const int32_t *)(b + o_az);
  d.atom_mol = (const int32_t *)(b + o_am);
  d.atom_sh0 = (const int32_t *)(b + o_as0);
  d.atom_nsh = (const int32_t *)(b + o_ans);
  d.sh_atom = (const int32_t *)(b + o_sa);
  d.sh_rec = (const int32_t *)(b + o_sr);
  d.sh_ao = (const int32_t *)(b + o_so);
  d.sh_l = (const int32_t *)(b + o_sl);
  d.sh_mol = (const int32_t *)(b + o_sm);
  d.ao_sh = (const int32_t *)(b + o_aos);
  d.ao_n0 = (const double *)(b + o_n0);
  for (int c = 0; c < kSmemBins; ++c) {
    d.bin_mols[c] = (const int32_t *)(b + o_bin[c]);
    d.bin_count[c] = (int)bins[c].size();
    d.bin_maxn[c] = bin_maxn[c];
  }
  e = set_linalg_smem_limits(maxn);
  if (e != cudaSuccess) {
    cudaFree(pl->dbuf);
    delete pl;
    return cuda_fail(e, "shared memory limit");
  }
  e = cudaMallocHost(&pl->h_active, sizeof(int32_t) * 4);
  if (e != cudaSuccess) {
    cudaFree(pl->dbuf);
    delete pl;
    return cuda_fail(e, "cudaMallocHost");
  }
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&pl->num_sms, cudaDevAttrMultiProcessorCount, dev);
  }
  for (int c = 0; c < kSmemBins; ++c) pl->smem_launches += bins[c].empty() ? 0 : 1;
  pl->ws_bytes = make_layout(d).total;
  *workspace_bytes = pl->ws_bytes;
  *out = pl;
  return GBXTB_OK;
}

void gbxtb_plan_destroy(gbxtb_plan *plan) {
  if (!plan) return;
  if (plan->ev_ready)
    for (int c = 0; c < GBXTB_PROF_CLASSES; ++c)
      for (int k = 0; k < 2; ++k) cudaEventDestroy(plan->ev[c][k]);
  if (plan->dbuf) cudaFree(plan->dbuf);
  if (plan->h_active) cudaFreeHost(plan->h_active);
  delete plan;
}

int gbxtb_plan_sizes(const gbxtb_plan *plan, int64_t *s) {
  if (!plan || !s) return fail(GBXTB_ERR_ARG, "null argument");
  s[0] = plan->pl.nmol;
  s[1] = plan->pl.natom;
  s[2] = plan->pl.nsh;
  s[3] = plan->pl.nao;
  s[4] = plan->pl.nmat;
  s[5] = plan->pl.ngam;
  return GBXTB_OK;
}

static int prepare(gbxtb_plan *plan, const double *pos, void *ws, size_t ws_bytes, Work &w) {
  if (!plan || !pos || !ws) return fail(GBXTB_ERR_ARG, "null argument");
  if (ws_bytes < plan->ws_bytes) return fail(GBXTB_ERR_WORKSPACE, "workspace too small");
  if (reinterpret_cast<uintptr_t>(ws) % 256 != 0) return fail(GBXTB_ERR_ARG, "workspace must be 256-byte aligned");
  w = make_work(plan->pl, ws);
  return GBXTB_OK;
}

int gbxtb_integrals(gbxtb_plan *plan, const double *positions_dev, double *overlap_dev,
                    double *hcore_dev, void *workspace_dev, size_t workspace_bytes, void *stream) {
  Work w;
  int rc = prepare(plan, positions_dev, workspace_dev, workspace_bytes, w);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const DevPlan &pl = plan->pl;
  const DevParams &p = plan->ctx->p;
  launch_atoms(p, pl, w, positions_dev, false, s);
  launch_shellpairs(p, pl, w, positions_dev, s);
  CK(cudaGetLastError());
  if (overlap_dev) CK(cudaMemcpyAsync(overlap_dev, w.S, sizeof(double) * pl.nmat, cudaMemcpyDeviceToDevice, s));
  if (hcore_dev) CK(cudaMemcpyAsync(hcore_dev, w.H0, sizeof(double) * pl.nmat, cudaMemcpyDeviceToDevice, s));
  return GBXTB_OK;
}

namespace {
// Stream-ordered timing of kernel classes: begin/end record events; the
// elapsed times are harvested after each host synchronisation.
struct Prof {
  gbxtb_plan *pl;
  cudaStream_t s;
  bool on;
  bool pending[GBXTB_PROF_CLASSES] = {};
  void begin(int c) {
    if (on) cudaEventRecord(pl->ev[c][0], s);
  }
  void end(int c, int launches) {
    pl->total_launches += launches;
    pl->prof_launches[c] += launches;
    if (on) {
      cudaEventRecord(pl->ev[c][1], s);
      pending[c] = true;
    }
  }
  // after a stream synchronisation
  void harvest() {
    if (!on) return;
    for (int c = 0; c < GBXTB_PROF_CLASSES; ++c)
      if (pending[c]) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, pl->ev[c][0], pl->ev[c][1]) == cudaSuccess) pl->prof_ms[c] += ms;
        pending[c] = false;
      }
  }
};
}  // namespace

int gbxtb_singlepoint(gbxtb_plan *plan, const gbxtb_options *opts, const double *positions_dev,
                      double *energy_dev, double *charges_dev, double *gradient_dev,
                      void *workspace_dev, size_t workspace_bytes, void *stream) {
  if (!opts || !energy_dev) return fail(GBXTB_ERR_ARG, "null argument");
  if (opts->want_forces && !gradient_dev) return fail(GBXTB_ERR_ARG, "forces requested without gradient buffer");
  if (opts->maxiter < 0 || opts->fermi_maxiter < 1 || !(opts->kt > 0.0) || opts->broyden_memory < 1 ||
      opts->broyden_memory > kHistMax)
    return fail(GBXTB_ERR_ARG, "invalid options");
  Work w;
  int rc = prepare(plan, positions_dev, workspace_dev, workspace_bytes, w);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const DevPlan &pl = plan->pl;
  const DevParams &p = plan->ctx->p;
  if (opts->profile && !plan->ev_ready) {
    for (int c = 0; c < GBXTB_PROF_CLASSES; ++c)
      for (int k = 0; k < 2; ++k) CK(cudaEventCreate(&plan->ev[c][k]));
    plan->ev_ready = true;
  }
  for (int c = 0; c < GBXTB_PROF_CLASSES; ++c) {
    plan->prof_ms[c] = 0.0;
    plan->prof_launches[c] = 0;
  }
  plan->total_launches = 0;
  Prof pf{plan, s, opts->profile != 0};
  // reset state
  CK(cudaMemsetAsync(w.status, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.phase, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.iter, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.kvec, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.nhist, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.npass32, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.stall32, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.best32, 0x7f, sizeof(double) * pl.nmol, s));  // 1.4e306: no pass yet
  // 0: the first passes run in FP32; any non-zero byte pattern means FP64
  CK(cudaMemsetAsync(w.prec, opts->mixed_precision ? 0 : 1, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.vin, 0, sizeof(double) * pl.nsh, s));
  CK(cudaMemsetAsync(w.energy, 0, sizeof(double) * 6 * pl.nmol, s));
  // geometry-dependent terms
  pf.begin(GBXTB_PROF_ATOMS);
  launch_atoms(p, pl, w, positions_dev, opts->want_forces != 0, s);
  pf.end(GBXTB_PROF_ATOMS, 1);
  pf.begin(GBXTB_PROF_SHELLPAIRS);
  launch_shellpairs(p, pl, w, positions_dev, s);
  pf.end(GBXTB_PROF_SHELLPAIRS, 1);
  pf.begin(GBXTB_PROF_CHOLESKY);
  launch_cholesky(pl, w, s);
  // H0' = L^-1 H0 L^-T once per geometry (the potential is still zero)
  launch_gemm(pl, w, plan->tile0, plan->ntile, 0, 0, s);
  launch_gemm(pl, w, plan->tile0, plan->ntile, 5, 0, s);
  if (opts->mixed_precision) launch_lowp_copies(pl, w, s);
  pf.end(GBXTB_PROF_CHOLESKY, opts->mixed_precision ? 4 : 3);
  CK(cudaGetLastError());
  // SCF: maxiter mixing iterations + the first evaluation + the final pass
  const int max_loops = opts->maxiter + 3;
  int active = pl.nmol;  // molecules iterating (known after each pass)
  for (int it = 0; it < max_loops; ++it) {
    pf.begin(GBXTB_PROF_FOCK);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 6, 0, s);
    pf.end(GBXTB_PROF_FOCK, 1);
    pf.begin(GBXTB_PROF_TRIDIAG);
    // fewer molecules than SMs (the tail of the batch): spread each molecule
    // over more SMs (an 8-SM cluster for the tridiagonalisation, more blocks
    // for bisection and back-transformation), working from the device-side
    // list of molecules still iterating
    const bool tail = it > 0 && active <= plan->num_sms;
    if (opts->mixed_precision) launch_tridiag_smem(pl, w, s);
    if (tail)
      launch_tridiag_cluster(pl, w, w.active_list, active, plan->maxn, s);
    else
      launch_tridiag(pl, w, plan->maxn, s);
    pf.end(GBXTB_PROF_TRIDIAG, opts->mixed_precision ? 1 + plan->smem_launches : 1);
    pf.begin(GBXTB_PROF_BISECT);
    if (tail)
      launch_bisect(pl, w, plan->maxn, opts->kt, w.active_list, active, 32, s);
    else
      launch_bisect(pl, w, plan->maxn, opts->kt, nullptr, pl.nmol, 256, s);
    pf.end(GBXTB_PROF_BISECT, 1);
    pf.begin(GBXTB_PROF_FERMI);
    launch_fermi(pl, w, opts->kt, opts->fermi_maxiter, s);
    pf.end(GBXTB_PROF_FERMI, 1);
    pf.begin(GBXTB_PROF_INVIT);
    launch_invit(pl, w, plan->maxn, s);
    pf.end(GBXTB_PROF_INVIT, 1);
    pf.begin(GBXTB_PROF_BACKTRANSFORM);
    if (tail)
      launch_backtransform(pl, w, plan->maxn, w.active_list, active, s);
    else
      launch_backtransform(pl, w, plan->maxn, nullptr, pl.nmol, s);
    pf.end(GBXTB_PROF_BACKTRANSFORM, 1);
    pf.begin(GBXTB_PROF_DENSITY);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 2, 0, s);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 3, 0, s);
    pf.end(GBXTB_PROF_DENSITY, 2);
    pf.begin(GBXTB_PROF_MIX);
    launch_charges_mix(p, pl, w, *opts, it, s);
    launch_count_active(pl, w, s);
    pf.end(GBXTB_PROF_MIX, 2);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(plan->h_active, w.active, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    pf.harvest();
    active = plan->h_active[0];
    if (active == 0) break;
  }
  launch_energies(p, pl, w, opts->kt, energy_dev, charges_dev, s);
  plan->total_launches += 1;
  if (opts->want_forces) {
    pf.begin(GBXTB_PROF_FORCES);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 4, 1, s);
    launch_forces(p, pl, w, positions_dev, gradient_dev, s);
    pf.end(GBXTB_PROF_FORCES, 3);
  }
  CK(cudaGetLastError());
  if (pf.on) {
    CK(cudaStreamSynchronize(s));
    pf.harvest();
  }
  plan->last_stream = s;
  plan->last_work = w;
  plan->has_run = true;
  return GBXTB_OK;
}

int gbxtb_get_status(gbxtb_plan *plan, int32_t *status, int32_t *iterations) {
  if (!plan || !plan->has_run) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  CK(cudaStreamSynchronize(plan->last_stream));
  const int n = plan->pl.nmol;
  if (status) CK(cudaMemcpy(status, plan->last_work.status, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  if (iterations) CK(cudaMemcpy(iterations, plan->last_work.iter, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
  return GBXTB_OK;
}

int gbxtb_get_fp32_passes(gbxtb_plan *plan, int32_t *passes) {
  if (!plan || !plan->has_run || !passes) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  CK(cudaStreamSynchronize(plan->last_stream));
  CK(cudaMemcpy(passes, plan->last_work.npass32, sizeof(int32_t) * plan->pl.nmol, cudaMemcpyDeviceToHost));
  return GBXTB_OK;
}

int gbxtb_get_profile(gbxtb_plan *plan, double *ms, int64_t *launches, int64_t *total_launches) {
  if (!plan || !plan->has_run) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  CK(cudaStreamSynchronize(plan->last_stream));
  for (int c = 0; c < GBXTB_PROF_CLASSES; ++c) {
    if (ms) ms[c] = plan->prof_ms[c];
    if (launches) launches[c] = plan->prof_launches[c];
  }
  if (total_launches) *total_launches = plan->total_launches;
  return GBXTB_OK;
}

int gbxtb_get_shell_potential(gbxtb_plan *plan, double *potential) {
  if (!plan || !plan->has_run || !potential) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  CK(cudaStreamSynchronize(plan->last_stream));
  CK(cudaMemcpy(potential, plan->last_work.vout, sizeof(double) * plan->pl.nsh, cudaMemcpyDeviceToHost));
  return GBXTB_OK;
}

}  // extern "C"
