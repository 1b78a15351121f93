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
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace gbxtb;

namespace {
thread_local std::string g_err;
}  // namespace

namespace gbxtb {
int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return GBXTB_ERR_CUDA;
}
}  // namespace gbxtb

namespace gbxtb {
int describe_molecule(const gbxtb_ctx *ctx, const int32_t *numbers, int natoms, double charge, int uhf,
                      MolMaps &mm) {
  mm = MolMaps();
  double n0sum = 0.0;
  for (int a = 0; a < natoms; ++a) {
    const int z = numbers[a];
    if (z < 1 || z > ctx->p.max_z || ctx->elem_nshell[z] < 1)
      return fail(GBXTB_ERR_ELEMENT, "atomic number " + std::to_string(z) + " has no GFN1 parameters");
    mm.atom_z.push_back(z);
    mm.atom_sh0.push_back(mm.nsh);
    mm.atom_nsh.push_back(ctx->elem_nshell[z]);
    for (int s = 0; s < ctx->elem_nshell[z]; ++s) {
      const int rec = ctx->elem_shell0[z] + s;
      const int l = ctx->shell_int[(size_t)rec * GBXTB_SHELL_INTS];
      const double refocc = ctx->shell_data[(size_t)rec * GBXTB_SHELL_DOUBLES + 19];
      mm.sh_atom.push_back(a);
      mm.sh_rec.push_back(rec);
      mm.sh_ao.push_back(mm.nao);
      mm.sh_l.push_back(l);
      for (int k = 0; k < 2 * l + 1; ++k) {
        mm.ao_sh.push_back(mm.nsh);
        mm.ao_n0.push_back(refocc / (2 * l + 1));
        n0sum += refocc / (2 * l + 1);
      }
      mm.nao += 2 * l + 1;
      mm.nsh += 1;
    }
  }
  mm.natom = natoms;
  // electrons (scf/iterator.py:183-187, filling.py:41-113)
  const double nel = std::nearbyint(n0sum - charge);
  if (nel < 0.0) return fail(GBXTB_ERR_ARG, "negative number of electrons");
  const int nel_i = (int)nel;
  int u;
  if (uhf >= 0) {
    u = uhf;
    if (u > nel_i) return fail(GBXTB_ERR_ARG, "more unpaired electrons than electrons");
    if ((u % 2) != (nel_i % 2)) return fail(GBXTB_ERR_ARG, "parity of unpaired electrons and electrons differs");
  } else {
    u = nel_i % 2;
  }
  const double nb = (nel - u) / 2.0;
  mm.nel[0] = nb + u;
  mm.nel[1] = nb;
  return GBXTB_OK;
}

int set_error(int code, const std::string &msg) { return fail(code, msg); }
size_t plan_workspace_bytes(const gbxtb_plan *plan) { return plan ? plan->ws_bytes : 0; }
int plan_device(const gbxtb_plan *plan) { return plan ? plan->ctx->device : -1; }

int check_options(const gbxtb_options *o) {
  if (!o) return fail(GBXTB_ERR_ARG, "null options");
  if (o->maxiter < 0) return fail(GBXTB_ERR_ARG, "maxiter must be >= 0");
  if (o->fermi_maxiter < 1) return fail(GBXTB_ERR_ARG, "fermi_maxiter must be >= 1");
  if (!(o->kt > 0.0)) return fail(GBXTB_ERR_ARG, "the electronic temperature must be positive");
  if (!(std::isfinite(o->x_atol) && std::isfinite(o->x_atol_max)))
    return fail(GBXTB_ERR_ARG, "x_atol and x_atol_max must be finite");
  switch (o->mixer) {
    case GBXTB_MIXER_BROYDEN:
      if (o->broyden_memory < 1 || o->broyden_memory > kHistMax)
        return fail(GBXTB_ERR_ARG, "broyden_memory must be in 1.." + std::to_string(kHistMax));
      if (!std::isfinite(o->broyden_alpha)) return fail(GBXTB_ERR_ARG, "broyden_alpha must be finite");
      break;
    case GBXTB_MIXER_ANDERSON:
      if (o->generations < 1 || o->generations > kHistMax - 1)
        return fail(GBXTB_ERR_ARG, "generations must be in 1.." + std::to_string(kHistMax - 1));
      if (!(std::isfinite(o->damp) && std::isfinite(o->damp_init) && std::isfinite(o->diagonal_offset)))
        return fail(GBXTB_ERR_ARG, "damp, damp_init and diagonal_offset must be finite");
      break;
    case GBXTB_MIXER_SIMPLE:
      if (!std::isfinite(o->damp)) return fail(GBXTB_ERR_ARG, "damp must be finite");
      break;
    default:
      return fail(GBXTB_ERR_ARG, "unknown mixer " + std::to_string(o->mixer));
  }
  if (!std::isfinite(o->fermi_thresh)) return fail(GBXTB_ERR_ARG, "fermi_thresh must be finite");
  if (o->restart_at < 0) return fail(GBXTB_ERR_ARG, "restart_at must be >= 0");
  if (o->fp64_split < 0 || o->fp64_split > 2) return fail(GBXTB_ERR_ARG, "fp64_split must be 0, 1 or 2");
  if (o->restart_at > 0 && (o->generations < 1 || o->generations > kHistMax - 1 || !std::isfinite(o->damp) ||
                            !std::isfinite(o->damp_init) || !std::isfinite(o->diagonal_offset)))
    return fail(GBXTB_ERR_ARG, "restart_at needs valid Anderson options (generations, damp, damp_init, offset)");
  if (o->damp_dynamic && !std::isfinite(o->damp_dynamic_factor))
    return fail(GBXTB_ERR_ARG, "damp_dynamic_factor must be finite");
  return GBXTB_OK;
}
}  // namespace gbxtb

extern "C" {

int gbxtb_version(void) { return GBXTB_VERSION; }

void gbxtb_default_options(gbxtb_options *o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->maxiter = 100;
  o->fermi_maxiter = 200;
  o->broyden_memory = 20;
  o->want_forces = 0;
  o->x_atol = 1.0e-4;
  o->x_atol_max = 1.0e-5;
  o->kt = 300.0 * (1.3806488e-23 / 4.35974434e-18);  // 300 K in Hartree: k_B / E_h (CODATA 2010)
  o->broyden_alpha = 0.2;
  o->profile = 0;
  o->mixed_precision = 0;
  o->mixer = GBXTB_MIXER_ANDERSON;
  o->generations = 5;
  o->damp = 0.5;
  o->damp_init = 0.1;
  o->diagonal_offset = 0.01;
  o->soft_start = 1;
  o->mix_guess = 1;
  o->damp_dynamic = 0;
  o->damp_dynamic_factor = 0.99;
  o->fermi_thresh = 0.0;
}

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
    MolMaps mm;
    const int rc = describe_molecule(ctx, numbers + a0, (int)(a1 - a0), charge ? charge[m] : 0.0,
                                     (uhf && uhf[m] >= 0) ? uhf[m] : -1, mm);
    if (rc) return rc;
    MolDesc &md = mol[m];
    md.atom0 = (int32_t)atom_z.size();
    md.natom = mm.natom;
    md.sh0 = (int32_t)sh_atom.size();
    md.ao0 = (int32_t)ao_sh.size();
    md.nsh = mm.nsh;
    md.nao = mm.nao;
    md.nel[0] = mm.nel[0];
    md.nel[1] = mm.nel[1];
    for (int a = 0; a < mm.natom; ++a) {
      atom_z.push_back(mm.atom_z[a]);
      atom_mol.push_back(m);
      atom_sh0.push_back(md.sh0 + mm.atom_sh0[a]);
      atom_nsh.push_back(mm.atom_nsh[a]);
    }
    for (int k = 0; k < mm.nsh; ++k) {
      sh_atom.push_back(md.atom0 + mm.sh_atom[k]);
      sh_rec.push_back(mm.sh_rec[k]);
      sh_ao.push_back(mm.sh_ao[k]);
      sh_l.push_back(mm.sh_l[k]);
      sh_mol.push_back(m);
    }
    for (int k = 0; k < mm.nao; ++k) {
      ao_sh.push_back(md.sh0 + mm.ao_sh[k]);
      ao_n0.push_back(mm.ao_n0[k]);
    }
    const int nao = mm.nao;
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
    d.bin_warps[c] = kSmemBinWarps[c];
  }
  d.bisect_threads = 256;
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
  for (int m = 0; m < nmol; ++m) pl->nbig += (mol[m].nao > kClusterMinN) ? 1 : 0;
  pl->ws_bytes = make_layout(d).total;
  *workspace_bytes = pl->ws_bytes;
  *out = pl;
  return GBXTB_OK;
}

void gbxtb_plan_destroy(gbxtb_plan *plan) {
  if (!plan) return;
  for (int g = 0; g < 2; ++g)
    if (plan->pass_graph[g]) cudaGraphExecDestroy(plan->pass_graph[g]);
  if (plan->capture_stream) cudaStreamDestroy(plan->capture_stream);
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
  CK(cudaMemsetAsync(w.status, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.phase, 0, sizeof(int32_t) * pl.nmol, s));
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

namespace {
// Reset the SCF state and enqueue the geometry terms of a call.
int enqueue_setup(gbxtb_plan *plan, const Work &w, const gbxtb_options &o, const double *positions_dev,
                  cudaStream_t s, Prof &pf) {
  const DevPlan &pl = plan->pl;
  const DevParams p = call_params(plan->ctx->p, o);
  const gbxtb_options *opts = &o;
  // reset state
  CK(cudaMemsetAsync(w.status, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.phase, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.iter, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.kvec, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.nhist, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.npass32, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.stall32, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.mixstep, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.dampsw, 0, sizeof(int32_t) * pl.nmol, s));
  CK(cudaMemsetAsync(w.mixsel, 0, sizeof(int32_t) * pl.nmol, s));
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
  const int nchol = launch_cholesky(pl, w, plan->maxn, s);
  // H0' = L^-1 H0 L^-T once per geometry (the potential is still zero)
  launch_gemm(pl, w, plan->tile0, plan->ntile, 0, 0, s);
  launch_gemm(pl, w, plan->tile0, plan->ntile, 5, 0, s);
  if (opts->mixed_precision) launch_lowp_copies(pl, w, s);
  pf.end(GBXTB_PROF_CHOLESKY, nchol + (opts->mixed_precision ? 3 : 2));
  CK(cudaGetLastError());
  return GBXTB_OK;
}
}  // namespace

namespace {
// Enqueue one SCF pass on stream s: lists of iterating molecules at most
// `active` long (tail shapes), cluster passes at most `nclus`.  Returns
// the number of kernel launches; times kernel classes when pf is given.
int enqueue_pass(gbxtb_plan *plan, const Work &w, const gbxtb_options &o, bool tail, int active, int nclus,
                 cudaStream_t s, Prof *pf) {
  const DevPlan &pl = plan->pl;
  const DevParams &p = plan->ctx->p;
  const gbxtb_options *opts = &o;
  Prof none{plan, s, false};
  Prof &prof = pf ? *pf : none;
  const int64_t before = plan->total_launches;
  prof.begin(GBXTB_PROF_FOCK);
  launch_gemm(pl, w, plan->tile0, plan->ntile, 6, 0, s);
  prof.end(GBXTB_PROF_FOCK, 1);
  prof.begin(GBXTB_PROF_TRIDIAG);
  // FP32 passes in shared memory, except large molecules in the tail
  if (opts->mixed_precision) launch_tridiag_smem(pl, w, s, tail);
  int ntrd = opts->mixed_precision ? plan->smem_launches : 0;
  if (tail) {
    ntrd += launch_tridiag_cluster(pl, w, w.active_list, active, plan->maxn, s, true, split64(*opts));
  } else {
    // large FP64 passes and FP32 passes too large for shared memory on 8-SM
    // clusters, the rest one CTA per molecule
    if (nclus > 0)
      ntrd += launch_tridiag_cluster(pl, w, w.cluster_list, nclus, plan->maxn, s, false, split64(*opts));
    launch_tridiag(pl, w, plan->maxn, s);
    ntrd += 1;
  }
  prof.end(GBXTB_PROF_TRIDIAG, ntrd);
  prof.begin(GBXTB_PROF_BISECT);
  if (tail)
    launch_bisect(pl, w, plan->maxn, opts->kt, w.active_list, active, 32, s);
  else
    launch_bisect(pl, w, plan->maxn, opts->kt, nullptr, pl.nmol, pl.bisect_threads, s);
  prof.end(GBXTB_PROF_BISECT, 1);
  prof.begin(GBXTB_PROF_FERMI);
  launch_fermi(pl, w, opts->kt, opts->fermi_maxiter, opts->fermi_thresh, s);
  prof.end(GBXTB_PROF_FERMI, 1);
  prof.begin(GBXTB_PROF_INVIT);
  launch_invit(pl, w, plan->maxn, s);
  prof.end(GBXTB_PROF_INVIT, 1);
  prof.begin(GBXTB_PROF_BACKTRANSFORM);
  if (tail)
    launch_backtransform(pl, w, plan->maxn, w.active_list, active, s);
  else
    launch_backtransform(pl, w, plan->maxn, nullptr, pl.nmol, s);
  prof.end(GBXTB_PROF_BACKTRANSFORM, 1);
  prof.begin(GBXTB_PROF_DENSITY);
  launch_gemm(pl, w, plan->tile0, plan->ntile, 2, 0, s);
  launch_gemm(pl, w, plan->tile0, plan->ntile, 3, 0, s);
  prof.end(GBXTB_PROF_DENSITY, 2);
  prof.begin(GBXTB_PROF_MIX);
  launch_charges_mix(p, pl, w, *opts, s);
  launch_count_active(pl, w, s);
  prof.end(GBXTB_PROF_MIX, 2);
  const int n = (int)(plan->total_launches - before);
  if (!pf) plan->total_launches = before;  // counted when the graph is launched
  return n;
}
}  // namespace

int gbxtb_singlepoint(gbxtb_plan *plan, const gbxtb_options *opts, const double *positions_dev,
                      double *energy_dev, double *charges_dev, double *gradient_dev,
                      void *workspace_dev, size_t workspace_bytes, void *stream) {
  if (!opts || !energy_dev) return fail(GBXTB_ERR_ARG, "null argument");
  if (opts->want_forces && !gradient_dev) return fail(GBXTB_ERR_ARG, "forces requested without gradient buffer");
  if (const int orc = check_options(opts)) return orc;
  Work w;
  int rc = prepare(plan, positions_dev, workspace_dev, workspace_bytes, w);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const DevPlan &pl = plan->pl;
  const DevParams p = call_params(plan->ctx->p, *opts);
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
  rc = enqueue_setup(plan, w, *opts, positions_dev, s, pf);
  if (rc) return rc;
  // SCF: maxiter mixing iterations + the first evaluation + the final pass,
  // and with restart_at the passes before the restart on top (a restarted
  // molecule gets a fresh maxiter budget)
  const int max_loops = opts->maxiter + 3 + (opts->restart_at > 0 ? opts->restart_at : 0);
  int active = pl.nmol;  // molecules iterating (known after each pass)
  int nclus = 0;         // of those, passes that tridiagonalise on a cluster
  launch_count_active(pl, w, s);
  CK(cudaMemcpyAsync(plan->h_active, w.active, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  nclus = plan->h_active[1];
  plan->total_launches += 1;
  // the passes: replayed as a CUDA graph of one pass (one graph launch and
  // one 8-byte copy per pass), or launched one by one with per-class timing
  // when profiling
  const bool use_graph = !pf.on;
  if (use_graph) {
    const bool stale = plan->graph_ws != workspace_dev ||
                       std::memcmp(&plan->graph_opts, opts, sizeof(gbxtb_options)) != 0;
    if (stale) {
      for (int g = 0; g < 2; ++g) {
        if (plan->pass_graph[g]) cudaGraphExecDestroy(plan->pass_graph[g]);
        plan->pass_graph[g] = nullptr;
      }
      plan->graph_ws = workspace_dev;
      plan->graph_opts = *opts;
    }
    // captured on a stream of the plan's own: the caller's stream may be
    // the legacy default stream, which cannot be captured; capturing runs
    // nothing, so it needs no ordering with the caller's work
    if (!plan->capture_stream) CK(cudaStreamCreateWithFlags(&plan->capture_stream, cudaStreamNonBlocking));
    cudaStream_t cs = plan->capture_stream;
    for (int g = 0; g < 2; ++g) {
      if (plan->pass_graph[g]) continue;
      cudaGraph_t graph = nullptr;
      CK(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
      const int nl = g ? std::min(pl.nmol, plan->num_sms) : pl.nmol;
      const int n = enqueue_pass(plan, w, *opts, g == 1, nl, plan->nbig, cs, nullptr);
      const cudaError_t ce =
          cudaMemcpyAsync(plan->h_active, w.active, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, cs);
      // end the capture on every path, so that the stream is usable again
      const cudaError_t ee = cudaStreamEndCapture(cs, &graph);
      if (n < 0 || ce != cudaSuccess || ee != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        if (n < 0) return n;
        return cuda_fail(ce != cudaSuccess ? ce : ee, "pass capture");
      }
      const cudaError_t ge = cudaGraphInstantiate(&plan->pass_graph[g], graph, 0);
      cudaGraphDestroy(graph);
      if (ge != cudaSuccess) return cuda_fail(ge, "cudaGraphInstantiate");
      plan->pass_graph_launches[g] = n;
    }
  }
  for (int it = 0; it < max_loops; ++it) {
    // fewer molecules than SMs (the tail of the batch): spread each molecule
    // over more SMs (an 8-SM cluster for the tridiagonalisation, more blocks
    // for bisection and back-transformation), working from the device-side
    // list of molecules still iterating
    const bool tail = it > 0 && active <= plan->num_sms;
    if (use_graph) {
      CK(cudaGraphLaunch(plan->pass_graph[tail ? 1 : 0], s));
      plan->total_launches += plan->pass_graph_launches[tail ? 1 : 0];
    } else {
      enqueue_pass(plan, w, *opts, tail, active, nclus, s, &pf);
      CK(cudaMemcpyAsync(plan->h_active, w.active, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(s));
    pf.harvest();
    active = plan->h_active[0];
    nclus = plan->h_active[1];
    if (active == 0) break;
  }
  // every molecule ends within max_loops passes; one still iterating would
  // have no final state, so it is an error, never a silent result
  if (active != 0)
    return fail(GBXTB_ERR_CUDA, "internal: " + std::to_string(active) + " molecules still iterating after " +
                                    std::to_string(max_loops) + " SCF passes");
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
  plan->last_ws = workspace_dev;
  plan->last_opts = *opts;
  plan->has_run = true;
  return GBXTB_OK;
}

int gbxtb_forces(gbxtb_plan *plan, const double *positions_dev, double *gradient_dev, void *workspace_dev,
                 size_t workspace_bytes, void *stream) {
  if (!gradient_dev) return fail(GBXTB_ERR_ARG, "null argument");
  if (!plan || !plan->has_run) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  if (workspace_dev != plan->last_ws)
    return fail(GBXTB_ERR_ARG, "the workspace is not the one of the plan's last singlepoint");
  Work w;
  const int rc = prepare(plan, positions_dev, workspace_dev, workspace_bytes, w);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  launch_gemm(plan->pl, w, plan->tile0, plan->ntile, 4, 1, s);
  launch_forces(call_params(plan->ctx->p, plan->last_opts), plan->pl, w, positions_dev, gradient_dev, s);
  CK(cudaGetLastError());
  plan->last_stream = s;
  return GBXTB_OK;
}

int gbxtb_plan_autotune(gbxtb_plan *plan, const gbxtb_options *opts, const double *positions_dev,
                        void *workspace_dev, size_t workspace_bytes, void *stream, int32_t *choice) {
  if (!opts) return fail(GBXTB_ERR_ARG, "null argument");
  if (const int orc = check_options(opts)) return orc;
  Work w;
  int rc = prepare(plan, positions_dev, workspace_dev, workspace_bytes, w);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  DevPlan &pl = plan->pl;
  gbxtb_options o = *opts;
  o.mixed_precision = 1;  // the tuned kernels serve the FP32 passes
  o.profile = 0;
  Prof none{plan, s, false};
  rc = enqueue_setup(plan, w, o, positions_dev, s, none);
  if (rc) return rc;
  // the first pass's FP32 Fock matrices are the tuning input
  launch_gemm(pl, w, plan->tile0, plan->ntile, 6, 0, s);
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  auto time_ms = [&](auto &&launch) -> float {
    launch();  // warm
    cudaEventRecord(e0, s);
    launch();
    launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return ms;
  };
  // warps per CTA of the on-chip tridiagonalisation, per size class (the
  // kernel reads its matrix from the lower triangle, which a run leaves
  // intact, so repeated runs time the same work)
  const int cand_w[3] = {8, 16, 32};
  for (int c = 0; c < kSmemBins; ++c) {
    if (pl.bin_count[c] <= 0) continue;
    float best = 1e30f;
    int pick = pl.bin_warps[c];
    for (int nw : cand_w) {
      DevPlan one = pl;
      for (int q = 0; q < kSmemBins; ++q) one.bin_count[q] = (q == c) ? pl.bin_count[q] : 0;
      one.bin_warps[c] = nw;
      const float ms = time_ms([&] { launch_tridiag_smem(one, w, s); });
      if (ms < best) {
        best = ms;
        pick = nw;
      }
    }
    pl.bin_warps[c] = pick;
  }
  launch_tridiag_smem(pl, w, s);
  // threads per CTA of the batch-wide eigenvalue search
  {
    const int cand_t[3] = {64, 128, 256};
    float best = 1e30f;
    int pick = pl.bisect_threads;
    for (int t : cand_t) {
      const float ms = time_ms([&] { launch_bisect(pl, w, plan->maxn, o.kt, nullptr, pl.nmol, t, s); });
      if (ms < best) {
        best = ms;
        pick = t;
      }
    }
    pl.bisect_threads = pick;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  // captured passes used the old shapes
  for (int g = 0; g < 2; ++g) {
    if (plan->pass_graph[g]) cudaGraphExecDestroy(plan->pass_graph[g]);
    plan->pass_graph[g] = nullptr;
  }
  if (choice) {
    for (int c = 0; c < kSmemBins; ++c) choice[c] = pl.bin_warps[c];
    choice[kSmemBins] = pl.bisect_threads;
  }
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

int gbxtb_get_orbital_charges(gbxtb_plan *plan, double *charges) {
  if (!plan || !plan->has_run || !charges) return fail(GBXTB_ERR_ARG, "no singlepoint has run on this plan");
  CK(cudaStreamSynchronize(plan->last_stream));
  CK(cudaMemcpy(charges, plan->last_work.q, sizeof(double) * plan->pl.nao, cudaMemcpyDeviceToHost));
  return GBXTB_OK;
}

}  // extern "C"
