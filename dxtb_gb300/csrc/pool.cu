// Slot pool: continuous batching of single points (the serving form of the
// engine).
//
// A pool owns a fixed number of slots, each with room for a molecule of up
// to cap_atoms atoms, cap_sh shells and cap_ao AOs.  Every per-molecule
// array of the engine is laid out by slot capacity, so a slot's matrices and
// vectors stay at fixed offsets while molecules of different sizes pass
// through it.  A step runs, on the pool's stream:
//   1. the set-up of the molecules admitted since the last step: their index
//      maps and positions are uploaded into their slots, their SCF state is
//      reset, and the geometry kernels run for them only (phase Setup);
//   2. one SCF pass for every slot that is iterating (the same kernels as a
//      batch call; newly admitted molecules join at their first pass);
//   3. the forces of the molecules that converged in this pass (phase
//      Finished), and a device-side list of the slots that ended.
// The host reads that list after the step, copies each ended molecule's
// energy, charges, gradient and status out, and frees its slot for the next
// request.  Molecules therefore enter and leave the batch between any two
// passes, and their SCF state stays on the device for their whole stay.
//
// Reference behaviour per molecule: calculators/types/energy.py:78-402 and
// types/autograd.py:82-201, with the reference's convergence test and the
// last unmixed potential defining the final state
// (scf/unrolling/default.py:71-136).
#include "engine.h"

#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

using namespace gbxtb;

namespace {

// Reset the SCF state of the admitted slots and mark them for set-up.
__global__ void k_pool_reset(DevPlan pl, Work w, const int32_t *slots, int n, int mixed) {
  const int k = blockIdx.x;
  if (k >= n) return;
  const int m = slots[k];
  const MolDesc md = pl.mol[m];
  if (threadIdx.x == 0) {
    w.status[m] = 0;
    w.phase[m] = kPhaseSetup;
    w.iter[m] = 0;
    w.kvec[m] = 0;
    w.nhist[m] = 0;
    w.prec[m] = mixed ? 0 : 1;
    w.npass32[m] = 0;
    w.stall32[m] = 0;
    w.mixstep[m] = 0;
    w.dampsw[m] = 0;
    w.mixsel[m] = 0;
    w.best32[m] = 1.0e300;
    for (int c = 0; c < 6; ++c) w.energy[(size_t)m * 6 + c] = 0.0;
  }
  for (int i = threadIdx.x; i < md.nsh; i += blockDim.x) w.vin[md.sh0 + i] = 0.0;
}

// Admitted slots whose set-up succeeded start iterating; append them to the
// device lists of iterating molecules (and of large FP64 passes) that the
// previous step left for this one.
__global__ void k_pool_begin(DevPlan pl, Work w, const int32_t *slots, int n) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int act = w.active[0], big = w.active[1];
  for (int k = 0; k < n; ++k) {
    const int m = slots[k];
    if (w.phase[m] != kPhaseSetup) continue;  // set-up failed (status says why)
    w.phase[m] = kPhaseIterate;
    w.active_list[act++] = m;
    if (cluster_pass(w.prec[m], pl.mol[m].nao)) w.cluster_list[big++] = m;
  }
  w.active[0] = act;
  w.active[1] = big;
}

// Evict one iterating slot between steps: it no longer takes part in the
// passes, is not reported as ended, and the device lists of iterating
// molecules are rebuilt without it (k_count_active runs after this).
__global__ void k_pool_evict(Work w, int32_t *inflight, int slot) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  w.phase[slot] = kPhaseDone;
  inflight[slot] = 0;
}

// Slots that ended in this step (converged, hit maxiter, or failed): list
// them for the host and free their phase.  out[0] = count, out[1..] slots;
// out[nslots + 1], out[nslots + 2] = iterating molecules, large FP64 passes.
__global__ void k_pool_collect(DevPlan pl, Work w, int32_t *inflight, int32_t *out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int c = 0;
  for (int m = 0; m < pl.nmol; ++m) {
    if (!inflight[m]) continue;
    const int ph = w.phase[m];
    if (ph == kPhaseFinished || ph == kPhaseDone) {
      w.phase[m] = kPhaseDone;
      inflight[m] = 0;
      out[1 + c++] = m;
    }
  }
  out[0] = c;
  out[pl.nmol + 1] = w.active[0];
  out[pl.nmol + 2] = w.active[1];
}

}  // namespace

struct gbxtb_pool {
  gbxtb_plan *plan = nullptr;  // slot plan (owns the index arrays)
  gbxtb_options opts{};
  int nslots = 0, cap_atoms = 0, cap_sh = 0, cap_ao = 0;
  void *ws = nullptr;          // engine workspace of the slot plan
  Work w{};
  double *pos = nullptr;       // [nslots * cap_atoms * 3]
  double *grad = nullptr;      // [nslots * cap_atoms * 3]
  int32_t *inflight = nullptr; // [nslots]
  int32_t *slots_dev = nullptr;  // [nslots] admitted in this step
  int32_t *out_dev = nullptr;    // [nslots + 3] collect output
  int32_t *out_host = nullptr;   // pinned copy
  // host mirrors of the index arrays (uploaded per admitted slot)
  std::vector<MolDesc> mol;
  std::vector<int32_t> atom_z, atom_mol, atom_sh0, atom_nsh;
  std::vector<int32_t> sh_atom, sh_rec, sh_ao, sh_l, sh_mol, ao_sh;
  std::vector<double> ao_n0;
  // slot bookkeeping
  std::vector<int> free_slots;
  std::vector<int> state;  // 0 free, 1 admitted (pending), 2 in flight, 3 ended (result ready)
  std::vector<int> pending;
  std::vector<std::vector<double>> pending_pos;
  int active = 0, nclus = 0;
  cudaStream_t stream = nullptr;  // stream of the step in flight
  cudaEvent_t done_event = nullptr;  // recorded after the step's last copy
  bool launched = false;
};

namespace {

// Device pointers of the slot plan's index arrays, in upload order.
struct PlanArrays {
  MolDesc *mol;
  int32_t *atom_z, *atom_mol, *atom_sh0, *atom_nsh;
  int32_t *sh_atom, *sh_rec, *sh_ao, *sh_l, *sh_mol, *ao_sh;
  double *ao_n0;
};

PlanArrays plan_arrays(const gbxtb_plan *p) {
  const DevPlan &d = p->pl;
  return PlanArrays{const_cast<MolDesc *>(d.mol),      const_cast<int32_t *>(d.atom_z),
                    const_cast<int32_t *>(d.atom_mol), const_cast<int32_t *>(d.atom_sh0),
                    const_cast<int32_t *>(d.atom_nsh), const_cast<int32_t *>(d.sh_atom),
                    const_cast<int32_t *>(d.sh_rec),   const_cast<int32_t *>(d.sh_ao),
                    const_cast<int32_t *>(d.sh_l),     const_cast<int32_t *>(d.sh_mol),
                    const_cast<int32_t *>(d.ao_sh),    const_cast<double *>(d.ao_n0)};
}

template <typename T>
cudaError_t upload(T *dst, const std::vector<T> &src, size_t first, size_t count, cudaStream_t s) {
  if (count == 0) return cudaSuccess;
  return cudaMemcpyAsync(dst + first, src.data() + first, sizeof(T) * count, cudaMemcpyHostToDevice, s);
}

}  // namespace

extern "C" {

int gbxtb_pool_create(gbxtb_ctx *ctx, const gbxtb_options *opts, int32_t nslots, int32_t cap_atoms,
                      int32_t cap_shells, int32_t cap_aos, gbxtb_pool **out, size_t *device_bytes) {
  if (!ctx || !opts || !out || nslots < 1 || cap_atoms < 1 || cap_shells < 1 || cap_aos < 1)
    return fail(GBXTB_ERR_ARG, "null argument or empty pool");
  if (const int orc = check_options(opts)) return orc;
  if (opts->profile) return fail(GBXTB_ERR_ARG, "profiling is not available for pools");
  auto *pool = new (std::nothrow) gbxtb_pool();
  if (!pool) return fail(GBXTB_ERR_NOMEM, "host allocation failed");
  pool->opts = *opts;
  pool->opts.want_forces = 1;
  pool->nslots = nslots;
  pool->cap_atoms = cap_atoms;
  pool->cap_sh = cap_shells;
  pool->cap_ao = cap_aos;
  auto *plan = new (std::nothrow) gbxtb_plan();
  if (!plan) {
    delete pool;
    return fail(GBXTB_ERR_NOMEM, "host allocation failed");
  }
  pool->plan = plan;
  plan->ctx = ctx;
  plan->maxn = cap_aos;
  // slot layout: every offset by capacity
  pool->mol.resize(nslots);
  std::vector<int64_t> tile0(nslots + 1);
  const int64_t ntc = (cap_aos + 63) / 64;
  for (int m = 0; m < nslots; ++m) {
    MolDesc &md = pool->mol[m];
    md.atom0 = m * cap_atoms;
    md.natom = 0;
    md.sh0 = m * cap_shells;
    md.nsh = 0;
    md.ao0 = m * cap_aos;
    md.nao = 0;
    md.mat0 = (int64_t)m * cap_aos * cap_aos;
    md.gam0 = (int64_t)m * cap_shells * cap_shells;
    md.pair0 = (int64_t)m * cap_shells * (cap_shells + 1) / 2;
    md.nel[0] = md.nel[1] = 0.0;
    tile0[m] = (int64_t)m * ntc * ntc;
  }
  tile0[nslots] = (int64_t)nslots * ntc * ntc;
  const size_t na = (size_t)nslots * cap_atoms, ns = (size_t)nslots * cap_shells, no = (size_t)nslots * cap_aos;
  pool->atom_z.assign(na, 1);
  pool->atom_mol.assign(na, 0);
  pool->atom_sh0.assign(na, 0);
  pool->atom_nsh.assign(na, 0);
  pool->sh_atom.assign(ns, 0);
  pool->sh_rec.assign(ns, 0);
  pool->sh_ao.assign(ns, 0);
  pool->sh_l.assign(ns, 0);
  pool->sh_mol.assign(ns, 0);
  pool->ao_sh.assign(no, 0);
  pool->ao_n0.assign(no, 0.0);
  for (int m = 0; m < nslots; ++m) {
    for (int a = 0; a < cap_atoms; ++a) pool->atom_mol[(size_t)m * cap_atoms + a] = m;
    for (int k = 0; k < cap_shells; ++k) pool->sh_mol[(size_t)m * cap_shells + k] = m;
  }
  DevPlan &d = plan->pl;
  d.nmol = nslots;
  d.natom = (int)na;
  d.nsh = (int)ns;
  d.nao = (int)no;
  d.nmat = (int64_t)nslots * cap_aos * cap_aos;
  d.ngam = (int64_t)nslots * cap_shells * cap_shells;
  d.npair = (int64_t)nslots * cap_shells * (cap_shells + 1) / 2;
  d.pool = 1;
  plan->ntile = tile0[nslots];
  // every slot in the shared-memory size class of its capacity; a pool
  // whose capacity exceeds the on-chip limit still lists every slot in the
  // largest class, since its molecules of up to kSmemTridiagMaxN AOs run
  // their FP32 passes there (larger ones on a cluster)
  std::vector<int32_t> bin_slots(nslots);
  for (int m = 0; m < nslots; ++m) bin_slots[m] = m;
  int bin = kSmemBins - 1;
  for (int c = 0; c < kSmemBins; ++c)
    if (cap_aos <= kSmemBinN[c]) {
      bin = c;
      break;
    }
  Layout L;
  const size_t o_mol = L.add(sizeof(MolDesc) * nslots);
  const size_t o_tile = L.add(sizeof(int64_t) * (nslots + 1));
  const size_t o_az = L.add(4 * na), o_am = L.add(4 * na), o_as0 = L.add(4 * na), o_ans = L.add(4 * na);
  const size_t o_sa = L.add(4 * ns), o_sr = L.add(4 * ns), o_so = L.add(4 * ns), o_sl = L.add(4 * ns);
  const size_t o_sm = L.add(4 * ns);
  const size_t o_aos = L.add(4 * no);
  const size_t o_n0 = L.add(8 * no);
  const size_t o_bin = L.add(4 * (size_t)nslots);
  const size_t o_pos = L.add(8 * 3 * na), o_grad = L.add(8 * 3 * na);
  const size_t o_infl = L.add(4 * (size_t)nslots), o_sl2 = L.add(4 * (size_t)nslots);
  const size_t o_out = L.add(4 * ((size_t)nslots + 3));
  cudaError_t e = cudaMalloc(&plan->dbuf, L.total);
  if (e != cudaSuccess) {
    delete plan;
    delete pool;
    return cuda_fail(e, "cudaMalloc(pool)");
  }
  char *b = static_cast<char *>(plan->dbuf);
  d.mol = (const MolDesc *)(b + o_mol);
  plan->tile0 = (int64_t *)(b + o_tile);
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
    d.bin_mols[c] = (const int32_t *)(b + o_bin);
    d.bin_count[c] = (c == bin) ? nslots : 0;
    d.bin_maxn[c] = (c == bin) ? std::min(cap_aos, kSmemTridiagMaxN) : 0;
    d.bin_warps[c] = kSmemBinWarps[c];
  }
  d.bisect_threads = 256;
  plan->smem_launches = 1;
  pool->pos = (double *)(b + o_pos);
  pool->grad = (double *)(b + o_grad);
  pool->inflight = (int32_t *)(b + o_infl);
  pool->slots_dev = (int32_t *)(b + o_sl2);
  pool->out_dev = (int32_t *)(b + o_out);
  PlanArrays pa = plan_arrays(plan);
  cudaMemcpy(pa.mol, pool->mol.data(), sizeof(MolDesc) * nslots, cudaMemcpyHostToDevice);
  cudaMemcpy(plan->tile0, tile0.data(), sizeof(int64_t) * (nslots + 1), cudaMemcpyHostToDevice);
  cudaMemcpy(pa.atom_z, pool->atom_z.data(), 4 * na, cudaMemcpyHostToDevice);
  cudaMemcpy(pa.atom_mol, pool->atom_mol.data(), 4 * na, cudaMemcpyHostToDevice);
  cudaMemset(pa.atom_sh0, 0, 4 * na);
  cudaMemset(pa.atom_nsh, 0, 4 * na);
  cudaMemset(pa.sh_atom, 0, 4 * ns);
  cudaMemset(pa.sh_rec, 0, 4 * ns);
  cudaMemset(pa.sh_ao, 0, 4 * ns);
  cudaMemset(pa.sh_l, 0, 4 * ns);
  cudaMemcpy(pa.sh_mol, pool->sh_mol.data(), 4 * ns, cudaMemcpyHostToDevice);
  cudaMemset(pa.ao_sh, 0, 4 * no);
  cudaMemset(pa.ao_n0, 0, 8 * no);
  cudaMemcpy((void *)d.bin_mols[0], bin_slots.data(), 4 * (size_t)nslots, cudaMemcpyHostToDevice);
  cudaMemset(pool->pos, 0, 8 * 3 * na);
  cudaMemset(pool->inflight, 0, 4 * (size_t)nslots);
  e = set_linalg_smem_limits(cap_aos);
  if (e == cudaSuccess) e = cudaMallocHost(&plan->h_active, sizeof(int32_t) * 4);
  if (e == cudaSuccess) e = cudaMallocHost(&pool->out_host, sizeof(int32_t) * ((size_t)nslots + 3));
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&pool->done_event, cudaEventDisableTiming);
  if (e == cudaSuccess) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&plan->num_sms, cudaDevAttrMultiProcessorCount, dev);
    plan->ws_bytes = make_layout(d).total;
    e = cudaMalloc(&pool->ws, plan->ws_bytes);
  }
  if (e == cudaSuccess) {
    pool->w = make_work(d, pool->ws);
    // every slot free: phase Done, no molecule in the iterating lists
    e = cudaMemset(pool->w.phase, 0x00, sizeof(int32_t) * nslots);
  }
  if (e == cudaSuccess) {
    std::vector<int32_t> done(nslots, kPhaseDone);
    e = cudaMemcpy(pool->w.phase, done.data(), sizeof(int32_t) * nslots, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMemset(pool->w.active, 0, sizeof(int32_t) * 4);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e != cudaSuccess) {
    if (pool->ws) cudaFree(pool->ws);
    if (pool->out_host) cudaFreeHost(pool->out_host);
    if (plan->h_active) cudaFreeHost(plan->h_active);
    cudaFree(plan->dbuf);
    delete plan;
    delete pool;
    return cuda_fail(e, "pool set-up");
  }
  pool->state.assign(nslots, 0);
  for (int m = nslots - 1; m >= 0; --m) pool->free_slots.push_back(m);
  pool->pending_pos.resize(nslots);
  if (device_bytes) *device_bytes = L.total + plan->ws_bytes;
  *out = pool;
  return GBXTB_OK;
}

void gbxtb_pool_destroy(gbxtb_pool *pool) {
  if (!pool) return;
  if (pool->launched && pool->stream) cudaStreamSynchronize(pool->stream);
  if (pool->ws) cudaFree(pool->ws);
  if (pool->out_host) cudaFreeHost(pool->out_host);
  if (pool->done_event) cudaEventDestroy(pool->done_event);
  if (pool->plan) {
    if (pool->plan->h_active) cudaFreeHost(pool->plan->h_active);
    if (pool->plan->dbuf) cudaFree(pool->plan->dbuf);
    delete pool->plan;
  }
  delete pool;
}

int gbxtb_pool_free_slots(const gbxtb_pool *pool) {
  if (!pool) return fail(GBXTB_ERR_ARG, "null argument");
  return (int)pool->free_slots.size();
}

int gbxtb_pool_admit(gbxtb_pool *pool, int32_t natoms, const int32_t *numbers, const double *positions,
                     double charge, int32_t uhf, int32_t *slot_out) {
  if (!pool || !numbers || !positions || !slot_out || natoms < 1) return fail(GBXTB_ERR_ARG, "null argument");
  if (pool->free_slots.empty()) return fail(GBXTB_ERR_WORKSPACE, "no free slot in the pool");
  if (natoms > pool->cap_atoms) return fail(GBXTB_ERR_WORKSPACE, "molecule has more atoms than the slot capacity");
  MolMaps mm;
  const int rc = describe_molecule(pool->plan->ctx, numbers, natoms, charge, uhf, mm);
  if (rc) return rc;
  if (mm.nsh > pool->cap_sh || mm.nao > pool->cap_ao)
    return fail(GBXTB_ERR_WORKSPACE, "molecule has more shells or AOs than the slot capacity");
  const int m = pool->free_slots.back();
  pool->free_slots.pop_back();
  MolDesc &md = pool->mol[m];
  md.natom = mm.natom;
  md.nsh = mm.nsh;
  md.nao = mm.nao;
  md.nel[0] = mm.nel[0];
  md.nel[1] = mm.nel[1];
  for (int a = 0; a < mm.natom; ++a) {
    pool->atom_z[md.atom0 + a] = mm.atom_z[a];
    pool->atom_sh0[md.atom0 + a] = md.sh0 + mm.atom_sh0[a];
    pool->atom_nsh[md.atom0 + a] = mm.atom_nsh[a];
  }
  for (int k = 0; k < mm.nsh; ++k) {
    pool->sh_atom[md.sh0 + k] = md.atom0 + mm.sh_atom[k];
    pool->sh_rec[md.sh0 + k] = mm.sh_rec[k];
    pool->sh_ao[md.sh0 + k] = mm.sh_ao[k];
    pool->sh_l[md.sh0 + k] = mm.sh_l[k];
  }
  for (int k = 0; k < mm.nao; ++k) {
    pool->ao_sh[md.ao0 + k] = md.sh0 + mm.ao_sh[k];
    pool->ao_n0[md.ao0 + k] = mm.ao_n0[k];
  }
  pool->pending_pos[m].assign(positions, positions + 3 * (size_t)natoms);
  pool->pending.push_back(m);
  pool->state[m] = 1;
  *slot_out = m;
  return GBXTB_OK;
}

int gbxtb_pool_step_launch(gbxtb_pool *pool, void *stream) {
  if (!pool) return fail(GBXTB_ERR_ARG, "null argument");
  if (pool->launched) return fail(GBXTB_ERR_ARG, "the previous step has not been finished");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  gbxtb_plan *plan = pool->plan;
  const DevPlan &pl = plan->pl;
  const DevParams p = call_params(plan->ctx->p, pool->opts);
  const Work &w = pool->w;
  const gbxtb_options &o = pool->opts;
  const int nadm = (int)pool->pending.size();
  if (nadm > 0) {
    // index maps, positions and fresh SCF state of the admitted molecules
    PlanArrays pa = plan_arrays(plan);
    for (int m : pool->pending) {
      const MolDesc &md = pool->mol[m];
      CK(cudaMemcpyAsync(pa.mol + m, &md, sizeof(MolDesc), cudaMemcpyHostToDevice, s));
      CK(upload(pa.atom_z, pool->atom_z, md.atom0, md.natom, s));
      CK(upload(pa.atom_sh0, pool->atom_sh0, md.atom0, md.natom, s));
      CK(upload(pa.atom_nsh, pool->atom_nsh, md.atom0, md.natom, s));
      CK(upload(pa.sh_atom, pool->sh_atom, md.sh0, md.nsh, s));
      CK(upload(pa.sh_rec, pool->sh_rec, md.sh0, md.nsh, s));
      CK(upload(pa.sh_ao, pool->sh_ao, md.sh0, md.nsh, s));
      CK(upload(pa.sh_l, pool->sh_l, md.sh0, md.nsh, s));
      CK(upload(pa.ao_sh, pool->ao_sh, md.ao0, md.nao, s));
      CK(upload(pa.ao_n0, pool->ao_n0, md.ao0, md.nao, s));
      CK(cudaMemcpyAsync(pool->pos + 3 * (size_t)md.atom0, pool->pending_pos[m].data(),
                         sizeof(double) * 3 * md.natom, cudaMemcpyHostToDevice, s));
      const int32_t one = 1;
      CK(cudaMemcpyAsync(pool->inflight + m, &one, sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    CK(cudaMemcpyAsync(pool->slots_dev, pool->pending.data(), sizeof(int32_t) * nadm, cudaMemcpyHostToDevice, s));
    // the pageable sources above must stay alive until the copies ran
    CK(cudaStreamSynchronize(s));
    k_pool_reset<<<nadm, 128, 0, s>>>(pl, w, pool->slots_dev, nadm, o.mixed_precision);
    // geometry terms of the admitted molecules only (phase Setup)
    launch_atoms(p, pl, w, pool->pos, true, s);
    launch_shellpairs(p, pl, w, pool->pos, s);
    launch_cholesky(pl, w, plan->maxn, s);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 0, 0, s);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 5, 0, s);
    if (o.mixed_precision) launch_lowp_copies(pl, w, s);
    k_pool_begin<<<1, 32, 0, s>>>(pl, w, pool->slots_dev, nadm);
    CK(cudaGetLastError());
    for (int m : pool->pending) {
      pool->state[m] = 2;
      // (upper bounds of the device-side list lengths that k_pool_begin sets)
      if (cluster_pass(o.mixed_precision ? 0 : 1, pool->mol[m].nao)) pool->nclus += 1;
    }
    pool->active += nadm;
    pool->pending.clear();
  }
  if (pool->active > 0) {
    // one SCF pass for every iterating slot (the launch shapes of a batch
    // call: few molecules spread over more SMs)
    const int active = pool->active, nclus = pool->nclus;
    const bool tail = active <= plan->num_sms;
    launch_gemm(pl, w, plan->tile0, plan->ntile, 6, 0, s);
    if (o.mixed_precision) launch_tridiag_smem(pl, w, s, tail);
    if (tail) {
      launch_tridiag_cluster(pl, w, w.active_list, active, plan->maxn, s, true, split64(o));
      launch_bisect(pl, w, plan->maxn, o.kt, w.active_list, active, 32, s);
    } else {
      if (nclus > 0)
        launch_tridiag_cluster(pl, w, w.cluster_list, nclus, plan->maxn, s, false, split64(o));
      launch_tridiag(pl, w, plan->maxn, s);
      launch_bisect(pl, w, plan->maxn, o.kt, nullptr, pl.nmol, 256, s);
    }
    launch_fermi(pl, w, o.kt, o.fermi_maxiter, o.fermi_thresh, s);
    launch_invit(pl, w, plan->maxn, s);
    if (tail)
      launch_backtransform(pl, w, plan->maxn, w.active_list, active, s);
    else
      launch_backtransform(pl, w, plan->maxn, nullptr, pl.nmol, s);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 2, 0, s);
    launch_gemm(pl, w, plan->tile0, plan->ntile, 3, 0, s);
    launch_charges_mix(p, pl, w, o, s);
    launch_count_active(pl, w, s);
    // forces of the molecules that converged in this pass (phase Finished)
    launch_gemm(pl, w, plan->tile0, plan->ntile, 4, 1, s);
    launch_forces(p, pl, w, pool->pos, pool->grad, s);
  }
  k_pool_collect<<<1, 32, 0, s>>>(pl, w, pool->inflight, pool->out_dev);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(pool->out_host, pool->out_dev, sizeof(int32_t) * ((size_t)pool->nslots + 3),
                     cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(pool->done_event, s));
  pool->stream = s;
  pool->launched = true;
  return GBXTB_OK;
}

int gbxtb_pool_step_poll(gbxtb_pool *pool) {
  if (!pool) return fail(GBXTB_ERR_ARG, "null argument");
  if (!pool->launched) return 1;
  const cudaError_t e = cudaEventQuery(pool->done_event);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return cuda_fail(e, "cudaEventQuery");
}

int gbxtb_pool_step_finish(gbxtb_pool *pool, int32_t *ended, int32_t *nended, int32_t *iterating) {
  if (!pool || !nended) return fail(GBXTB_ERR_ARG, "null argument");
  if (!pool->launched) return fail(GBXTB_ERR_ARG, "no step in flight");
  CK(cudaStreamSynchronize(pool->stream));
  pool->launched = false;
  const int32_t *o = pool->out_host;
  const int c = o[0];
  for (int k = 0; k < c; ++k) {
    const int m = o[1 + k];
    pool->state[m] = 3;
    if (ended) ended[k] = m;
  }
  *nended = c;
  pool->active = o[pool->nslots + 1];
  pool->nclus = o[pool->nslots + 2];
  if (iterating) *iterating = pool->active;
  return GBXTB_OK;
}

int gbxtb_pool_evict(gbxtb_pool *pool, int32_t slot, void *stream) {
  if (!pool || slot < 0 || slot >= pool->nslots) return fail(GBXTB_ERR_ARG, "bad slot");
  if (pool->launched) return fail(GBXTB_ERR_ARG, "a step is in flight; finish it first");
  if (pool->state[slot] != 2) return fail(GBXTB_ERR_ARG, "slot holds no iterating molecule");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  k_pool_evict<<<1, 32, 0, s>>>(pool->w, pool->inflight, slot);
  launch_count_active(pool->plan->pl, pool->w, s);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(s));
  pool->state[slot] = 0;
  pool->free_slots.push_back(slot);
  return GBXTB_OK;
}

int gbxtb_pool_result(gbxtb_pool *pool, int32_t slot, double *energy, double *charges, double *gradient,
                      int32_t *status, int32_t *iterations) {
  if (!pool || slot < 0 || slot >= pool->nslots) return fail(GBXTB_ERR_ARG, "bad slot");
  if (pool->state[slot] != 3) return fail(GBXTB_ERR_ARG, "slot has no result");
  if (pool->launched) CK(cudaStreamSynchronize(pool->stream));
  const MolDesc &md = pool->mol[slot];
  const Work &w = pool->w;
  if (energy) CK(cudaMemcpy(energy, w.energy + (size_t)slot * 6, sizeof(double), cudaMemcpyDeviceToHost));
  if (charges) CK(cudaMemcpy(charges, w.qat + md.atom0, sizeof(double) * md.natom, cudaMemcpyDeviceToHost));
  if (gradient)
    CK(cudaMemcpy(gradient, pool->grad + 3 * (size_t)md.atom0, sizeof(double) * 3 * md.natom,
                  cudaMemcpyDeviceToHost));
  if (status) CK(cudaMemcpy(status, w.status + slot, sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (iterations) CK(cudaMemcpy(iterations, w.iter + slot, sizeof(int32_t), cudaMemcpyDeviceToHost));
  pool->state[slot] = 0;
  pool->free_slots.push_back(slot);
  return GBXTB_OK;
}

}  // extern "C"
