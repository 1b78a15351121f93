/*
 * gbxtb: GFN1-xTB single points (energy, charges, forces) on NVIDIA GB300.
 *
 * C ABI of libgbxtb.so.  All arrays named *_dev are device pointers owned by
 * the caller; all other pointers are host memory.  Every entry point returns
 * GBXTB_OK (0) or a negative error code and never aborts the process;
 * gbxtb_last_error() gives a message for the last failure on this thread.
 *
 * The library replaces the reference calculator's single-point path
 * (dxtb: src/dxtb/_src/calculators/types/energy.py:78-402 for the energy,
 * src/dxtb/_src/calculators/types/autograd.py:82-201 and
 * src/dxtb/_src/calculators/types/analytical.py:63-222 for the forces).
 * A Python (ctypes) binding that mirrors dxtb's GFN1Calculator sits in
 * dxtb_gb300/calculator.py, and dxtb_gb300/csrc/torch_ops.cpp exposes the
 * single point and its adjoint as torch operators (torch.ops.gbxtb.*).
 */
#ifndef GBXTB_H
#define GBXTB_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define GBXTB_API __attribute__((visibility("default")))
#else
#define GBXTB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBXTB_VERSION 1

/* return codes */
#define GBXTB_OK 0
#define GBXTB_ERR_ARG (-1)      /* invalid argument (null pointer, bad size) */
#define GBXTB_ERR_CUDA (-2)     /* a CUDA call failed */
#define GBXTB_ERR_ELEMENT (-3)  /* atomic number without parameters */
#define GBXTB_ERR_WORKSPACE (-4) /* workspace smaller than required */
#define GBXTB_ERR_NOMEM (-5)    /* host or device allocation failed */

/* per-molecule status bits (gbxtb_get_status) */
#define GBXTB_MOL_OK 0
#define GBXTB_MOL_NOT_CONVERGED 1 /* SCF hit maxiter; result is the last iterate,
                                     as the reference returns with an
                                     SCFConvergenceWarning
                                     (scf/unrolling/default.py:123-136) */
#define GBXTB_MOL_FERMI_FAIL 2    /* Fermi level not found in fermi_maxiter
                                     (reference raises, wavefunction/filling.py:366) */
#define GBXTB_MOL_CHOLESKY_FAIL 4 /* overlap not positive definite */
#define GBXTB_MOL_NONFINITE 8     /* NaN/Inf appeared */
#define GBXTB_MOL_RESTARTED 16    /* not a failure: the molecule did not converge in
                                     opts->restart_at passes and was solved again
                                     from the guess with the reference's Anderson
                                     mixer (iterations count that second run) */

typedef struct gbxtb_ctx gbxtb_ctx;
typedef struct gbxtb_plan gbxtb_plan;

/* Number of doubles per element / shell record in gbxtb_params. */
#define GBXTB_ELEM_DOUBLES 8   /* gam, gam3, zeff, arep, en, rad(bohr), rcov_d3(bohr), xbond */
#define GBXTB_SHELL_INTS 4     /* l, nprim, valence, 0 */
#define GBXTB_SHELL_DOUBLES 24 /* alpha[8], coeff[8], level(Eh), kcn(Eh), shpoly, refocc, lgam, 0, 0, 0 */
#define GBXTB_MAX_PRIM 8
#define GBXTB_GLOBALS 16
/* globals: 0 kpol, 1 enscale, 2 k_ss, 3 k_pp, 4 k_dd, 5 k_sp, 6 kexp (repulsion),
 *          7 cn steepness, 8 cn cutoff, 9 repulsion cutoff, 10 integral cutoff,
 *          11 gexp (must be 2), 12 halogen-bond damping, 13 halogen-bond radius
 *          scale, 14 halogen-bond cutoff (bohr), 15 unused */

/* GFN1 parameter tables (host).  Element z uses shell records
 * [elem_shell0[z], elem_shell0[z] + elem_nshell[z]).  Contraction
 * coefficients already include primitive normalisation and the GFN1
 * orthogonalisation of non-valence shells
 * (dxtb: basis/bas.py:149-193, basis/slater.py:69-135, basis/ortho.py:74-110). */
typedef struct {
  int32_t max_z;              /* tables are indexed 0..max_z */
  int32_t n_shell_records;
  const int32_t *elem_shell0; /* [max_z+1] */
  const int32_t *elem_nshell; /* [max_z+1], 0 = element not parametrised */
  const double *elem_data;    /* [(max_z+1) * GBXTB_ELEM_DOUBLES] */
  const int32_t *shell_int;   /* [n_shell_records * GBXTB_SHELL_INTS] */
  const double *shell_data;   /* [n_shell_records * GBXTB_SHELL_DOUBLES] */
  const double *kpair;        /* [(max_z+1) * (max_z+1)] */
  const double *globals;      /* [GBXTB_GLOBALS] */
} gbxtb_params;

/* SCF mixers (gbxtb_options.mixer). */
#define GBXTB_MIXER_BROYDEN 0  /* modified Broyden (Johnson 1988): the engine's default */
#define GBXTB_MIXER_ANDERSON 1 /* the reference's Anderson/Eyert mixer, step for step
                                  (scf/mixer/anderson.py:200-317): the mixer its
                                  default full-mode SCF runs (scf/unrolling/base.py:81-99) */
#define GBXTB_MIXER_SIMPLE 2   /* linear mixing x + damp (F(x) - x) (scf/mixer/simple.py) */

/* SCF options (dxtb: calculators/config/scf.py:32-433; defaults.py:130-260).
 * gbxtb_default_options() fills every field with the reference's defaults. */
typedef struct {
  int32_t maxiter;        /* SCF iterations (reference option "maxiter") */
  int32_t fermi_maxiter;  /* Newton steps for the Fermi level (200) */
  int32_t broyden_memory; /* Broyden history length (1..29) */
  int32_t want_forces;    /* 0: energy only; 1: energy and forces */
  double x_atol;          /* L2 norm of the potential change ("x_atol") */
  double x_atol_max;      /* max norm of the potential change ("x_atol_max") */
  double kt;              /* electronic temperature in Hartree (fermi_etemp * k_B) */
  double broyden_alpha;   /* Broyden step */
  int32_t profile;        /* 1: time each kernel class with CUDA events (gbxtb_get_profile) */
  int32_t mixed_precision; /* 1: SCF passes run their linear algebra in FP32 while the
                              potential change is above 1e-4 and still falling
                              (8 passes without halving below 1e-3 end them);
                              convergence and the final state are always FP64.
                              0: every pass in FP64 */
  int32_t mixer;           /* GBXTB_MIXER_* */
  int32_t generations;     /* Anderson history ("damp_generations", 5; 1..28) */
  double damp;             /* Anderson / simple mixing parameter ("damp", 0.5) */
  double damp_init;        /* Anderson soft-start parameter ("damp_init", 0.1) */
  double diagonal_offset;  /* Anderson diagonal rescaling ("damp_diagonal_offset",
                              0.01); negative: no rescaling (the reference's None) */
  int32_t soft_start;      /* Anderson: simple mixing for the first `generations`
                              steps ("damp_soft_start", 1) */
  int32_t mix_guess;       /* 1: the first potential is mixed with the guess
                              ("mix_guess", 1); 0: taken unmixed
                              (scf/unrolling/default.py:92-96) */
  int32_t damp_dynamic;    /* 1: once the potential change is below 0.1, later
                              steps use damp_dynamic_factor ("damp_dynamic", 0) */
  int32_t no_halogen;      /* 1: without the halogen-bond term (reference option
                              exclude=["hal"]); 0: with it (the default) */
  double damp_dynamic_factor; /* ("damp_dynamic_factor", 0.99) */
  double fermi_thresh;     /* |sum f - n| at which the Fermi-level Newton search
                              stops ("fermi_thresh"); <= 0: sqrt(machine eps),
                              the reference's default (wavefunction/filling.py:
                              269-366) */
  int32_t restart_at;      /* with the Broyden or simple mixer: a molecule still
                              iterating after this many passes starts again from
                              the guess with the reference's Anderson mixer
                              (generations, damp, damp_init, diagonal_offset,
                              soft_start above), every pass in FP64, with a fresh
                              maxiter budget, so that it follows the reference's
                              own SCF where the faster mixer does not converge;
                              0: never */
  int32_t fp64_split;      /* arithmetic of the FP64 passes of the on-chip cluster
                              tridiagonalisation (molecules of 129-400 AOs, and
                              of up to 400 AOs once fewer molecules than SMs
                              iterate) and of their back-transformation: 0 (auto):
                              double-float pairs on the FP32 pipe (~48 bits)
                              with mixed_precision, native FP64 without;
                              1: native FP64; 2: double-float */
} gbxtb_options;

/* The reference's default SCF options (calculators/config/scf.py:139-190,
 * constants/defaults.py): maxiter 100, x_atol 1e-4, x_atol_max 1e-5, 300 K,
 * Anderson with damp 0.5, damp_init 0.1, 5 generations, offset 0.01, soft
 * start, mixed guess.  Mixed precision, profiling and forces are off. */
GBXTB_API void gbxtb_default_options(gbxtb_options *opts);

/* Kernel classes reported by gbxtb_get_profile. */
#define GBXTB_PROF_ATOMS 0        /* coordination numbers, repulsion */
#define GBXTB_PROF_SHELLPAIRS 1   /* overlap, H0, gamma */
#define GBXTB_PROF_CHOLESKY 2     /* S = L L^T, L^-1 */
#define GBXTB_PROF_FOCK 3         /* L^-1 F L^-T (two GEMMs) */
#define GBXTB_PROF_TRIDIAG 4      /* Householder tridiagonalisation */
#define GBXTB_PROF_BISECT 5       /* tridiagonal eigenvalues */
#define GBXTB_PROF_FERMI 6        /* occupations */
#define GBXTB_PROF_INVIT 7        /* tridiagonal eigenvectors */
#define GBXTB_PROF_BACKTRANSFORM 8
#define GBXTB_PROF_DENSITY 9      /* C = L^-T Y, P = C f C^T (two GEMMs) */
#define GBXTB_PROF_MIX 10         /* charges, potential, mixing */
#define GBXTB_PROF_FORCES 11      /* W, adjoint kernels */
#define GBXTB_PROF_CLASSES 12

/* Library version (GBXTB_VERSION). */
GBXTB_API int gbxtb_version(void);

/* Message describing the last error on the calling thread. */
GBXTB_API const char *gbxtb_last_error(void);

/* Upload the parameter tables to the current CUDA device.
 * Replaces dxtb's parameter loading (param/gfn1/load.py,
 * calculators/types/base.py:451-734 constructor). */
GBXTB_API int gbxtb_ctx_create(const gbxtb_params *params, gbxtb_ctx **out);
GBXTB_API void gbxtb_ctx_destroy(gbxtb_ctx *ctx);

/* Plan a batch of molecules: ragged atomic numbers (host), atom offsets
 * (host, nmol+1), total charge and number of unpaired electrons per molecule
 * (host; uhf may be NULL = derived from electron parity).  Builds the
 * atom/shell/orbital maps on the host and uploads them (replaces
 * basis/indexhelper.py:283-491 and scf/iterator.py:147-189).
 * *workspace_bytes receives the device scratch size needed by
 * gbxtb_singlepoint for this plan. */
GBXTB_API int gbxtb_plan_create(gbxtb_ctx *ctx, int32_t nmol, const int32_t *numbers,
                      const int64_t *atom_offsets, const double *charge,
                      const int32_t *uhf, gbxtb_plan **out,
                      size_t *workspace_bytes);
GBXTB_API void gbxtb_plan_destroy(gbxtb_plan *plan);

/* Sizes of a plan: [nmol, natoms, nshells, naos, nmat_doubles, nshellpair_doubles]. */
GBXTB_API int gbxtb_plan_sizes(const gbxtb_plan *plan, int64_t *sizes6);

/* Overlap and core Hamiltonian for ragged positions (bohr, [natoms][3]).
 * Outputs are per-molecule dense row-major nao x nao blocks, packed one after
 * another (offset of molecule m = sum_{k<m} nao_k^2).
 * Replaces integral/driver/pytorch/impls/overlap.py:147-243 and
 * xtb/base.py:251-360. */
GBXTB_API int gbxtb_integrals(gbxtb_plan *plan, const double *positions_dev,
                    double *overlap_dev, double *hcore_dev, void *workspace_dev,
                    size_t workspace_bytes, void *stream);

/* Full single point: energy per molecule, Mulliken atomic charges (nullable)
 * and the energy gradient dE/dR ([natoms][3], nullable; required when
 * opts->want_forces).  Replaces calculators/types/energy.py:78-402 (energy)
 * and calculators/types/autograd.py:82-201 (forces = -gradient). */
GBXTB_API int gbxtb_singlepoint(gbxtb_plan *plan, const gbxtb_options *opts,
                      const double *positions_dev, double *energy_dev,
                      double *charges_dev, double *gradient_dev,
                      void *workspace_dev, size_t workspace_bytes,
                      void *stream);

/* Energy gradient dE/dR ([natoms][3]) of the final state of the plan's last
 * gbxtb_singlepoint, which must have run on the same positions and the same
 * workspace, untouched since.  Gives the same gradient as that call with
 * opts->want_forces = 1, so a caller that asked for the energy first gets
 * the forces without a second SCF (the reference serves get_forces after
 * get_energy from its cache: calculators/types/decorators.py:228-275,
 * types/autograd.py:82-201). */
GBXTB_API int gbxtb_forces(gbxtb_plan *plan, const double *positions_dev, double *gradient_dev,
                           void *workspace_dev, size_t workspace_bytes, void *stream);

/* Autotune the launch shapes of the eigensolver kernels for this plan on
 * real data: sets up the geometry of `positions_dev`, forms the first
 * pass's FP32 Fock matrices, and times the candidates of (a) warps per CTA
 * of the on-chip FP32 tridiagonalisation for each molecule-size class
 * (8, 16, 32) and (b) threads per CTA of the eigenvalue search (64, 128,
 * 256), keeping the fastest.  Later gbxtb_singlepoint calls use them.
 * choice (nullable, 4 ints): the warps of the 3 size classes, then the
 * threads.  No counterpart in the reference (which calls LAPACK/cuSOLVER). */
GBXTB_API int gbxtb_plan_autotune(gbxtb_plan *plan, const gbxtb_options *opts,
                                  const double *positions_dev, void *workspace_dev,
                                  size_t workspace_bytes, void *stream, int32_t *choice);

/* Per-molecule status bits and SCF iteration counts of the last
 * gbxtb_singlepoint on this plan (host arrays of nmol). Synchronises the
 * stream of that call. */
GBXTB_API int gbxtb_get_status(gbxtb_plan *plan, int32_t *status, int32_t *iterations);

/* Number of SCF passes per molecule that ran in FP32 in the last
 * gbxtb_singlepoint (host array of nmol; 0 without mixed precision).  The
 * molecule's remaining passes (gbxtb_get_status iterations + 1 in total)
 * ran in FP64.  No counterpart in the reference (its SCF is FP64 or FP32
 * throughout).  Synchronises the stream of that call. */
GBXTB_API int gbxtb_get_fp32_passes(gbxtb_plan *plan, int32_t *passes);

/* Per-class device time (ms) and kernel-launch counts of the last
 * gbxtb_singlepoint run with opts->profile = 1 (host arrays of
 * GBXTB_PROF_CLASSES); *total_launches receives all kernel launches of that
 * call (counted with or without profiling). */
GBXTB_API int gbxtb_get_profile(gbxtb_plan *plan, double *ms, int64_t *launches, int64_t *total_launches);

/* Shell-resolved SCF potential of the final state of the last
 * gbxtb_singlepoint (host array of nshells, in plan order); the orbital
 * potential of the reference (scf/base.py:701-727) is this value repeated
 * over the 2l+1 orbitals of each shell.  Synchronises that call's stream. */
GBXTB_API int gbxtb_get_shell_potential(gbxtb_plan *plan, double *potential);

/* Orbital-resolved Mulliken charges q_mu = n0_mu - (P S)_mu,mu of the final
 * state of the last gbxtb_singlepoint (host array of naos, in plan order);
 * replaces get_charges / get_mulliken_charges (calculators/types/abc.py:
 * 429-495, the `mono` charges of scf/base.py:764-815).  The atomic charges
 * that gbxtb_singlepoint writes are their sums over each atom's orbitals.
 * Synchronises that call's stream. */
GBXTB_API int gbxtb_get_orbital_charges(gbxtb_plan *plan, double *charges);

/* ---------------------------------------------------------------------------
 * Slot pool: continuous batching of single points with forces (serving).
 * A pool holds nslots molecules of up to cap_atoms atoms, cap_shells shells
 * and cap_aos AOs each, with their SCF state resident on the device.
 * Requests are admitted into free slots at any time (gbxtb_pool_admit); each
 * step (gbxtb_pool_step_launch + gbxtb_pool_step_finish) sets up the newly
 * admitted molecules, runs one SCF pass for every molecule in the pool, and
 * computes the forces of those that converged; their slots report as ended,
 * and gbxtb_pool_result copies a result out and frees its slot for the next
 * request.  Several pools (size classes) can step on different streams at
 * once: launch them all, then finish them.
 * Per molecule this is the reference's single point with autograd forces
 * (calculators/types/energy.py:78-402, types/autograd.py:82-201); the
 * reference has no serving form (it is a library called once per input).
 * opts->want_forces is implied; opts->profile must be 0.
 * ------------------------------------------------------------------------- */
typedef struct gbxtb_pool gbxtb_pool;

GBXTB_API int gbxtb_pool_create(gbxtb_ctx *ctx, const gbxtb_options *opts, int32_t nslots,
                                int32_t cap_atoms, int32_t cap_shells, int32_t cap_aos,
                                gbxtb_pool **out, size_t *device_bytes);
GBXTB_API void gbxtb_pool_destroy(gbxtb_pool *pool);

/* Free slots of the pool (or a negative error code). */
GBXTB_API int gbxtb_pool_free_slots(const gbxtb_pool *pool);

/* Admit one molecule (host arrays: numbers[natoms], positions[natoms][3] in
 * bohr; uhf < 0: from the electron parity).  *slot receives its slot; it
 * starts at the next step.  GBXTB_ERR_WORKSPACE: no free slot, or the
 * molecule exceeds the slot capacity. */
GBXTB_API int gbxtb_pool_admit(gbxtb_pool *pool, int32_t natoms, const int32_t *numbers,
                               const double *positions, double charge, int32_t uhf, int32_t *slot);

/* Enqueue one step on `stream` (a cudaStream_t). */
GBXTB_API int gbxtb_pool_step_launch(gbxtb_pool *pool, void *stream);

/* 1 if the launched step has completed (or none is in flight), 0 if it is
 * still running, negative on error.  Lets a host drive several pools, each
 * at its own pace, without blocking on the slowest. */
GBXTB_API int gbxtb_pool_step_poll(gbxtb_pool *pool);

/* Wait for the step; ended[0..*nended) receive the slots whose molecule
 * ended in it (host array of nslots; nullable), *iterating the molecules
 * still iterating (nullable). */
GBXTB_API int gbxtb_pool_step_finish(gbxtb_pool *pool, int32_t *ended, int32_t *nended,
                                     int32_t *iterating);

/* Take an iterating molecule out of the pool between steps (no step in
 * flight) and free its slot; it is not reported as ended.  A server uses it
 * to move a molecule that has not converged after many passes out of the
 * way of new requests and to solve it again elsewhere (a fresh SCF of the
 * same molecule gives the same result, so nothing is lost but the passes
 * already spent).  No counterpart in the reference (it has no serving
 * form). */
GBXTB_API int gbxtb_pool_evict(gbxtb_pool *pool, int32_t slot, void *stream);

/* Result of an ended slot (host arrays: energy[1], charges[natoms],
 * gradient[natoms][3] = dE/dR, status[1], iterations[1]; each nullable);
 * frees the slot. */
GBXTB_API int gbxtb_pool_result(gbxtb_pool *pool, int32_t slot, double *energy, double *charges,
                                double *gradient, int32_t *status, int32_t *iterations);

/* Device scratch compiled into the library for gbxtb_singlepoint_noalloc. */
#define GBXTB_NOALLOC_SCRATCH_BYTES ((size_t)32 * 1024 * 1024)

/* gbxtb_singlepoint for callers that cannot allocate device memory.
 * It has no counterpart in the reference, whose PyTorch path allocates as it
 * goes.  Some callers cannot do that when they compute: for example, a host
 * framework whose memory pool must not grow once it is set up, a real-time
 * loop that forbids cudaMalloc after start-up, or a plugin callback that is
 * given only a stream.  This entry point takes no workspace.  Its scratch is
 * a fixed device array of GBXTB_NOALLOC_SCRATCH_BYTES inside the library.
 * It calls no cudaMalloc, cudaFree or allocating library routine.  The
 * caller still owns the positions and outputs (same meaning as
 * gbxtb_singlepoint).  Limits and rules:
 *   - plans whose workspace_bytes (gbxtb_plan_create) exceed the array are
 *     rejected with GBXTB_ERR_WORKSPACE; opts->profile must be 0; the
 *     current device must be the plan's (else GBXTB_ERR_ARG);
 *   - the first call on a device looks up the array's device address (with
 *     that device current); under CUDA's lazy module loading this is also
 *     when the array is loaded onto the device, which holds it from then
 *     until the process exits.  The looked-up address does not survive
 *     cudaDeviceReset;
 *   - the first call on a plan, and the first after its options or scratch
 *     address changed (e.g. a gbxtb_singlepoint call with a workspace in
 *     between), creates the plan's capture stream and instantiates its
 *     pass graphs: driver work that can take device memory.  Make one
 *     warm-up call per plan and options at set-up, before any stream
 *     capture; later calls with the same plan and options do none of this;
 *   - all calls share the one array, which keeps the last call's contents
 *     (the driver clears what it reads first): calls whose GPU work overlaps,
 *     on other streams or threads, race on it and must be serialised. */
GBXTB_API int gbxtb_singlepoint_noalloc(gbxtb_plan *plan, const gbxtb_options *opts,
                                        const double *positions_dev, double *energy_dev,
                                        double *charges_dev, double *gradient_dev, void *stream);

/* Measured FP64 FMA throughput of the current device in GFLOP/s (a short
 * microbenchmark, ~10 ms); used as the roofline denominator of the
 * FP64-bound kernels.  No counterpart in the reference. */
GBXTB_API int gbxtb_fp64_peak(double *gflops);

/* Measured FP64 tensor-core (warp-level m8n8k4 MMA) throughput of the
 * current device in GFLOP/s (a short microbenchmark): whether FP64 panel
 * updates would run faster as MMA than as FMA.  No counterpart in the
 * reference. */
GBXTB_API int gbxtb_fp64_mma_peak(double *gflops);

#ifdef __cplusplus
}
#endif

#endif /* GBXTB_H */
