"""ctypes binding of ``libgbxtb.so`` (declarations in ``include/gbxtb.h``).

The CUDA engine is the only implementation: if the library is missing the
import fails loudly; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libgbxtb.so"

GBXTB_OK = 0
MOL_OK = 0
MOL_NOT_CONVERGED = 1
MOL_FERMI_FAIL = 2
MOL_CHOLESKY_FAIL = 4
MOL_NONFINITE = 8
MOL_RESTARTED = 16

EXPORTED = (
    "gbxtb_version", "gbxtb_last_error", "gbxtb_ctx_create", "gbxtb_ctx_destroy",
    "gbxtb_plan_create", "gbxtb_plan_destroy", "gbxtb_plan_sizes", "gbxtb_integrals",
    "gbxtb_singlepoint", "gbxtb_get_status", "gbxtb_get_shell_potential", "gbxtb_get_orbital_charges",
    "gbxtb_get_profile",
    "gbxtb_fp64_peak", "gbxtb_fp64_mma_peak", "gbxtb_get_fp32_passes", "gbxtb_singlepoint_noalloc",
    "gbxtb_pool_create", "gbxtb_pool_destroy", "gbxtb_pool_free_slots", "gbxtb_pool_admit",
    "gbxtb_pool_step_launch", "gbxtb_pool_step_finish", "gbxtb_pool_result", "gbxtb_pool_step_poll",
    "gbxtb_plan_autotune", "gbxtb_default_options", "gbxtb_forces", "gbxtb_pool_evict",
)

NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024  # GBXTB_NOALLOC_SCRATCH_BYTES

PROF_CLASSES = ("atoms", "shellpairs", "cholesky", "fock", "tridiag", "bisect", "fermi", "invit",
                "backtransform", "density", "mix", "forces")


class Params(C.Structure):
    _fields_ = [
        ("max_z", C.c_int32),
        ("n_shell_records", C.c_int32),
        ("elem_shell0", C.POINTER(C.c_int32)),
        ("elem_nshell", C.POINTER(C.c_int32)),
        ("elem_data", C.POINTER(C.c_double)),
        ("shell_int", C.POINTER(C.c_int32)),
        ("shell_data", C.POINTER(C.c_double)),
        ("kpair", C.POINTER(C.c_double)),
        ("globals", C.POINTER(C.c_double)),
    ]


class Options(C.Structure):
    _fields_ = [
        ("maxiter", C.c_int32),
        ("fermi_maxiter", C.c_int32),
        ("broyden_memory", C.c_int32),
        ("want_forces", C.c_int32),
        ("x_atol", C.c_double),
        ("x_atol_max", C.c_double),
        ("kt", C.c_double),
        ("broyden_alpha", C.c_double),
        ("profile", C.c_int32),
        ("mixed_precision", C.c_int32),
        ("mixer", C.c_int32),
        ("generations", C.c_int32),
        ("damp", C.c_double),
        ("damp_init", C.c_double),
        ("diagonal_offset", C.c_double),
        ("soft_start", C.c_int32),
        ("mix_guess", C.c_int32),
        ("damp_dynamic", C.c_int32),
        ("no_halogen", C.c_int32),
        ("damp_dynamic_factor", C.c_double),
        ("fermi_thresh", C.c_double),
        ("restart_at", C.c_int32),
        ("fp64_split", C.c_int32),
    ]


MIXER_BROYDEN = 0
MIXER_ANDERSON = 1
MIXER_SIMPLE = 2
MIXERS = {"broyden": MIXER_BROYDEN, "anderson": MIXER_ANDERSON, "simple": MIXER_SIMPLE}


def default_options() -> "Options":
    """Options filled by ``gbxtb_default_options`` (the reference's defaults)."""
    o = Options()
    load().gbxtb_default_options(C.byref(o))
    return o


class GbxtbError(RuntimeError):
    pass


_lib = None


def load() -> C.CDLL:
    """Load the engine library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise GbxtbError(
            f"{LIB_PATH.name} is not built; run `python -m dxtb_gb300.build` "
            "(the CUDA engine is required, there is no CPU fallback)"
        )
    lib = C.CDLL(str(LIB_PATH))
    vp = C.c_void_p
    lib.gbxtb_version.restype = C.c_int
    lib.gbxtb_default_options.argtypes = [C.POINTER(Options)]
    lib.gbxtb_default_options.restype = None
    lib.gbxtb_forces.argtypes = [vp, vp, vp, vp, C.c_size_t, vp]
    lib.gbxtb_forces.restype = C.c_int
    lib.gbxtb_last_error.restype = C.c_char_p
    lib.gbxtb_ctx_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    lib.gbxtb_ctx_destroy.argtypes = [vp]
    lib.gbxtb_ctx_destroy.restype = None
    lib.gbxtb_plan_create.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(vp),
                                      C.POINTER(C.c_size_t)]
    lib.gbxtb_plan_destroy.argtypes = [vp]
    lib.gbxtb_plan_destroy.restype = None
    lib.gbxtb_plan_sizes.argtypes = [vp, C.POINTER(C.c_int64)]
    lib.gbxtb_integrals.argtypes = [vp, vp, vp, vp, vp, C.c_size_t, vp]
    lib.gbxtb_singlepoint.argtypes = [vp, C.POINTER(Options), vp, vp, vp, vp, vp, C.c_size_t, vp]
    lib.gbxtb_get_status.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
    lib.gbxtb_get_shell_potential.argtypes = [vp, C.POINTER(C.c_double)]
    lib.gbxtb_get_orbital_charges.argtypes = [vp, C.POINTER(C.c_double)]
    lib.gbxtb_get_fp32_passes.argtypes = [vp, C.POINTER(C.c_int32)]
    lib.gbxtb_singlepoint_noalloc.argtypes = [vp, C.POINTER(Options), vp, vp, vp, vp, vp]
    i32p, f64p = C.POINTER(C.c_int32), C.POINTER(C.c_double)
    lib.gbxtb_pool_create.argtypes = [vp, C.POINTER(Options), C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.POINTER(vp), C.POINTER(C.c_size_t)]
    lib.gbxtb_pool_destroy.argtypes = [vp]
    lib.gbxtb_pool_destroy.restype = None
    lib.gbxtb_pool_free_slots.argtypes = [vp]
    lib.gbxtb_pool_admit.argtypes = [vp, C.c_int32, i32p, f64p, C.c_double, C.c_int32, i32p]
    lib.gbxtb_pool_step_launch.argtypes = [vp, vp]
    lib.gbxtb_pool_step_poll.argtypes = [vp]
    lib.gbxtb_pool_evict.argtypes = [vp, C.c_int32, vp]
    lib.gbxtb_pool_evict.restype = C.c_int
    lib.gbxtb_plan_autotune.argtypes = [vp, C.POINTER(Options), vp, vp, C.c_size_t, vp, C.POINTER(C.c_int32)]
    lib.gbxtb_pool_step_finish.argtypes = [vp, i32p, i32p, i32p]
    lib.gbxtb_pool_result.argtypes = [vp, C.c_int32, f64p, f64p, f64p, i32p, i32p]
    lib.gbxtb_fp64_peak.argtypes = [C.POINTER(C.c_double)]
    lib.gbxtb_fp64_peak.restype = C.c_int
    lib.gbxtb_fp64_mma_peak.argtypes = [C.POINTER(C.c_double)]
    lib.gbxtb_fp64_mma_peak.restype = C.c_int
    lib.gbxtb_get_profile.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
    for name in ("gbxtb_ctx_create", "gbxtb_plan_create", "gbxtb_plan_sizes", "gbxtb_integrals",
                 "gbxtb_singlepoint", "gbxtb_get_status", "gbxtb_get_shell_potential", "gbxtb_get_profile",
                 "gbxtb_get_orbital_charges", "gbxtb_get_fp32_passes", "gbxtb_singlepoint_noalloc", "gbxtb_pool_create",
                 "gbxtb_pool_free_slots", "gbxtb_pool_admit", "gbxtb_pool_step_launch",
                 "gbxtb_pool_step_finish", "gbxtb_pool_result", "gbxtb_pool_step_poll", "gbxtb_plan_autotune"):
        getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != GBXTB_OK:
        msg = load().gbxtb_last_error().decode(errors="replace")
        raise GbxtbError(f"gbxtb error {rc}: {msg}")


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))
