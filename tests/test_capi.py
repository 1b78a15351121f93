"""The C-ABI library loads and exports every symbol of include/gbxtb.h
(no device calls: this runs without a GPU)."""
import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def lib():
    from dxtb_gb300 import _lib, build

    build.build()
    return _lib.load()


def declared():
    text = (ROOT / "include" / "gbxtb.h").read_text()
    return sorted(set(re.findall(r"\b(gbxtb_\w+)\s*\(", text)))


def test_header_matches_binding():
    from dxtb_gb300 import _lib

    assert sorted(_lib.EXPORTED) == declared()


def test_exports(lib):
    for name in declared():
        assert hasattr(lib, name), name


def test_version_and_errors(lib):
    from dxtb_gb300 import _lib

    assert lib.gbxtb_version() == 1
    # argument errors are reported without touching a device
    assert lib.gbxtb_ctx_create(None, None) == _lib.GBXTB_OK - 1
    assert b"null" in lib.gbxtb_last_error()
    h = C.c_void_p()
    ws = C.c_size_t()
    assert lib.gbxtb_plan_create(None, 0, None, None, None, None, C.byref(h), C.byref(ws)) == -1
    assert lib.gbxtb_get_status(None, None, None) == -1


def test_null_arguments_of_every_entry_point(lib):
    """Each entry point refuses null handles and buffers with
    GBXTB_ERR_ARG (-1) and a message, before any device call."""
    from dxtb_gb300 import _lib

    opts = _lib.Options()
    h = C.c_void_p()
    n = C.c_size_t()
    i32 = C.c_int32()
    calls = {
        "gbxtb_integrals": lambda: lib.gbxtb_integrals(None, None, None, None, None, 0, None),
        "gbxtb_singlepoint": lambda: lib.gbxtb_singlepoint(None, None, None, None, None, None, None, 0, None),
        "gbxtb_singlepoint_noalloc": lambda: lib.gbxtb_singlepoint_noalloc(None, None, None, None, None, None,
                                                                           None),
        "gbxtb_plan_autotune": lambda: lib.gbxtb_plan_autotune(None, C.byref(opts), None, None, 0, None, None),
        "gbxtb_get_fp32_passes": lambda: lib.gbxtb_get_fp32_passes(None, None),
        "gbxtb_get_shell_potential": lambda: lib.gbxtb_get_shell_potential(None, None),
        "gbxtb_get_orbital_charges": lambda: lib.gbxtb_get_orbital_charges(None, None),
        "gbxtb_get_profile": lambda: lib.gbxtb_get_profile(None, None, None, None),
        "gbxtb_pool_create": lambda: lib.gbxtb_pool_create(None, C.byref(opts), 1, 1, 1, 1, C.byref(h),
                                                           C.byref(n)),
        "gbxtb_pool_admit": lambda: lib.gbxtb_pool_admit(None, 1, None, None, 0.0, -1, C.byref(i32)),
        "gbxtb_pool_step_launch": lambda: lib.gbxtb_pool_step_launch(None, None),
        "gbxtb_pool_result": lambda: lib.gbxtb_pool_result(None, 0, None, None, None, None, None),
        "gbxtb_forces": lambda: lib.gbxtb_forces(None, None, None, None, 0, None),
    }
    for name, call in calls.items():
        assert call() == _lib.GBXTB_OK - 1, name
        assert lib.gbxtb_last_error(), name


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """Without the built engine the package refuses to run: there is no CPU
    fallback."""
    from dxtb_gb300 import _lib

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", tmp_path / "libgbxtb.so")
    with pytest.raises(_lib.GbxtbError, match="no CPU fallback"):
        _lib.load()


def test_default_options_are_the_references(lib):
    """gbxtb_default_options: the reference's SCF defaults
    (constants/defaults.py, calculators/config/scf.py) with its Anderson
    mixer; the engine-only switches are off."""
    from dxtb_gb300 import _lib, params

    o = _lib.default_options()
    assert (o.maxiter, o.fermi_maxiter, o.want_forces, o.profile, o.mixed_precision) == (100, 200, 0, 0, 0)
    assert (o.x_atol, o.x_atol_max) == (1e-4, 1e-5)
    assert abs(o.kt - 300.0 * params.KELVIN2AU) < 1e-15
    assert o.mixer == _lib.MIXER_ANDERSON
    assert (o.generations, o.damp, o.damp_init, o.diagonal_offset) == (5, 0.5, 0.1, 0.01)
    assert (o.soft_start, o.mix_guess, o.damp_dynamic, o.damp_dynamic_factor) == (1, 1, 0, 0.99)
    assert o.fermi_thresh == 0.0


def test_invalid_options_are_refused_before_any_device_call(lib):
    """Out-of-range options fail with GBXTB_ERR_ARG and a message (the plan
    pointer is checked after the options, so no device is touched)."""
    from dxtb_gb300 import _lib

    e = C.c_double()
    bad = []
    for field, value in (("mixer", 7), ("generations", 0), ("generations", 29), ("broyden_memory", 0),
                         ("fermi_maxiter", 0), ("kt", 0.0), ("damp", float("nan")),
                         ("fermi_thresh", float("inf"))):
        o = _lib.default_options()
        if field == "broyden_memory":
            o.mixer = _lib.MIXER_BROYDEN
        if field == "damp":
            o.mixer = _lib.MIXER_SIMPLE
        setattr(o, field, value)
        rc = lib.gbxtb_singlepoint(C.c_void_p(1), C.byref(o), None, C.byref(e), None, None, None, 0, None)
        bad.append((field, rc, lib.gbxtb_last_error()))
    for field, rc, msg in bad:
        assert rc == -1 and msg, field
