"""The calculator's option dict (the reference's ``opts``,
calculators/config/main.py:86-156): options the engine honours reach the
C options, options it cannot honour raise instead of being dropped.  No
device is needed."""
import pytest

from dxtb_gb300 import _lib
from dxtb_gb300.calculator import engine_options, resolve_opts

BASE = {"exclude": ["disp"]}


def test_mixer_options_reach_the_engine():
    o = resolve_opts({**BASE, "mixer": "anderson", "damp": 0.3, "damp_init": 0.2, "damp_generations": 7,
                      "damp_diagonal_offset": None, "damp_soft_start": False, "mix_guess": False,
                      "damp_dynamic": True, "damp_dynamic_factor": 0.9, "fermi_thresh": 1e-12})
    e = engine_options(o, forces=True)
    assert e.mixer == _lib.MIXER_ANDERSON and e.want_forces == 1
    assert (e.damp, e.damp_init, e.generations) == (0.3, 0.2, 7)
    assert e.diagonal_offset < 0  # None: no rescaling
    assert (e.soft_start, e.mix_guess, e.damp_dynamic, e.damp_dynamic_factor) == (0, 0, 1, 0.9)
    assert e.fermi_thresh == 1e-12
    assert engine_options(resolve_opts({**BASE, "mixer": "simple"}), False).mixer == _lib.MIXER_SIMPLE
    assert engine_options(resolve_opts(BASE), False).mixer == _lib.MIXER_BROYDEN
    assert engine_options(resolve_opts(BASE), False).fermi_thresh == 0.0  # sqrt(eps)


@pytest.mark.parametrize("opts, err", [
    ({"mixer": "pulay"}, ValueError),
    ({"guess": "eeq"}, ValueError),
    ({"guess": "random"}, ValueError),
    ({"scp_mode": "charge"}, NotImplementedError),
    ({"scp_mode": "fock"}, NotImplementedError),
    ({"damp_generations": 0}, ValueError),
    ({"broyden_memory": 40}, ValueError),
    ({"no_such_option": 1}, ValueError),
    ({"exclude": []}, ValueError),
    ({"exclude": ["disp", "es3"]}, NotImplementedError),
    ({"exclude": ["disp", "rep"]}, NotImplementedError),
    ({"fp64_tridiag": "quad"}, ValueError),
])
def test_unsupported_options_raise(opts, err):
    with pytest.raises(err):
        resolve_opts({**BASE, **opts})


def test_options_without_numerical_effect_are_accepted():
    o = resolve_opts({**BASE, "scf_mode": "implicit", "int_driver": "pytorch", "batch_mode": 1,
                      "f_atol": 1e-6, "verbosity": 0})
    assert o["mixer"] == "broyden"


def test_halogen_bond_switch():
    assert engine_options(resolve_opts(BASE), False).no_halogen == 0
    assert engine_options(resolve_opts({"exclude": ["disp", "hal"]}), False).no_halogen == 1
    # GFN2-only terms are absent from GFN1 anyway
    assert engine_options(resolve_opts({"exclude": ["disp", "aes2", "d4sc"]}), False).no_halogen == 0


def test_fp64_tridiag_switch():
    """The arithmetic of the FP64 on-chip tridiagonalisation reaches the C
    options (0 auto, 1 native FP64, 2 double-float)."""
    assert engine_options(resolve_opts(BASE), False).fp64_split == 0
    assert engine_options(resolve_opts({**BASE, "fp64_tridiag": "native"}), False).fp64_split == 1
    assert engine_options(resolve_opts({**BASE, "fp64_tridiag": "df64"}), False).fp64_split == 2
