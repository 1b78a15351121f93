"""The oracle against the reference project's own golden files and
known-answer values (only where the reference tree is present)."""
import numpy as np
import pytest

from oracle import gfn1_oracle as go
from oracle import reference_run as rr

pytestmark = pytest.mark.reference

MOLS = ["H2", "LiH", "H2O", "CH4", "SiH4"]
# SCF energies (no classical terms) of tblite, test/test_scf/samples.py:67-172
TBLITE_SCF = {"H2": -1.0585984032484, "LiH": -8.8306406116865e-01, "H2O": -5.8052489623704,
              "CH4": -4.3393059719255, "SiH4": -4.0384093532453}


def _mol(name):
    return rr.read_coord(rr.REFERENCE_ROOT / "test" / "test_singlepoint" / "mols" / name / "coord")


@pytest.mark.parametrize("name", MOLS)
def test_overlap_and_h0_golden(name):
    num, pos = _mol(name)
    s_ref = np.load(rr.REFERENCE_ROOT / "test/test_overlap/overlap.npz")[name.lower()]
    h_ref = np.load(rr.REFERENCE_ROOT / "test/test_hamiltonian/h0.npz")[name.lower()]
    b = go.Basis(num)
    s = go.overlap(b, pos)
    h = go.core_hamiltonian(b, pos, s, go.coordination_number(num, pos)).h0
    # golden files are float32
    assert np.abs(s - s_ref.reshape(s.shape)).max() < 5e-7
    assert np.abs(h - h_ref).max() < 5e-7


@pytest.mark.parametrize("name", MOLS)
def test_scf_energy_tblite(name):
    num, pos = _mol(name)
    r = go.singlepoint(num, pos, forces=False)
    e_scf = r.e_h0 + r.e_es2 + r.e_es3
    assert abs(e_scf - TBLITE_SCF[name]) < 1e-9


@pytest.mark.parametrize("name", ["h", "c", "rn"])
def test_single_atom_h0(name):
    z = {"h": 1, "c": 6, "rn": 86}[name]
    h_ref = np.load(rr.REFERENCE_ROOT / "test/test_hamiltonian/h0.npz")[name]
    num = np.array([z])
    pos = np.zeros((1, 3))
    b = go.Basis(num)
    s = go.overlap(b, pos)
    h = go.core_hamiltonian(b, pos, s, go.coordination_number(num, pos)).h0
    assert np.abs(h - h_ref).max() < 5e-7


def test_fermi_matches_reference_function():
    """The oracle's Fermi occupations against the reference's own function
    on a spectrum with a small gap (wavefunction/filling.py:269-366)."""
    rr._setup_path()
    import torch
    from dxtb._src.wavefunction.filling import get_fermi_occupation

    rng = np.random.default_rng(3)
    emo = np.sort(rng.normal(scale=0.3, size=40))
    emo[19] = emo[20] - 2e-3
    kt = 300.0 * go.KELVIN2AU
    nab = np.array([20.0, 20.0])
    ref = get_fermi_occupation(torch.tensor(nab), torch.tensor(emo).expand(2, -1).clone(),
                               kt=torch.tensor(kt, dtype=torch.float64)).numpy()
    occ = go.fermi_occupation(emo, nab, kt)
    assert np.abs(occ - ref).max() < 1e-14
