"""Structure input (dxtb_gb300.io): Turbomole coord, xyz, .CHRG and .UHF,
the formats the reference reads with tad-mctc (test/test_singlepoint/
test_energy.py:49-51, cli/driver.py:118-270)."""
import numpy as np
import pytest

from dxtb_gb300 import io
from tests.helpers import GOLDEN, load_golden

COORD = """$coord
    0.00000000000000      0.00000000000000     -0.74288549752983      o
   -1.43472674945442      0.00000000000000      0.37144274876492      h
    1.43472674945442      0.00000000000000      0.37144274876492      H
$periodic 0
$end
"""

XYZ = """3
water
O    0.000000   0.000000  -0.393118
H   -0.759235   0.000000   0.196559
H    0.759235   0.000000   0.196559
"""


def test_coord_and_xyz(tmp_path):
    (tmp_path / "coord").write_text(COORD)
    num, pos = io.read(tmp_path / "coord")
    assert num.tolist() == [8, 1, 1] and pos.dtype == np.float64
    assert pos[1, 0] == pytest.approx(-1.43472674945442)
    (tmp_path / "w.xyz").write_text(XYZ)
    num2, pos2 = io.read(tmp_path / "w.xyz")
    assert num2.tolist() == [8, 1, 1]
    assert np.abs(pos2 - pos).max() < 1e-4  # the same water to the 6 digits of the file (Angstrom)
    (tmp_path / "a.coord").write_text(COORD.replace("$coord", "$coord angs"))
    _, pos3 = io.read(tmp_path / "a.coord")
    assert np.allclose(pos3 * io.BOHR_AA, pos)


def test_charge_and_spin_files(tmp_path):
    (tmp_path / "coord").write_text(COORD)
    (tmp_path / ".CHRG").write_text("1\n")
    (tmp_path / ".UHF").write_text("1\n")
    mol = io.read_molecule(tmp_path / "coord")
    assert mol["charge"] == 1.0 and mol["uhf"] == 1
    (tmp_path / ".UHF").unlink()
    assert io.read_molecule(tmp_path / "coord")["uhf"] is None


@pytest.mark.parametrize("text, name, msg", [
    ("$end\n", "coord", "no \\$coord block"),
    ("$coord\n 0 0 0 xx\n$end\n", "coord", "unknown element"),
    ("$coord\n 0 0\n$end\n", "coord", "expected 'x y z element'"),
    ("5\n\nH 0 0 0\n", "m.xyz", "5 atoms announced"),
    ("H\n", "m.xyz", "number of atoms"),
])
def test_malformed_files_raise(tmp_path, text, name, msg):
    (tmp_path / name).write_text(text)
    with pytest.raises(ValueError, match=msg):
        io.read(tmp_path / name)


def test_unknown_format_raises(tmp_path):
    (tmp_path / "mol.pdb").write_text("x")
    with pytest.raises(ValueError, match="cannot tell the format"):
        io.read(tmp_path / "mol.pdb")


@pytest.mark.reference
def test_reference_molecule_files():
    """The reference's own test molecules (test/test_singlepoint/mols/*):
    the reader gives the geometries and charges of the golden fixtures
    (tests/golden/reference_mols.npz), and NO2's xyz file its coord file."""
    from oracle import reference_run as rr

    base = rr.REFERENCE_ROOT / "test" / "test_singlepoint" / "mols"
    for mol in load_golden("reference_mols.npz"):
        d = base / mol["name"]
        m = io.read_molecule(d / "coord")
        assert np.array_equal(m["numbers"], mol["numbers"])
        assert np.array_equal(m["positions"], mol["positions"])
        assert m["charge"] == mol["charge"]
    n1, p1 = io.read(base / "NO2" / "coord")
    n2, p2 = io.read(base / "NO2" / "mol.xyz")
    assert np.array_equal(n1, n2) and np.abs(p1 - p2).max() < 1e-5
