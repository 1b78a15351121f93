"""Parameter tables of the engine versus the oracle's restatement."""
import numpy as np
import pytest

from dxtb_gb300 import params
from oracle import gfn1_oracle as go


def test_radii_tables_agree_with_oracle_and_shim():
    from importlib import import_module
    import sys
    from pathlib import Path

    shim = str(Path(go.__file__).resolve().parent / "shims")
    sys.path.insert(0, shim)
    try:
        radii = import_module("tad_mctc.data.radii")
        units = import_module("tad_mctc.units")
    finally:
        sys.path.remove(shim)
    assert tuple(radii._ATOMIC_RAD) == params.ATOMIC_RADII_AA == tuple(go._ATOMIC_RAD)
    assert tuple(radii._COV_D3) == params.COV_D3_AA == tuple(go._COV_D3)
    assert units.EV2AU == params.EV2AU == go.EV2AU
    assert units.KELVIN2AU == params.KELVIN2AU == go.KELVIN2AU


@pytest.mark.parametrize("z", list(range(1, 87)))
def test_contracted_shells_agree_with_oracle(z):
    a = params.contracted_shells(z)
    b = go.element_basis(z)
    assert len(a) == len(b)
    for sa, sb in zip(a, b):
        assert sa["l"] == sb["l"]
        assert np.allclose(sa["alpha"], sb["alpha"], rtol=1e-15, atol=0)
        assert np.allclose(sa["coeff"], sb["coeff"], rtol=1e-14, atol=0)


def test_tables_layout():
    t = params.tables()
    assert t.elem_data.shape == (params.MAX_Z + 1, params.ELEM_DOUBLES)
    assert t.shell_data.shape[1] == params.SHELL_DOUBLES
    assert (t.shell_int[:, 1] <= params.MAX_PRIM).all()
    assert (t.shell_int[:, 0] <= 2).all()
    # hydrogen: 1s (4 primitives), 2s orthogonalised (3 + 4 primitives)
    h0, hn = t.elem_shell0[1], t.elem_nshell[1]
    assert hn == 2 and t.shell_int[h0, 1] == 4 and t.shell_int[h0 + 1, 1] == 7
    assert t.shell_int[h0 + 1, 2] == 0  # non-valence
    assert np.allclose(t.kpair, t.kpair.T)
    assert t.globals[11] == 2.0


def test_orthogonalised_hydrogen_2s():
    sh = params.contracted_shells(1)
    s = params._s_self_overlap(sh[0]["alpha"], sh[0]["coeff"], sh[1]["alpha"], sh[1]["coeff"])
    n = params._s_self_overlap(sh[1]["alpha"], sh[1]["coeff"], sh[1]["alpha"], sh[1]["coeff"])
    # residual overlap reflects the 1e-10 normalisation of the tabulated 1s contraction
    assert abs(s) < 1e-8 and abs(n - 1.0) < 1e-14
