"""Unit conversions, CODATA 2010 (Bohr radius 0.52917721092 Angstrom,
Hartree 27.21138505 eV = 4.35974434e-18 J, k_B = 1.3806488e-23 J/K).

The CODATA 2010 Hartree-to-eV factor is the one under which the reference
reproduces tblite's GFN1 SCF energies in ``test/test_scf/samples.py`` to
5e-11 Eh (H2, LiH, H2O, CH4, SiH4); the CODATA 2018 value misses them by a
uniform 4.4e-8 relative error.
"""
BOHR_IN_AA = 0.52917721092
AA2AU = 1.0 / BOHR_IN_AA
AU2AA = BOHR_IN_AA
HARTREE_IN_EV = 27.21138505
EV2AU = 1.0 / HARTREE_IN_EV
AU2EV = HARTREE_IN_EV
HARTREE_IN_J = 4.35974434e-18
KB_J = 1.3806488e-23
KELVIN2AU = KB_J / HARTREE_IN_J
AU2KELVIN = 1.0 / KELVIN2AU
AU2AA4AMU = 1.0
AU2KMMOL = 1.0
AU2RCM = 219474.6313708

from . import energy  # noqa: E402,F401
