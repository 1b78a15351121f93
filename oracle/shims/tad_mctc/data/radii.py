"""Atomic radii (bohr), index 0 is padding.

ATOMIC_RADII: the covalent radii used by the GFN1 distance polynomial
(``xtb/base.py:138``), in Angstrom in the table below and converted with
the CODATA 2018 Bohr radius.  COV_D3: D3 covalent radii (Grimme et al.,
J. Chem. Phys. 132, 154104 (2010), taken from Pyykko & Atsumi, Chem. Eur. J.
15, 186 (2009) with metal values reduced by 10 %) scaled by k2 = 4/3, used by
the exponential coordination number (``xtb/gfn1.py:62-64``).  Both tables are
pinned for H, Li, C, N, O, Si and S by the reference golden files
``test/test_hamiltonian/h0.npz`` and ``grad_no_overlap.npz``.
"""
import torch

from ..units import AA2AU

# Angstrom, Z = 1..86
_ATOMIC_RAD = [
    0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60, 0.62,
    1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01,
    2.00, 1.74,
    1.59, 1.48, 1.44, 1.30, 1.29, 1.24, 1.18, 1.17, 1.22, 1.20,
    1.23, 1.20, 1.20, 1.18, 1.17, 1.16,
    2.15, 1.90,
    1.76, 1.64, 1.56, 1.46, 1.38, 1.36, 1.34, 1.30, 1.36, 1.40,
    1.42, 1.40, 1.40, 1.37, 1.32, 1.36,
    2.38, 2.06,
    1.94, 1.84, 1.90, 1.88, 1.86, 1.85, 1.83, 1.82, 1.81, 1.80, 1.79, 1.77, 1.77, 1.78, 1.74,
    1.64, 1.58, 1.50, 1.41, 1.36, 1.32, 1.30, 1.30, 1.32,
    1.44, 1.45, 1.50, 1.42, 1.48, 1.46,
]

# Angstrom, Z = 1..86 (before the 4/3 scaling)
_COV_D3 = [
    0.32, 0.46, 1.20, 0.94, 0.77, 0.75, 0.71, 0.63, 0.64, 0.67,
    1.40, 1.25, 1.13, 1.04, 1.10, 1.02, 0.99, 0.96,
    1.76, 1.54,
    1.33, 1.22, 1.21, 1.10, 1.07, 1.04, 1.00, 0.99, 1.01, 1.09,
    1.12, 1.09, 1.15, 1.10, 1.14, 1.17,
    1.89, 1.67,
    1.47, 1.39, 1.32, 1.24, 1.15, 1.13, 1.13, 1.08, 1.15, 1.23,
    1.28, 1.26, 1.26, 1.23, 1.32, 1.31,
    2.09, 1.76,
    1.62, 1.47, 1.58, 1.57, 1.56, 1.55, 1.51, 1.52, 1.51, 1.50, 1.49, 1.49, 1.48, 1.53, 1.46,
    1.37, 1.31, 1.23, 1.18, 1.16, 1.11, 1.12, 1.13, 1.32,
    1.30, 1.30, 1.36, 1.31, 1.38, 1.42,
]


def ATOMIC_RADII(device=None, dtype=torch.double):  # noqa: N802
    return torch.tensor([0.0] + _ATOMIC_RAD, device=device, dtype=dtype) * AA2AU


def COV_D3(device=None, dtype=torch.double):  # noqa: N802
    return torch.tensor([0.0] + _COV_D3, device=device, dtype=dtype) * (4.0 / 3.0) * AA2AU


def VDW_D3(device=None, dtype=torch.double):  # noqa: N802
    raise NotImplementedError("D3 van-der-Waals radii are not needed for GFN1 without D3.")


def VDW_PAIRWISE(device=None, dtype=torch.double):  # noqa: N802
    raise NotImplementedError("D3 pairwise radii are not available (tad_dftd3 data missing).")
