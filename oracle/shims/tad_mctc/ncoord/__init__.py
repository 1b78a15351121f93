"""D3-type coordination number with exponential counting
(dxtb call sites: ``xtb/gfn1.py:62-64``, ``xtb/base.py:285``,
``calculators/types/analytical.py:202,214``).

CN_A = sum_{B != A, R_AB < cutoff} 1 / (1 + exp(-k1 (R0_AB / R_AB - 1)))
with R0_AB = Rcov_A + Rcov_B (D3 covalent radii scaled by 4/3), k1 = 16 and
a real-space cutoff of 25 bohr (Grimme et al., J. Chem. Phys. 132, 154104).
"""
from __future__ import annotations

import math

import torch

from ..batch import real_pairs
from ..data.radii import COV_D3
from . import count  # noqa: F401
from .count import derf_count, dexp_count, dgfn2_count, erf_count, exp_count, gfn2_count  # noqa: F401

KCN_D3 = 16.0
CUTOFF_D3 = 25.0

__all__ = ["cn_d3", "cn_d3_gradient", "cn_d4", "exp_count", "dexp_count", "erf_count",
           "derf_count", "gfn2_count", "dgfn2_count", "coordination_number"]


def _dist(positions):
    diff = positions.unsqueeze(-2) - positions.unsqueeze(-3)
    d2 = (diff * diff).sum(-1)
    eps = torch.finfo(positions.dtype).eps
    return torch.sqrt(torch.clamp(d2, min=eps)), diff


def cn_d3(numbers, positions, *, counting_function=exp_count, rcov=None, cutoff=None, **kwargs):
    if cutoff is None:
        cutoff = CUTOFF_D3
    if rcov is None:
        rcov = COV_D3(device=positions.device, dtype=positions.dtype)[numbers]
    mask = real_pairs(numbers, mask_diagonal=True)
    dist, _ = _dist(positions)
    mask = mask & (dist <= cutoff)
    r0 = rcov.unsqueeze(-1) + rcov.unsqueeze(-2)
    safe = torch.where(mask, dist, torch.ones_like(dist))
    cf = torch.where(mask, counting_function(r0, safe, **kwargs), torch.zeros_like(dist))
    return cf.sum(-1)


def cn_d3_gradient(numbers, positions, *, dcounting_function=dexp_count, rcov=None, cutoff=None, **kwargs):
    """dcndr[..., i, j, :] = d CN_i / d r_j for j != i."""
    if cutoff is None:
        cutoff = CUTOFF_D3
    if rcov is None:
        rcov = COV_D3(device=positions.device, dtype=positions.dtype)[numbers]
    mask = real_pairs(numbers, mask_diagonal=True)
    dist, diff = _dist(positions)
    mask = mask & (dist <= cutoff)
    r0 = rcov.unsqueeze(-1) + rcov.unsqueeze(-2)
    safe = torch.where(mask, dist, torch.ones_like(dist))
    dcf = torch.where(mask, dcounting_function(r0, safe, **kwargs), torch.zeros_like(dist))
    # diff[i, j] = r_i - r_j ; d R_ij / d r_j = -(r_i - r_j) / R_ij
    return -(dcf / safe).unsqueeze(-1) * diff


def cn_d4(*args, **kwargs):
    raise NotImplementedError("D4 coordination numbers are not needed for GFN1.")


def coordination_number(*args, **kwargs):
    raise NotImplementedError
