"""Padding helpers (dxtb call sites: ``basis/indexhelper.py``,
``integral/driver/pytorch/impls/overlap.py:176-221``,
``components/classicals/repulsion/base.py:221``)."""
from __future__ import annotations

import torch

__all__ = ["pack", "deflate", "real_atoms", "real_pairs", "real_triples", "eye"]


def real_atoms(numbers: torch.Tensor) -> torch.Tensor:
    return numbers != 0


def real_pairs(numbers: torch.Tensor, mask_diagonal: bool = True) -> torch.Tensor:
    real = real_atoms(numbers)
    mask = real.unsqueeze(-2) * real.unsqueeze(-1)
    if mask_diagonal:
        n = numbers.shape[-1]
        mask = mask & ~torch.eye(n, dtype=torch.bool, device=numbers.device)
    return mask


def real_triples(numbers, mask_diagonal=True, mask_self=True):
    real = real_pairs(numbers, mask_diagonal=False)
    mask = real.unsqueeze(-3) * real.unsqueeze(-2) * real.unsqueeze(-1)
    if mask_diagonal:
        n = numbers.shape[-1]
        e = torch.eye(n, dtype=torch.bool, device=numbers.device)
        mask = mask & ~(e.unsqueeze(-1) | e.unsqueeze(-2) | e.unsqueeze(-3))
    return mask


def pack(tensors, axis: int = 0, value=0, size=None):
    """Stack tensors of different shapes, padding each dimension with ``value``."""
    if isinstance(tensors, torch.Tensor):
        return tensors
    tensors = list(tensors)
    if len(tensors) == 0:
        raise ValueError("nothing to pack")
    if size is None:
        size = [max(t.shape[d] for t in tensors) for d in range(tensors[0].ndim)]
    out = tensors[0].new_full((len(tensors), *size), value)
    for i, t in enumerate(tensors):
        out[(i, *[slice(0, s) for s in t.shape])] = t
    if axis != 0:
        out = out.movedim(0, axis)
    return out


def deflate(tensor: torch.Tensor, value=0, axis: int | None = None) -> torch.Tensor:
    """Remove trailing padding (slices made only of ``value``) from every
    dimension except ``axis``."""
    nd = tensor.ndim
    slices = []
    for d in range(nd):
        if axis is not None and d == (axis % nd):
            slices.append(slice(None))
            continue
        keep = _any_except(tensor != value, d)
        idx = torch.nonzero(keep).flatten()
        n = int(idx.max().item()) + 1 if idx.numel() > 0 else 0
        slices.append(slice(0, n))
    return tensor[tuple(slices)]


def _any_except(mask: torch.Tensor, d: int) -> torch.Tensor:
    m = mask.movedim(d, 0)
    return m.reshape(m.shape[0], -1).any(-1)


def eye(shape, value=1.0, device=None, dtype=None):
    n = shape[-1]
    e = torch.eye(n, device=device, dtype=dtype) * value
    return e.expand(*shape[:-1], n) if len(shape) > 1 else e
