"""Safe elementwise operations (dxtb call sites: ``xtb/base.py:297-303``,
``coulomb/secondorder.py:843``, ``coulomb/average.py:55``,
``repulsion/base.py:319``)."""
from __future__ import annotations

import torch

from . import linalg  # noqa: F401
from .linalg import eighb  # noqa: F401

__all__ = ["cdist", "divide", "sqrt", "reciprocal", "pow", "eighb", "linalg"]


def _eps(x: torch.Tensor) -> float:
    return torch.finfo(x.dtype).eps if x.is_floating_point() else 1e-16


def cdist(x: torch.Tensor, y: torch.Tensor | None = None, p: int = 2) -> torch.Tensor:
    """Euclidean distance matrix from explicit coordinate differences.

    Zero distances (same atom) stay exactly zero and have a finite gradient.
    """
    if y is None:
        y = x
    diff = x.unsqueeze(-2) - y.unsqueeze(-3)
    d2 = torch.sum(diff * diff, dim=-1)
    eps = _eps(x)
    return torch.where(d2 > eps, torch.sqrt(torch.clamp(d2, min=eps)), d2.new_zeros(()))


def divide(x, y, eps=None, **_):
    """x / y with a zero denominator replaced by machine epsilon."""
    y = torch.as_tensor(y, dtype=x.dtype if torch.is_tensor(x) else None)
    e = _eps(y) if eps is None else eps
    return x / torch.where(y == 0, torch.full_like(y, e), y)


def sqrt(x, eps=None, **_):
    """sqrt(x) clamped at machine epsilon (finite gradient at zero)."""
    e = _eps(x) if eps is None else eps
    return torch.sqrt(torch.clamp(x, min=e))


def reciprocal(x, eps=None, **_):
    """1/x with zero replaced by machine epsilon."""
    e = _eps(x) if eps is None else eps
    return 1.0 / torch.where(x == 0, torch.full_like(x, e), x)


def pow(x, exponent, eps=None, **_):  # noqa: A001
    """x**exponent with the base clamped at machine epsilon."""
    e = _eps(x) if eps is None else eps
    return torch.pow(torch.clamp(x, min=e), exponent)
