"""Conversion helpers (dxtb call sites: ``xtb/base.py:358``,
``integral/driver/pytorch/overlap.py:74``, many ``any_to_tensor`` calls)."""
from __future__ import annotations

import numpy as np
import torch

__all__ = ["any_to_tensor", "symmetrize", "tensor_to_numpy", "numpy_to_tensor", "str_to_device", "reshape_fortran"]


def any_to_tensor(x, device=None, dtype=None):
    if isinstance(x, torch.Tensor):
        return x.to(device=device if device is not None else x.device,
                    dtype=dtype if dtype is not None else x.dtype)
    if isinstance(x, (list, tuple)) and len(x) > 0 and isinstance(x[0], torch.Tensor):
        return torch.stack([any_to_tensor(v, device, dtype) for v in x])
    if isinstance(x, np.ndarray):
        return torch.from_numpy(x).to(device=device, dtype=dtype)
    if isinstance(x, str):
        x = float(x)
    if dtype is None:
        dtype = torch.get_default_dtype() if isinstance(x, float) else None
    return torch.tensor(x, device=device, dtype=dtype)


def symmetrize(x: torch.Tensor, force: bool = False) -> torch.Tensor:
    """Return (x + x^T)/2; raise if x is far from symmetric unless forced."""
    xt = x.transpose(-2, -1)
    if not force:
        atol = 100 * torch.finfo(x.dtype).eps if x.is_floating_point() else 0
        if not torch.allclose(x, xt, atol=max(atol, 1e-12), rtol=0):
            raise RuntimeError("Matrix appears to be not symmetric.")
    return 0.5 * (x + xt)


def tensor_to_numpy(x, dtype=np.float64):
    return x.detach().cpu().numpy().astype(dtype)


def numpy_to_tensor(x, device=None, dtype=None):
    return torch.from_numpy(x).to(device=device, dtype=dtype)


def str_to_device(s: str) -> torch.device:
    return torch.device(s)


def reshape_fortran(x: torch.Tensor, shape):
    if len(x.shape) > 0:
        x = x.permute(*reversed(range(len(x.shape))))
    return x.reshape(*reversed(shape)).permute(*reversed(range(len(shape))))
