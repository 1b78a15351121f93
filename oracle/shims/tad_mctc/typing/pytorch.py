"""``TensorLike``: base for dxtb containers that own tensors and carry a
device/dtype (``basis/indexhelper.py:122``, ``components/base.py:35-81``)."""
from __future__ import annotations

import copy
from typing import Any, TypedDict

import torch

Tensor = torch.Tensor


class DD(TypedDict):
    device: Any
    dtype: Any


class Molecule(TypedDict):
    numbers: Tensor
    positions: Tensor


class MockTensor(torch.Tensor):
    pass


def get_default_device():
    return torch.tensor(0.0).device


def get_default_dtype():
    return torch.get_default_dtype()


class TensorLike:
    __slots__ = ["__device", "__dtype"]

    def __init__(self, device=None, dtype=None):
        self.__device = device if device is not None else get_default_device()
        self.__dtype = dtype if dtype is not None else get_default_dtype()

    @property
    def device(self):
        return self.__device

    @device.setter
    def device(self, *_):
        raise AttributeError("Move object to other device with '.to' method.")

    @property
    def dtype(self):
        return self.__dtype

    @dtype.setter
    def dtype(self, *_):
        raise AttributeError("Change dtype of object with '.type' method.")

    @property
    def dd(self) -> DD:
        return {"device": self.device, "dtype": self.dtype}

    @property
    def allowed_dtypes(self):
        return (torch.float16, torch.float32, torch.float64)

    def _attrs(self):
        names = []
        for cls in type(self).__mro__:
            for n in getattr(cls, "__slots__", ()):
                if n.startswith("__"):
                    continue
                names.append(n)
        if hasattr(self, "__dict__"):
            names.extend(self.__dict__.keys())
        return names

    def _clone_with(self, fn, device=None, dtype=None):
        new = copy.copy(self)
        for n in self._attrs():
            try:
                v = getattr(self, n)
            except AttributeError:
                continue
            if isinstance(v, torch.Tensor):
                try:
                    object.__setattr__(new, n, fn(v))
                except AttributeError:
                    pass
            elif isinstance(v, TensorLike):
                try:
                    object.__setattr__(new, n, v.to(device) if device is not None else v.type(dtype))
                except AttributeError:
                    pass
        if device is not None:
            new._TensorLike__device = device
        if dtype is not None:
            new._TensorLike__dtype = dtype
        return new

    def to(self, device):
        if device == self.device:
            return self
        return self._clone_with(lambda t: t.to(device), device=device)

    def type(self, dtype):
        if dtype == self.dtype:
            return self
        if dtype not in self.allowed_dtypes:
            raise ValueError(f"dtype {dtype} not allowed")
        return self._clone_with(
            lambda t: t.type(dtype) if t.is_floating_point() else t, dtype=dtype
        )


__all__ = ["DD", "MockTensor", "Molecule", "Tensor", "TensorLike",
           "get_default_device", "get_default_dtype"]
