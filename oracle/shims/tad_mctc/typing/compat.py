from __future__ import annotations

import os
from typing import (  # noqa: F401
    Any, Callable, Generator, Literal, NoReturn, Protocol, Sequence, TypedDict,
    Union,
)

import torch

try:
    from typing import Self, TypeAlias, TypeGuard, override  # noqa: F401
except ImportError:  # pragma: no cover
    from typing_extensions import Self, TypeAlias, TypeGuard, override  # noqa: F401

Tensor = torch.Tensor
PathLike = Union[str, os.PathLike]
Size = Union[tuple[int, ...], torch.Size]
Sliceable = Union[list, tuple, Tensor]
TensorOrTensors = Union[Tensor, Sequence[Tensor]]
CountingFunction = Callable[..., Tensor]
DampingFunction = Callable[..., Tensor]
CNFunction = Callable[..., Tensor]
CNGradFunction = Callable[..., Tensor]

__all__ = [
    "Any", "Callable", "CountingFunction", "DampingFunction", "Generator",
    "PathLike", "Self", "Sequence", "Size", "Sliceable", "TensorOrTensors",
    "TypeAlias", "TypeGuard", "override", "CNFunction", "CNGradFunction",
    "Literal", "TypedDict", "NoReturn", "Protocol",
]
