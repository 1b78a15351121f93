"""Type aliases and the ``TensorLike`` base class used across dxtb."""
from __future__ import annotations

from .compat import *  # noqa: F401,F403
from .pytorch import *  # noqa: F401,F403
from .compat import (  # noqa: F401
    Callable, CountingFunction, DampingFunction, Generator, PathLike, Self,
    Sequence, Size, Sliceable, TensorOrTensors, TypeAlias, TypeGuard, override,
    CNFunction, CNGradFunction, Any, Literal, TypedDict, NoReturn, Protocol,
)
from .pytorch import DD, MockTensor, Molecule, Tensor, TensorLike, get_default_device, get_default_dtype  # noqa: F401

CNFunc = CNFunction


def __getattr__(name):
    # Remaining names in tad_mctc.typing are pure annotations.
    import typing as _t

    return _t.Any
