"""GFN1-xTB single points (energy, charges, forces) on NVIDIA GB300.

``GFN1Calculator`` mirrors dxtb's calculator; the arithmetic runs in the
CUDA library ``libgbxtb.so`` built from ``csrc/`` (``python -m
dxtb_gb300.build``).
"""
from __future__ import annotations

__version__ = "0.1.0"

__all__ = ["GFN1Calculator", "SCFConvergenceWarning", "SCFConvergenceError", "build", "io"]


def __getattr__(name):
    if name in ("GFN1Calculator", "SCFConvergenceWarning", "SCFConvergenceError"):
        from . import calculator

        return getattr(calculator, name)
    if name == "build":
        from .build import build

        return build
    if name == "io":
        import importlib

        return importlib.import_module(f"{__name__}.io")
    raise AttributeError(name)
