"""Version information (the shim mimics tad_mctc 0.7.0)."""
import torch

__version__ = "0.7.0"
__tversion__ = tuple(
    int("".join(ch for ch in part if ch.isdigit()) or 0)
    for part in torch.__version__.split("+")[0].split(".")[:3]
)
