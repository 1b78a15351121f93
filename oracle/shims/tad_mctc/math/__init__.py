"""``einsum`` wrapper (accepts and ignores opt_einsum's ``optimize``)."""
import torch

__all__ = ["einsum"]


def einsum(*args, optimize=None, **kwargs):
    return torch.einsum(*args, **kwargs)
