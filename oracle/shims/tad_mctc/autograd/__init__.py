"""Autograd helpers (only ``jacrev``-style Jacobians are provided)."""
import torch

from . import checks  # noqa: F401


def jacrev(func, argnums=0, **kwargs):
    return torch.func.jacrev(func, argnums=argnums, **kwargs)


def jac(func, argnums=0, **kwargs):
    return torch.func.jacrev(func, argnums=argnums, **kwargs)


def hessian(func, inputs, argnums=0, **kwargs):
    return torch.func.hessian(func, argnums=argnums)(*inputs)


def dgradcheck(func, inputs, **kwargs):
    return torch.autograd.gradcheck(func, inputs, **kwargs)


def dgradgradcheck(func, inputs, **kwargs):
    return torch.autograd.gradgradcheck(func, inputs, **kwargs)
