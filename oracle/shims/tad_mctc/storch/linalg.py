"""Generalised symmetric eigenproblem (dxtb call site:
``scf/unrolling/base.py:141-175``).

``eighb(a, b, is_posdef=True, factor, broadening_method)`` solves
A C = B C diag(w) by Cholesky reduction: B = L L^T, A' = L^-1 A L^-T,
A' = U diag(w) U^T, C = L^-T U.  Eigenvalues ascend.  When gradients are
required the standard-eigenproblem backward uses Lorentzian broadening of the
eigenvalue differences, d -> d / (d^2 + factor), which keeps the backward
finite for degenerate eigenvalues (the "lorn" method named at the call site).
"""
from __future__ import annotations

import torch


class _EighLorentz(torch.autograd.Function):
    @staticmethod
    def forward(ctx, a, factor):
        w, u = torch.linalg.eigh(a)
        ctx.save_for_backward(w, u)
        ctx.factor = factor
        return w, u

    @staticmethod
    def backward(ctx, w_bar, u_bar):
        w, u = ctx.saved_tensors
        ut = u.transpose(-2, -1)
        inner = torch.zeros_like(u)
        if w_bar is not None:
            inner = inner + torch.diag_embed(w_bar)
        if u_bar is not None:
            d = w.unsqueeze(-2) - w.unsqueeze(-1)  # d[i, j] = w_j - w_i
            f = d / (d * d + ctx.factor)
            inner = inner + f * (ut @ u_bar)
        a_bar = u @ inner @ ut
        a_bar = 0.5 * (a_bar + a_bar.transpose(-2, -1))
        return a_bar, None


def eighb(a, b=None, is_posdef=True, factor=None, broadening_method=None, **_):
    if factor is None:
        factor = torch.finfo(a.dtype).eps ** 0.5
    if b is None:
        if broadening_method is None:
            return torch.linalg.eigh(a)
        return _EighLorentz.apply(a, factor)
    lmat = torch.linalg.cholesky(b)
    linv = torch.linalg.inv(lmat)
    linv_t = linv.transpose(-2, -1)
    a_red = linv @ a @ linv_t
    a_red = 0.5 * (a_red + a_red.transpose(-2, -1))
    if broadening_method is None:
        w, u = torch.linalg.eigh(a_red)
    else:
        w, u = _EighLorentz.apply(a_red, factor)
    return w, linv_t @ u
