"""Counting functions f(R0, R) and their derivatives df/dR."""
import math

import torch

KCN_D3 = 16.0


def exp_count(rc, r, kcn=KCN_D3):
    return 1.0 / (1.0 + torch.exp(-kcn * (rc / r - 1.0)))


def dexp_count(rc, r, kcn=KCN_D3):
    expterm = torch.exp(-kcn * (rc / r - 1.0))
    return (-kcn * rc * expterm) / (r * r * ((expterm + 1.0) ** 2))


def erf_count(rc, r, kcn=7.5):
    return 0.5 * (1.0 + torch.erf(-kcn * (r / rc - 1.0)))


def derf_count(rc, r, kcn=7.5):
    return -kcn / math.sqrt(math.pi) / rc * torch.exp(-(kcn ** 2) * (r / rc - 1.0) ** 2)


def gfn2_count(rc, r, kcn=10.0, ka=None):
    return exp_count(rc, r, kcn) * exp_count(rc + 2.0, r, kcn)


def dgfn2_count(rc, r, kcn=10.0):
    raise NotImplementedError
