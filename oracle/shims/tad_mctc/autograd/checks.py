import torch


def is_batched(x=None) -> bool:
    try:
        return torch._C._functorch.is_batchedtensor(x)
    except Exception:  # pragma: no cover
        return False


def is_gradtracking(x=None) -> bool:
    try:
        return torch._C._functorch.is_gradtrackingtensor(x)
    except Exception:  # pragma: no cover
        return False
