"""Input checks used at ``calculators/types/energy.py:96-108``."""
import torch

__all__ = ["shape_checks", "content_checks", "deflatable_check"]


def shape_checks(numbers, positions, allow_batched=True):
    if positions.shape[:-1] != numbers.shape or positions.shape[-1] != 3:
        raise ValueError(
            f"Shape of positions ({positions.shape}) does not match numbers ({numbers.shape})."
        )
    if not allow_batched and numbers.ndim > 1:
        raise ValueError("Batched input not allowed.")
    return True


def content_checks(numbers, positions, max_element=86, allow_batched=True):
    if (numbers < 0).any() or (numbers > max_element).any():
        raise ValueError("Atomic number out of range.")
    return True


def deflatable_check(*args, **kwargs):
    return True
