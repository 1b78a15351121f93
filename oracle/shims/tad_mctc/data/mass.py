def ATOMIC_MASS(*args, **kwargs):  # noqa: N802
    raise NotImplementedError
