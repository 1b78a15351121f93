def is_linear(*args, **kwargs):  # pragma: no cover
    raise NotImplementedError
