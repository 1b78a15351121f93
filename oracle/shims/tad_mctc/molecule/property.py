def inertia_moment(*args, **kwargs):  # pragma: no cover
    raise NotImplementedError


def positions_rel_com(*args, **kwargs):  # pragma: no cover
    raise NotImplementedError
