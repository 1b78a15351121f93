class Mol:  # pragma: no cover
    def __init__(self, *args, **kwargs):
        raise NotImplementedError
