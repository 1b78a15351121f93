"""Placeholder for attributes of unavailable third-party packages: attribute
access and calls succeed (so modules import); numeric use raises.  Test infrastructure only."""


class Missing:
    def __init__(self, name):
        self._name = name

    def __getattr__(self, item):
        if item.startswith("__"):
            raise AttributeError(item)
        return Missing(f"{self._name}.{item}")

    def __call__(self, *args, **kwargs):
        # Constructors run at import time for default arguments; the result
        # is another placeholder that fails when actually computed with.
        return Missing(f"{self._name}()")

    def __float__(self):
        raise NotImplementedError(f"{self._name} is not available in this container")

    def __mro_entries__(self, bases):
        return (object,)
