from . import checks  # noqa: F401
