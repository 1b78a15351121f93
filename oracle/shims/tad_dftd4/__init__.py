"""Import-time stand-in for tad-dftd4 0.8.0 (GFN2 only).  TEST INFRASTRUCTURE ONLY."""
from . import defaults  # noqa: F401


class Param(dict):
    pass


def __getattr__(name):
    from _missing import Missing

    return Missing(f"tad_dftd4.{name}")
