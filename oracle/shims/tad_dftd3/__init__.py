"""Import-time stand-in for tad-dftd3 0.6.0.  TEST INFRASTRUCTURE ONLY.

The D3 reference C6 data is not available in this container, so the oracle
runs GFN1 with dispersion excluded (``opts={"exclude": ["disp"]}``); only the
default-parameter constants that dxtb reads while building its pydantic
parameter model (``param/dispersion.py:48-60``) are provided.
"""
from . import defaults  # noqa: F401


def __getattr__(name):
    from _missing import Missing

    return Missing(f"tad_dftd3.{name}")
