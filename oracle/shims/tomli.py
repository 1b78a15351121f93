"""``tomli`` alias for the stdlib ``tomllib`` (dxtb imports tomli at
``loader/lazy/lazy_param.py:96``).  Test infrastructure only."""
from tomllib import *  # noqa: F401,F403
from tomllib import load, loads  # noqa: F401
