"""Element data used by dxtb (``param/module/utils.py:363-566``,
``xtb/base.py:138``)."""
from . import pse, radii  # noqa: F401
from .radii import ATOMIC_RADII, COV_D3, VDW_D3  # noqa: F401
from .pse import PAULING  # noqa: F401
