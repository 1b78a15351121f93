"""Minimal stand-in for the ``tad_mctc`` 0.7.0 API subset that dxtb imports.

TEST INFRASTRUCTURE ONLY.  This package exists so that the unmodified dxtb
sources can be imported in the development container (which has no network
and no ``tad_mctc`` wheel) to act as the parity oracle and to generate golden
fixtures.  Nothing in the product (``dxtb_gb300``) imports it.

Every function is written from the mathematics and from how dxtb calls it
(the call sites are cited per function); none of tad_mctc's own source was
available or used.  Numerical constants (covalent radii, unit conversions)
come from the published literature cited in ``data/radii.py`` and
``units/__init__.py`` and are pinned by the reference's golden files
``test/test_hamiltonian/h0.npz`` and ``grad_no_overlap.npz``.
"""
from . import (  # noqa: F401
    _version,
    autograd,
    batch,
    convert,
    data,
    exceptions,
    io,
    math,
    molecule,
    ncoord,
    storch,
    typing,
    units,
)
from ._version import __tversion__, __version__  # noqa: F401
