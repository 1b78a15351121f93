"""Run the unmodified dxtb reference (imported read-only from its source tree)
behind the ``oracle/shims`` stand-ins for its missing third-party packages.

TEST INFRASTRUCTURE ONLY: used in the development container to pin the
oracle and to generate the golden fixtures under ``tests/golden``.  The
reference tree is not present where the GPU tests run, so nothing on the
product path or in the GPU tests imports this module.

Options mirror the reference's own tight-gradient tests
(``test/test_singlepoint/test_grad_gfn1.py:106-109``):
``int_driver="dxtb"`` (the PyTorch McMurchie-Davidson driver,
``integral/driver/pytorch/impls/overlap.py:147-243``), ``scf_mode="full"``
with Anderson mixing (``scf/unrolling/default.py:71-401``), SAD guess
(``scf/guess.py:82-85``), D3 excluded (its data is not available),
``x_atol = x_atol_max = f_atol = 1e-10``, Fermi smearing at 300 K.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# The reference's source tree: $DXTB_REFERENCE_SRC, else a `reference/src`
# directory beside the repository's directory.
REFERENCE_SRC = Path(os.environ.get("DXTB_REFERENCE_SRC",
                                    Path(__file__).resolve().parents[2] / "reference" / "src"))
REFERENCE_ROOT = REFERENCE_SRC.parent


def available() -> bool:
    return (REFERENCE_SRC / "dxtb" / "__init__.py").exists()


def _setup_path() -> None:
    for p in (str(REFERENCE_SRC), str(HERE / "shims")):
        if p not in sys.path:
            sys.path.insert(0, p)


DEFAULT_OPTS = {
    "int_driver": "dxtb",
    "scf_mode": "full",
    "mixer": "anderson",
    "guess": "sad",
    "exclude": ["disp"],
    "x_atol": 1e-10,
    "x_atol_max": 1e-10,
    "f_atol": 1e-10,
    "maxiter": 300,
    "fermi_etemp": 300.0,
    "verbosity": 0,
}


def read_coord(path) -> tuple["np.ndarray", "np.ndarray"]:
    """Read a Turbomole ``$coord`` block (bohr)."""
    import numpy as np

    from dxtb_gb300.elements import symbol_to_number

    nums, pos = [], []
    on = False
    for line in open(path):
        if line.startswith("$coord"):
            on = True
            continue
        if line.startswith("$"):
            on = False
            continue
        if on and line.strip():
            x, y, z, s = line.split()[:4]
            pos.append([float(x), float(y), float(z)])
            nums.append(symbol_to_number(s))
    return np.array(nums, dtype=np.int64), np.array(pos, dtype=np.float64)


def singlepoint(numbers, positions, chrg: float = 0.0, spin=None, forces: bool = True, opts=None,
                analytical: bool = False) -> dict:
    """Energy (and autograd forces) of one molecule through the reference's
    ``GFN1Calculator`` (``calculators/types/energy.py:78-402``,
    ``autograd.py:82-201``); with ``analytical`` also the reference's
    analytical-gradient forces (``calculators/types/analytical.py:63-222``)."""
    _setup_path()
    import numpy as np
    import torch

    import dxtb

    o = dict(DEFAULT_OPTS)
    if opts:
        o.update(opts)
    num = torch.as_tensor(np.asarray(numbers), dtype=torch.int64)
    pos = torch.as_tensor(np.asarray(positions), dtype=torch.float64).clone()
    calc = dxtb.calculators.GFN1Calculator(num, opts=o, dtype=torch.float64)
    pos.requires_grad_(forces)
    res = calc.singlepoint(pos, chrg=chrg, spin=spin)
    # the reference counts V -> Q -> V passes: the first one plus at most
    # maxiter loop passes; reaching maxiter + 1 means it stopped unconverged
    # (its OutputHandler records the SCFConvergenceWarning instead of raising)
    converged = int(res.iter) <= int(o["maxiter"])
    total = res.total.sum(-1)
    out = {
        "energy": float(total.detach()),
        "scf": float(res.scf.sum(-1).detach()),
        "fenergy": float(res.fenergy.sum(-1).detach()),
        "iterations": int(res.iter),
        "converged": converged,
        "charges_atom": calc.ihelp.reduce_orbital_to_atom(res.charges.mono).detach().numpy().copy(),
        "emo": res.emo.detach().numpy().copy(),
    }
    if forces:
        (g,) = torch.autograd.grad(total, pos)
        out["forces"] = (-g).detach().numpy().copy()
    if analytical:
        calc2 = dxtb.calculators.GFN1Calculator(num, opts=o, dtype=torch.float64)
        pos2 = torch.as_tensor(np.asarray(positions), dtype=torch.float64).clone().requires_grad_(True)
        out["forces_analytical"] = calc2.forces_analytical(pos2, chrg=chrg, spin=spin).detach().numpy().copy()
    return out


def halogen_energy(numbers, positions) -> tuple["np.ndarray", "np.ndarray"]:
    """The reference's halogen-bond correction alone
    (``components/classicals/halogen/hal.py:168-364``): per-atom energies
    and the gradient of their sum (autograd), for a single molecule."""
    _setup_path()
    import numpy as np
    import torch

    from dxtb import GFN1_XTB, IndexHelper
    from dxtb._src.components.classicals import new_halogen

    num = torch.as_tensor(np.asarray(numbers), dtype=torch.int64)
    pos = torch.as_tensor(np.asarray(positions), dtype=torch.float64).clone().requires_grad_(True)
    xb = new_halogen(torch.unique(num), GFN1_XTB, dtype=torch.float64)
    if xb is None:
        return np.zeros(len(num)), np.zeros((len(num), 3))
    cache = xb.get_cache(num, IndexHelper.from_numbers(num, GFN1_XTB))
    e = xb.get_energy(pos, cache)
    (g,) = torch.autograd.grad(e.sum(), pos)
    return e.detach().numpy().copy(), g.numpy().copy()
