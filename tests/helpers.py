"""Shared helpers for the test suite."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def load_golden(name: str) -> list[dict]:
    """Molecules of a golden npz file as dicts (ragged arrays split)."""
    g = np.load(GOLDEN / name)
    offs = g["offsets"]
    out = []
    for k in range(len(offs) - 1):
        a, b = offs[k], offs[k + 1]
        out.append({
            "name": str(g["names"][k]), "numbers": g["numbers"][a:b], "positions": g["positions"][a:b],
            "charge": float(g["charge"][k]), "energy": float(g["energy"][k]),
            "scf_energy": float(g["scf_energy"][k]), "iterations": int(g["iterations"][k]),
            "charges": g["charges"][a:b], "forces": g["forces"][a:b],
        })
    return out


def same_state(e1: float, e2: float) -> bool:
    """Two SCF results belong to the same self-consistent solution if their
    energies agree far better than the gap between distinct solutions
    (distinct solutions of the synthetic molecules differ by >1e-4 Eh)."""
    return abs(e1 - e2) < 1e-5
