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


def restart_energy(numbers, positions, v_orbital):
    """Oracle SCF (the engine's Broyden loop in numpy) restarted from an
    orbital potential: (converged, iterations, energy).  A state that is a
    fixed point of the reference's equations converges at once and keeps
    its energy."""
    from oracle import gfn1_oracle as go

    r = go.singlepoint(numbers, positions, mixer="broyden", v_init=v_orbital, forces=False, maxiter=30)
    return bool(r.converged), int(r.iterations), float(r.energy)


def fd_force_component(numbers, positions, atom, axis, v_orbital, h=2e-4):
    """Five-point central difference (truncation error O(h^4)) of the oracle
    energy: the force component -dE/dR[atom, axis].  Every displaced SCF
    starts from the converged orbital potential of the undisplaced geometry,
    so that it stays on the same SCF solution (molecules with several
    solutions would otherwise mix branches), and is converged to 1e-12 with
    the electron count solved to 1e-13: at the reference's sqrt(eps) Fermi
    tolerance the energy carries ~5e-9 Eh of noise."""
    from oracle import gfn1_oracle as go

    e = {}
    for st in (-2, -1, 1, 2):
        p = np.array(positions, dtype=np.float64, copy=True)
        p[atom, axis] += st * h
        r = go.singlepoint(numbers, p, mixer="broyden", forces=False, fermi_thr=1e-13, v_init=v_orbital,
                           x_atol=1e-12, x_atol_max=1e-12, maxiter=200)
        if not r.converged:
            return float("nan")
        e[st] = r.energy
    return -(8.0 * (e[1] - e[-1]) - (e[2] - e[-2])) / (12.0 * h)


def _star(args):
    fn, a = args
    return fn(*a)


def oracle_map(fn, jobs):
    """Run oracle jobs on all host cores (spawned workers, one BLAS thread
    each; spawned, so that no worker inherits the parent's CUDA context)."""
    import multiprocessing as mp
    import os

    jobs = list(jobs)
    if len(jobs) <= 1:
        return [fn(*a) for a in jobs]
    for var in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ.setdefault(var, "1")
    nproc = min(len(jobs), os.cpu_count() or 1)
    with mp.get_context("spawn").Pool(nproc) as pool:
        return pool.map(_star, [(fn, a) for a in jobs], chunksize=1)
