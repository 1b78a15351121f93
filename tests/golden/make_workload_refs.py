"""Reference results for the full synthetic workloads, computed by the
reference itself (through ``oracle/reference_run.py``) in the development
container:

* ``workload_batch_ref.npz``: all 512 molecules of the 10-120-atom batch
  workload: energy, atomic charges, SCF iterations, convergence flag;
* ``workload_forces_ref.npz``: all 256 molecules of the perturbed 30-60-atom
  force workload: energy, charges, autograd forces (the reference's default
  ``get_forces``) and its analytical-gradient forces (``forces_analytical``).

Positions are not stored; they are regenerated from ``dxtb_gb300.molgen``
(seeded) and checked against the stored atom counts and a coordinate
checksum.

    python tests/golden/make_workload_refs.py [--procs 8] [--only batch|forces]
"""
from __future__ import annotations

import argparse
import multiprocessing as mp
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
HERE = Path(__file__).resolve().parent


def _work(args):
    kind, idx, forces = args
    sys.path.insert(0, str(ROOT))
    import torch

    torch.set_num_threads(1)
    from dxtb_gb300 import molgen
    from oracle import reference_run as rr

    mols = molgen.c2_batch(512) if kind == "batch" else molgen.c3_forces(256)
    num, pos = mols[idx]
    t = time.time()
    r = rr.singlepoint(num, pos, forces=forces, analytical=forces)
    r["time"] = time.time() - t
    r["natom"] = len(num)
    r["checksum"] = float(np.sum(pos * np.arange(1, pos.size + 1).reshape(pos.shape)))
    return idx, r


def run(kind: str, procs: int) -> None:
    n = 512 if kind == "batch" else 256
    forces = kind == "forces"
    ctx = mp.get_context("spawn")
    res = {}
    t0 = time.time()
    with ctx.Pool(procs) as pool:
        for i, r in pool.imap_unordered(_work, [(kind, i, forces) for i in range(n)]):
            res[i] = r
            if len(res) % 32 == 0:
                print(f"{kind}: {len(res)}/{n} done, {time.time() - t0:.0f}s", flush=True)
    order = range(n)
    out = {
        "natom": np.array([res[i]["natom"] for i in order]),
        "checksum": np.array([res[i]["checksum"] for i in order]),
        "energy": np.array([res[i]["energy"] for i in order]),
        "iterations": np.array([res[i]["iterations"] for i in order]),
        "charges": np.concatenate([res[i]["charges_atom"] for i in order]),
        "cpu_seconds": np.array([res[i]["time"] for i in order]),
    }
    out["converged"] = np.array([res[i]["converged"] for i in order])
    if forces:
        out["forces"] = np.concatenate([res[i]["forces"] for i in order])
        out["forces_analytical"] = np.concatenate([res[i]["forces_analytical"] for i in order])
    path = HERE / f"workload_{kind}_ref.npz"
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes) in {time.time() - t0:.0f}s")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--procs", type=int, default=8)
    ap.add_argument("--only", choices=["batch", "forces"], default=None)
    a = ap.parse_args()
    for kind in ("forces", "batch"):
        if a.only in (None, kind):
            run(kind, a.procs)
