"""Generate the golden fixtures of this directory by running the reference.

The reference (dxtb) is imported read-only from its source tree through
``oracle/reference_run.py`` (SAD guess, D3 excluded, x_atol = x_atol_max =
f_atol = 1e-10, maxiter 300, Fermi smearing at 300 K, autograd forces).  Run
in the development container:

    python tests/golden/make_golden.py [--quick]

Outputs (ragged arrays concatenated over molecules, ``offsets`` delimit them):

* ``reference_mols.npz``: the reference's own test geometries
  (``test/test_singlepoint/mols/*/coord``);
* ``synthetic.npz``: seeded synthetic CHNO molecules from
  ``dxtb_gb300.molgen`` (the 20-atom single-point molecule, molecules of the
  10-120-atom batch workload and of the perturbed 30-60-atom force workload);
* ``halogen.npz`` (``--halogen``): synthetic molecules with Br/I
  halogen-bond donors, with the reference's halogen-bond term alone as well.
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from dxtb_gb300 import molgen  # noqa: E402
from oracle import reference_run as rr  # noqa: E402

HERE = Path(__file__).resolve().parent
REF_MOLS = ["H2", "LiH", "H2O", "CH4", "SiH4", "NO2", "LYS_xao", "MB16_43_01", "C60"]


def _pack(records: list[dict], names: list[str], path: Path) -> None:
    offs = np.concatenate([[0], np.cumsum([len(r["numbers"]) for r in records])]).astype(np.int64)
    out = {
        "names": np.array(names),
        "offsets": offs,
        "numbers": np.concatenate([r["numbers"] for r in records]).astype(np.int64),
        "positions": np.concatenate([r["positions"] for r in records]),
        "charge": np.array([r.get("charge", 0.0) for r in records]),
        "energy": np.array([r["energy"] for r in records]),
        "scf_energy": np.array([r["scf"] for r in records]),
        "fenergy": np.array([r["fenergy"] for r in records]),
        "iterations": np.array([r["iterations"] for r in records]),
        "charges": np.concatenate([r["charges_atom"] for r in records]),
        "forces": np.concatenate([r["forces"] for r in records]),
    }
    np.savez_compressed(path, **out)
    print(f"wrote {path} ({path.stat().st_size} bytes, {len(records)} molecules)")


def run(numbers, positions, charge=0.0, label=""):
    t = time.time()
    r = rr.singlepoint(numbers, positions, chrg=charge, forces=True)
    r.update(numbers=np.asarray(numbers), positions=np.asarray(positions), charge=charge)
    print(f"  {label:28s} nat={len(numbers):4d} E={r['energy']:.10f} it={r['iterations']:3d} "
          f"{time.time() - t:6.1f}s", flush=True)
    return r


def main(quick: bool) -> None:
    if not rr.available():
        raise SystemExit("reference source tree not found")
    recs, names = [], []
    for name in REF_MOLS[: 5 if quick else None]:
        d = rr.REFERENCE_ROOT / "test" / "test_singlepoint" / "mols" / name
        num, pos = rr.read_coord(d / "coord")
        chg = float((d / ".CHRG").read_text().split()[0]) if (d / ".CHRG").exists() else 0.0
        recs.append(run(num, pos, chg, name))
        names.append(name)
    _pack(recs, names, HERE / "reference_mols.npz")

    recs, names = [], []
    num, pos = molgen.c1_single()[0]
    recs.append(run(num, pos, label="single-20"))
    names.append("single-20")
    batch = molgen.c2_batch(64)
    picked = [i for i, (n, _) in enumerate(batch) if len(n) <= 60][: 3 if quick else 10]
    for i in picked:
        num, pos = batch[i]
        recs.append(run(num, pos, label=f"batch-{i}"))
        names.append(f"batch-{i}")
    forces = molgen.c3_forces(16)
    for i in range(2 if quick else 6):
        num, pos = forces[i]
        recs.append(run(num, pos, label=f"forces-{i}"))
        names.append(f"forces-{i}")
    _pack(recs, names, HERE / "synthetic.npz")


def main_halogen() -> None:
    """``halogen.npz``: synthetic molecules with Br/I donors
    (``dxtb_gb300.molgen.halogenated``), with the reference's full single
    point (energy, charges, autograd forces) and its halogen-bond term alone
    (``xb_energy`` per molecule, ``xb_gradient`` per atom)."""
    if not rr.available():
        raise SystemExit("reference source tree not found")
    recs, names, xbe, xbg = [], [], [], []
    for i, (nat, nhal) in enumerate([(12, 1), (20, 2), (24, 2), (30, 3), (40, 2), (50, 4)]):
        num, pos = molgen.halogenated(nat, 9100 + i, nhal)
        recs.append(run(num, pos, label=f"halogen-{i}"))
        names.append(f"halogen-{i}")
        e, g = rr.halogen_energy(num, pos)
        xbe.append(float(e.sum()))
        xbg.append(g)
    _pack(recs, names, HERE / "halogen.npz")
    g = dict(np.load(HERE / "halogen.npz"))
    g["xb_energy"] = np.array(xbe)
    g["xb_gradient"] = np.concatenate(xbg)
    np.savez_compressed(HERE / "halogen.npz", **g)
    print("halogen-bond energies", xbe)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--halogen", action="store_true", help="only halogen.npz")
    a = ap.parse_args()
    if a.halogen:
        main_halogen()
    else:
        main(a.quick)
