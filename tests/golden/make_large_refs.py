"""Convergence of the reference on molecules of the large-molecule workload
(``dxtb_gb300.molgen.c5_large``, 1000-2000 atoms), written to
``tests/golden/large_ref.json``.

The reference itself (``oracle/reference_run.py``, energy only, its Anderson
mixer, maxiter 300, x_atol = x_atol_max = 1e-10) is run on the chosen
molecules in the development container; each takes tens of minutes on
8 cores.  The record holds the atom count, the basis size, whether the SCF
converged, its iteration count and the energy it returned.

    python tests/golden/make_large_refs.py 7 8
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from dxtb_gb300 import molgen, params  # noqa: E402
from oracle import reference_run as rr  # noqa: E402

OUT = Path(__file__).resolve().parent / "large_ref.json"


def main(indices: list[int]) -> None:
    if not rr.available():
        raise SystemExit("reference source tree not found")
    mols = molgen.c5_large(16)
    raw = params.raw()["elements"]
    out = json.loads(OUT.read_text()) if OUT.exists() else {}
    for k in indices:
        num, pos = mols[k]
        t = time.time()
        r = rr.singlepoint(num, pos, forces=False)
        out[str(k)] = {"natom": int(len(num)),
                       "nao": int(sum(2 * s["l"] + 1 for z in num for s in raw[str(int(z))]["shells"])),
                       "converged": bool(r["converged"]), "iterations": int(r["iterations"]),
                       "energy": float(r["energy"]), "seconds": round(time.time() - t, 1)}
        print(k, out[str(k)], flush=True)
        OUT.write_text(json.dumps(out, indent=1, sort_keys=True))


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [7, 8])
