"""Generate ``gfn1_params.json`` from the reference's GFN1 parameter file.

Run once in a checkout that has the reference source tree:

    python -m dxtb_gb300.data.make_params /path/to/dxtb/src

The GFN1-xTB model is defined by its published parameter set (Grimme,
Bannwarth, Shushkov, J. Chem. Theory Comput. 13, 1989 (2017)); the engine
must use exactly the values the reference uses, so they are extracted
verbatim from ``dxtb/_src/param/gfn1/gfn1-xtb.toml`` together with the
STO-nG expansion tables (Stewart, J. Chem. Phys. 52, 431 (1970)) stored in
``dxtb/_src/basis/sto-ng/sto-{1..6}g.npy``.  Only the entries GFN1 uses are
written.
"""
from __future__ import annotations

import json
import sys
import tomllib
from pathlib import Path

import numpy as np

from dxtb_gb300.elements import SYMBOLS

OUT = Path(__file__).resolve().parent / "gfn1_params.json"
LABEL2L = {"s": 0, "p": 1, "d": 2, "f": 3, "g": 4}


def sto_itype(n: int, l: int, ng: int) -> int:
    """Column of the STO-nG tables for principal/angular quantum numbers
    (layout of ``basis/slater.py:111-118``)."""
    itype = n + [0, 4, 7, 9, 10][l] - 1
    if n == 6 and ng == 6:
        itype = 15 + l
    return itype


def main(src: str) -> None:
    src = Path(src)
    toml = tomllib.loads((src / "dxtb/_src/param/gfn1/gfn1-xtb.toml").read_text())
    sto = [np.load(src / f"dxtb/_src/basis/sto-ng/sto-{n}g.npy") for n in range(1, 7)]

    xtb = toml["hamiltonian"]["xtb"]
    out = {
        "source": "GFN1-xTB parameter file of the reference (gfn1-xtb.toml) and its STO-nG tables",
        "kpol": xtb["kpol"],
        "enscale": xtb["enscale"],
        "shell": xtb["shell"],
        "kexp": toml["repulsion"]["effective"]["kexp"],
        "gexp": toml["charge"]["effective"]["gexp"],
        "average": toml["charge"]["effective"]["average"],
        "thirdorder_shell": toml["thirdorder"]["shell"],
        "halogen": {"damping": toml["halogen"]["classical"]["damping"],
                    "rscale": toml["halogen"]["classical"]["rscale"]},
        "kpair": {},
        "elements": {},
        "sto": {},
    }
    for key, val in xtb["kpair"].items():
        a, b = key.split("-")
        za, zb = SYMBOLS.index(a) + 1, SYMBOLS.index(b) + 1
        out["kpair"][f"{min(za, zb)}-{max(za, zb)}"] = val

    for z, sym in enumerate(SYMBOLS, start=1):
        el = toml["element"].get(sym)
        if el is None:
            continue
        shells = []
        seen = set()
        for i, label in enumerate(el["shells"]):
            n, l = int(label[0]), LABEL2L[label[-1]]
            ng = int(el["ngauss"][i])
            itype = sto_itype(n, l, ng)
            out["sto"].setdefault(f"{ng}-{itype}", sto[ng - 1][:, itype, :].tolist())
            shells.append({
                "n": n, "l": l, "ngauss": ng, "sto": f"{ng}-{itype}",
                "slater": el["slater"][i], "level": el["levels"][i],
                "refocc": el["refocc"][i], "shpoly": el["shpoly"][i],
                "kcn": el["kcn"][i], "lgam": el["lgam"][i],
                "valence": l not in seen,
            })
            seen.add(l)
        out["elements"][str(z)] = {
            "symbol": sym, "shells": shells, "gam": el["gam"], "gam3": el["gam3"],
            "zeff": el["zeff"], "arep": el["arep"], "en": el["en"], "xbond": el.get("xbond", 0.0),
        }
    OUT.write_text(json.dumps(out, indent=1, sort_keys=True))
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m dxtb_gb300.data.make_params /path/to/dxtb/src")
    main(sys.argv[1])
