"""GFN1-xTB parameter tables for the engine.

Reads ``data/gfn1_params.json`` (the reference's GFN1 parameter file, see
``data/make_params.py``) and builds the flat tables that ``gbxtb_ctx_create``
uploads:

* contracted Gaussian shells: STO-nG expansion with alpha = alpha_sto *
  zeta^2 and primitive normalisation (2a/pi)^(3/4) (4a)^(l/2) / sqrt((2l-1)!!)
  (dxtb ``basis/slater.py:69-135``); a non-valence shell (GFN1 hydrogen 2s) is
  Gram-Schmidt orthogonalised to the shell before it and renormalised
  (``basis/ortho.py:74-110``, ``basis/bas.py:149-193``);
* element data: Hubbard parameter, third-order derivative, repulsion
  Z_eff and alpha, electronegativity, the covalent radius of the GFN1
  distance polynomial and the D3 covalent radius of the coordination number;
* self energies and their CN shift converted from eV to Hartree with the
  CODATA 2010 factor 27.21138505 eV/Eh.

Radii (Angstrom): GFN1 polynomial radii as used by the reference
(``xtb/base.py:138`` -> tad-mctc ``ATOMIC_RADII``) and D3 covalent radii
(Grimme et al., J. Chem. Phys. 132, 154104 (2010); Pyykko & Atsumi,
Chem. Eur. J. 15, 186 (2009), metals reduced by 10 %) scaled by 4/3.  Both
are pinned by the reference's golden overlap/H0/CN-gradient files.
"""
from __future__ import annotations

import json
import math
from dataclasses import dataclass
from functools import lru_cache
from pathlib import Path

import numpy as np

DATA = Path(__file__).resolve().parent / "data" / "gfn1_params.json"

BOHR_AA = 0.52917721092
AA2AU = 1.0 / BOHR_AA
EV2AU = 1.0 / 27.21138505
KELVIN2AU = 1.3806488e-23 / 4.35974434e-18

MAX_Z = 86
MAX_PRIM = 8
ELEM_DOUBLES = 8
SHELL_INTS = 4
SHELL_DOUBLES = 24
GLOBALS = 16

CN_STEEPNESS = 16.0
CN_CUTOFF = 25.0
REPULSION_CUTOFF = 25.0
INTEGRAL_CUTOFF = 50.0
XB_CUTOFF = 20.0  # halogen-bond pair cutoff in bohr (constants/xtb.py:33)
# halogen-bond donors and acceptors (components/classicals/halogen/hal.py:117-118)
XB_DONORS = (17, 35, 53, 85)
XB_ACCEPTORS = (7, 8, 15, 16)

ATOMIC_RADII_AA = (
    0.32, 0.37, 1.30, 0.99, 0.84, 0.75, 0.71, 0.64, 0.60, 0.62,
    1.60, 1.40, 1.24, 1.14, 1.09, 1.04, 1.00, 1.01,
    2.00, 1.74,
    1.59, 1.48, 1.44, 1.30, 1.29, 1.24, 1.18, 1.17, 1.22, 1.20,
    1.23, 1.20, 1.20, 1.18, 1.17, 1.16,
    2.15, 1.90,
    1.76, 1.64, 1.56, 1.46, 1.38, 1.36, 1.34, 1.30, 1.36, 1.40,
    1.42, 1.40, 1.40, 1.37, 1.32, 1.36,
    2.38, 2.06,
    1.94, 1.84, 1.90, 1.88, 1.86, 1.85, 1.83, 1.82, 1.81, 1.80, 1.79, 1.77, 1.77, 1.78, 1.74,
    1.64, 1.58, 1.50, 1.41, 1.36, 1.32, 1.30, 1.30, 1.32,
    1.44, 1.45, 1.50, 1.42, 1.48, 1.46,
)
COV_D3_AA = (
    0.32, 0.46, 1.20, 0.94, 0.77, 0.75, 0.71, 0.63, 0.64, 0.67,
    1.40, 1.25, 1.13, 1.04, 1.10, 1.02, 0.99, 0.96,
    1.76, 1.54,
    1.33, 1.22, 1.21, 1.10, 1.07, 1.04, 1.00, 0.99, 1.01, 1.09,
    1.12, 1.09, 1.15, 1.10, 1.14, 1.17,
    1.89, 1.67,
    1.47, 1.39, 1.32, 1.24, 1.15, 1.13, 1.13, 1.08, 1.15, 1.23,
    1.28, 1.26, 1.26, 1.23, 1.32, 1.31,
    2.09, 1.76,
    1.62, 1.47, 1.58, 1.57, 1.56, 1.55, 1.51, 1.52, 1.51, 1.50, 1.49, 1.49, 1.48, 1.53, 1.46,
    1.37, 1.31, 1.23, 1.18, 1.16, 1.11, 1.12, 1.13, 1.32,
    1.30, 1.30, 1.36, 1.31, 1.38, 1.42,
)

_DFACT = (1.0, 1.0, 3.0, 15.0, 105.0)


@lru_cache(maxsize=1)
def raw() -> dict:
    return json.loads(DATA.read_text())


def _s_self_overlap(a1, c1, a2, c2) -> float:
    return float(np.sum((math.pi / (a1[:, None] + a2[None, :])) ** 1.5 * np.outer(c1, c2)))


def contracted_shells(z: int) -> list[dict]:
    """Primitive exponents and normalised contraction coefficients of the
    shells of element ``z`` in parameter-file order."""
    par = raw()
    el = par["elements"][str(z)]
    out: list[dict] = []
    for sh in el["shells"]:
        c_sto, a_sto = (np.asarray(v, dtype=np.float64) for v in par["sto"][sh["sto"]])
        l = int(sh["l"])
        alpha = a_sto * float(sh["slater"]) ** 2
        coeff = c_sto * (2.0 * alpha / math.pi) ** 0.75 * np.sqrt(4.0 * alpha) ** l / math.sqrt(_DFACT[l])
        if not sh["valence"]:
            prev = out[-1]
            ov = _s_self_overlap(prev["alpha"], prev["coeff"], alpha, coeff)
            alpha = np.concatenate([alpha, prev["alpha"]])
            coeff = np.concatenate([coeff, -ov * prev["coeff"]])
            coeff = coeff / math.sqrt(_s_self_overlap(alpha, coeff, alpha, coeff))
        out.append({"l": l, "valence": bool(sh["valence"]), "alpha": alpha, "coeff": coeff,
                    "level": float(sh["level"]), "kcn": float(sh["kcn"]),
                    "shpoly": float(sh["shpoly"]), "refocc": float(sh["refocc"]),
                    "lgam": float(sh["lgam"])})
    return out


@dataclass(frozen=True)
class Tables:
    elem_shell0: np.ndarray
    elem_nshell: np.ndarray
    elem_data: np.ndarray
    shell_int: np.ndarray
    shell_data: np.ndarray
    kpair: np.ndarray
    globals: np.ndarray


@lru_cache(maxsize=1)
def tables() -> Tables:
    par = raw()
    nz = MAX_Z + 1
    elem_shell0 = np.zeros(nz, dtype=np.int32)
    elem_nshell = np.zeros(nz, dtype=np.int32)
    elem_data = np.zeros((nz, ELEM_DOUBLES), dtype=np.float64)
    shell_int: list[list[int]] = []
    shell_data: list[np.ndarray] = []
    for z in range(1, nz):
        el = par["elements"].get(str(z))
        if el is None:
            continue
        elem_data[z] = [el["gam"], el["gam3"], el["zeff"], el["arep"], el["en"],
                        ATOMIC_RADII_AA[z - 1] * AA2AU, COV_D3_AA[z - 1] * (4.0 / 3.0) * AA2AU,
                        el.get("xbond", 0.0)]
        elem_shell0[z] = len(shell_int)
        shells = contracted_shells(z)
        elem_nshell[z] = len(shells)
        for sh in shells:
            npr = len(sh["alpha"])
            if npr > MAX_PRIM:
                raise ValueError(f"element {z}: {npr} primitives exceed {MAX_PRIM}")
            rec = np.zeros(SHELL_DOUBLES)
            rec[:npr] = sh["alpha"]
            rec[8:8 + npr] = sh["coeff"]
            rec[16] = sh["level"] * EV2AU
            rec[17] = sh["kcn"] * EV2AU
            rec[18] = sh["shpoly"]
            rec[19] = sh["refocc"]
            rec[20] = sh["lgam"]
            shell_int.append([sh["l"], npr, int(sh["valence"]), 0])
            shell_data.append(rec)
    kpair = np.ones((nz, nz), dtype=np.float64)
    for key, val in par["kpair"].items():
        a, b = (int(x) for x in key.split("-"))
        kpair[a, b] = kpair[b, a] = val
    sh = par["shell"]
    g = np.zeros(GLOBALS)
    g[:15] = [par["kpol"], par["enscale"], sh["ss"], sh["pp"], sh["dd"], sh["sp"], par["kexp"],
              CN_STEEPNESS, CN_CUTOFF, REPULSION_CUTOFF, INTEGRAL_CUTOFF, par["gexp"],
              par["halogen"]["damping"], par["halogen"]["rscale"], XB_CUTOFF]
    return Tables(
        elem_shell0=elem_shell0, elem_nshell=elem_nshell, elem_data=np.ascontiguousarray(elem_data),
        shell_int=np.ascontiguousarray(np.asarray(shell_int, dtype=np.int32)),
        shell_data=np.ascontiguousarray(np.asarray(shell_data)),
        kpair=np.ascontiguousarray(kpair), globals=g,
    )


def reference_electrons(numbers) -> float:
    """Sum of reference shell occupations (valence electrons of a neutral
    molecule)."""
    par = raw()
    return float(sum(sum(s["refocc"] for s in par["elements"][str(int(z))]["shells"]) for z in numbers))
