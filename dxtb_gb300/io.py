"""Structure input: Turbomole ``coord``, ``xyz`` and the ``.CHRG`` / ``.UHF``
files that travel with them, read on the host into the arrays the engine
takes (``numbers`` int64, ``positions`` float64 in bohr).

The reference reads these formats through tad-mctc 0.7.0 (``tad_mctc.io.
read``/``read_chrg``, used at ``test/test_singlepoint/test_energy.py:49-51``
and by its command line, ``cli/driver.py:118-270``).  Their layout is
public: a ``coord`` file has a ``$coord`` block of ``x y z element`` lines in
bohr (``$coord angs`` for Angstrom) closed by the next ``$`` keyword; an
``xyz`` file has the atom count, a comment line and ``element x y z`` lines
in Angstrom; ``.CHRG`` holds the total charge and ``.UHF`` the number of
unpaired electrons, each as the first token of the file.

    numbers, positions = read("mols/H2O/coord")
    calc = GFN1Calculator(torch.as_tensor(numbers), opts=...)
    energy = calc.get_energy(torch.as_tensor(positions, device="cuda"),
                             chrg=read_chrg("mols/H2O/.CHRG"))
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from .elements import symbol_to_number

__all__ = ["read", "read_coord", "read_xyz", "read_chrg", "read_uhf", "read_molecule", "BOHR_AA"]

BOHR_AA = 0.52917721092  # Angstrom per bohr (CODATA 2010, as the reference's units)


def _element(token: str, path, lineno: int) -> int:
    try:
        return symbol_to_number(token)
    except (KeyError, ValueError) as exc:
        raise ValueError(f"{path}:{lineno}: unknown element {token!r}") from exc


def read_coord(path) -> tuple[np.ndarray, np.ndarray]:
    """Turbomole ``$coord`` block: (numbers, positions in bohr)."""
    nums, pos = [], []
    scale = None
    for lineno, line in enumerate(Path(path).read_text().splitlines(), start=1):
        s = line.strip()
        if s.startswith("$"):
            if scale is not None:
                break  # the next keyword ends the block
            key = s.split()
            if key[0] == "$coord":
                unit = key[1].lower() if len(key) > 1 else "bohr"
                if unit.startswith("ang"):
                    scale = 1.0 / BOHR_AA
                elif unit in ("bohr", "au", "a.u."):
                    scale = 1.0
                else:
                    raise ValueError(f"{path}:{lineno}: unknown unit {key[1]!r} of $coord")
            continue
        if scale is None or not s:
            continue
        parts = s.split()
        if len(parts) < 4:
            raise ValueError(f"{path}:{lineno}: expected 'x y z element', got {s!r}")
        pos.append([float(x) * scale for x in parts[:3]])
        nums.append(_element(parts[3], path, lineno))
    if scale is None:
        raise ValueError(f"{path}: no $coord block")
    if not nums:
        raise ValueError(f"{path}: empty $coord block")
    return np.array(nums, dtype=np.int64), np.array(pos, dtype=np.float64)


def read_xyz(path) -> tuple[np.ndarray, np.ndarray]:
    """xyz file (Angstrom): (numbers, positions in bohr).  The first
    structure of a multi-structure file."""
    lines = Path(path).read_text().splitlines()
    if not lines:
        raise ValueError(f"{path}: empty file")
    try:
        nat = int(lines[0].split()[0])
    except (IndexError, ValueError) as exc:
        raise ValueError(f"{path}:1: expected the number of atoms") from exc
    if nat < 1 or len(lines) < 2 + nat:
        raise ValueError(f"{path}: {nat} atoms announced, {max(0, len(lines) - 2)} lines follow")
    nums, pos = [], []
    for lineno in range(3, 3 + nat):
        parts = lines[lineno - 1].split()
        if len(parts) < 4:
            raise ValueError(f"{path}:{lineno}: expected 'element x y z'")
        nums.append(_element(parts[0], path, lineno))
        pos.append([float(x) / BOHR_AA for x in parts[1:4]])
    return np.array(nums, dtype=np.int64), np.array(pos, dtype=np.float64)


def read(path, ftype: str | None = None) -> tuple[np.ndarray, np.ndarray]:
    """(numbers, positions in bohr) of a ``coord`` or ``xyz`` file; the type
    comes from ``ftype`` or the file name (``*.xyz``, ``coord``, ``*.coord``,
    ``*.tmol``)."""
    p = Path(path)
    kind = (ftype or "").lower()
    if not kind:
        if p.suffix.lower() == ".xyz":
            kind = "xyz"
        elif p.name == "coord" or p.suffix.lower() in (".coord", ".tmol"):
            kind = "coord"
        else:
            raise ValueError(f"{path}: cannot tell the format from the name; pass ftype='xyz' or 'coord'")
    if kind == "xyz":
        return read_xyz(p)
    if kind in ("coord", "tmol", "turbomole"):
        return read_coord(p)
    raise ValueError(f"unknown structure format {ftype!r}")


def _first_number(path, kind: type):
    tokens = Path(path).read_text().split()
    if not tokens:
        raise ValueError(f"{path}: empty file")
    try:
        return kind(float(tokens[0])) if kind is int else kind(tokens[0])
    except ValueError as exc:
        raise ValueError(f"{path}: expected a number, got {tokens[0]!r}") from exc


def read_chrg(path) -> float:
    """Total charge from a ``.CHRG`` file."""
    return _first_number(path, float)


def read_uhf(path) -> int:
    """Number of unpaired electrons from a ``.UHF`` file."""
    return _first_number(path, int)


def read_molecule(path) -> dict:
    """A structure file and the ``.CHRG`` / ``.UHF`` files beside it:
    ``{"numbers", "positions", "charge", "uhf"}`` (charge 0 and uhf None
    when the files are absent)."""
    p = Path(path)
    numbers, positions = read(p)
    chrg = p.parent / ".CHRG"
    uhf = p.parent / ".UHF"
    return {"numbers": numbers, "positions": positions,
            "charge": read_chrg(chrg) if chrg.exists() else 0.0,
            "uhf": read_uhf(uhf) if uhf.exists() else None}
