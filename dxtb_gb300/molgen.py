"""Seeded synthetic CHNO molecules.

Growth rule: heavy atoms C/N/O drawn with probabilities 0.70/0.15/0.15; the
first sits at the origin, each further heavy atom is bonded to a uniformly
chosen existing heavy atom at 2.8 bohr along a uniformly random direction and
rejected if it comes within 2.2 bohr of any atom.  Hydrogens are then placed
at 2.05 bohr from uniformly chosen heavy atoms (rejected if within 2.2 bohr of
any atom other than that heavy atom) until they make up half of the atoms;
if the valence-electron count (H 1, C 4, N 5, O 6) is odd one H is removed,
so every molecule is a neutral closed shell.  The seed of molecule ``i`` of
workload ``k`` is ``1000*k + i``.
"""
from __future__ import annotations

import numpy as np

VALENCE = {1: 1, 6: 4, 7: 5, 8: 6}
BOND_HEAVY = 2.8
BOND_H = 2.05
MIN_DIST = 2.2


def grow(natoms: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Return (numbers int64 (n,), positions float64 (n, 3) in bohr)."""
    if natoms < 2:
        raise ValueError("need at least two atoms")
    rng = np.random.Generator(np.random.PCG64(seed))
    n_heavy = (natoms + 1) // 2
    n_h = natoms - n_heavy
    zs = list(rng.choice(np.array([6, 7, 8]), size=n_heavy, p=[0.70, 0.15, 0.15]))
    pos = [np.zeros(3)]
    while len(pos) < n_heavy:
        anchor = int(rng.integers(len(pos)))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        cand = pos[anchor] + BOND_HEAVY * d
        if np.min(np.linalg.norm(np.asarray(pos) - cand, axis=1)) >= MIN_DIST - 1e-12:
            pos.append(cand)
    heavy = np.asarray(pos)
    hpos: list[np.ndarray] = []
    while len(hpos) < n_h:
        anchor = int(rng.integers(n_heavy))
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        cand = heavy[anchor] + BOND_H * d
        others = np.concatenate([np.delete(heavy, anchor, axis=0), np.asarray(hpos).reshape(-1, 3)])
        if others.shape[0] == 0 or np.min(np.linalg.norm(others - cand, axis=1)) >= MIN_DIST - 1e-12:
            hpos.append(cand)
    numbers = np.array(zs + [1] * n_h, dtype=np.int64)
    positions = np.concatenate([heavy, np.asarray(hpos).reshape(-1, 3)])
    if sum(VALENCE[int(z)] for z in numbers) % 2 == 1:
        numbers, positions = numbers[:-1], positions[:-1]
    return numbers, positions


def workload(config: int, count: int, nmin: int, nmax: int, perturb: float = 0.0,
             log_uniform: bool = False, shard: int = 0) -> list[tuple[np.ndarray, np.ndarray]]:
    """``count`` molecules for workload ``config``: atom counts uniform (or
    log-uniform) in [nmin, nmax] drawn from seed ``1000*config + 999``;
    positions optionally displaced by N(0, perturb) bohr.  ``shard`` > 0
    gives a further, disjoint set of the same distribution (seeds offset by
    ``10**6 * shard``), used to give every GPU its own molecules."""
    base = 10**6 * shard
    rng = np.random.Generator(np.random.PCG64(base + 1000 * config + 999))
    if log_uniform:
        sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax + 1), size=count)).astype(int)
        sizes = np.clip(sizes, nmin, nmax)
    else:
        sizes = rng.integers(nmin, nmax + 1, size=count)
    mols = []
    for i, n in enumerate(sizes):
        num, pos = grow(int(n), base + 1000 * config + i)
        if perturb > 0.0:
            prng = np.random.Generator(np.random.PCG64(base + 1000 * config + i + 500_000))
            pos = pos + prng.normal(scale=perturb, size=pos.shape)
        mols.append((num, pos))
    return mols


# Workloads, sized as in the benchmark description.
def c1_single() -> list:
    """One neutral 20-atom molecule."""
    return [grow(20, 1000 * 0 + 0)]


def c2_batch(count: int = 512, shard: int = 0) -> list:
    """Molecules of 10-120 atoms."""
    return workload(1, count, 10, 120, shard=shard)


def c3_forces(count: int = 256) -> list:
    """Molecules of 30-60 atoms with N(0, 0.05 bohr) displacements."""
    return workload(2, count, 30, 60, perturb=0.05)


def c4_stream(count: int) -> list:
    """Log-uniform 8-400 atoms (served stream)."""
    return workload(3, count, 8, 400, log_uniform=True)


def c5_large(count: int = 16) -> list:
    """Molecules of 1000-2000 atoms."""
    return workload(4, count, 1000, 2000)


# Halogen donors for the halogen-bond molecules and their bond length to a
# heavy atom (bohr).
HALOGEN_BOND = {35: 3.65, 53: 4.05}


def halogenated(natoms: int, seed: int, nhal: int = 2) -> tuple[np.ndarray, np.ndarray]:
    """A grown CHNO molecule in which ``nhal`` hydrogens become Br or I
    (chosen with equal probability), moved out along their bond to the
    halogen's bond length; a hydrogen whose halogen would come within 2.2
    bohr of another atom is left in place.  Br and I have odd valence
    counts like H, so the molecule stays a closed shell."""
    num, pos = grow(natoms, seed)
    num, pos = num.copy(), pos.copy()
    rng = np.random.Generator(np.random.PCG64(seed + 777_000))
    heavy = np.flatnonzero(num != 1)
    done = 0
    for h in rng.permutation(np.flatnonzero(num == 1)):
        if done == nhal:
            break
        z = int(rng.choice(list(HALOGEN_BOND)))
        anchor = heavy[np.argmin(np.linalg.norm(pos[heavy] - pos[h], axis=1))]
        d = pos[h] - pos[anchor]
        cand = pos[anchor] + HALOGEN_BOND[z] * d / np.linalg.norm(d)
        others = np.delete(np.arange(len(num)), [h, anchor])
        if np.min(np.linalg.norm(pos[others] - cand, axis=1)) < MIN_DIST:
            continue
        num[h], pos[h] = z, cand
        done += 1
    return num, pos
