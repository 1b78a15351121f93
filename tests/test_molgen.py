import numpy as np

from dxtb_gb300 import molgen


def test_deterministic():
    a = molgen.workload(1, 4, 10, 120)
    b = molgen.workload(1, 4, 10, 120)
    for (n1, p1), (n2, p2) in zip(a, b):
        assert (n1 == n2).all() and (p1 == p2).all()


def test_growth_rule():
    for seed in range(20):
        num, pos = molgen.grow(40, seed)
        assert len(num) in (39, 40)
        assert sum(molgen.VALENCE[int(z)] for z in num) % 2 == 0
        heavy = num > 1
        assert set(num[heavy]).issubset({6, 7, 8})
        assert abs(heavy.sum() - 20) == 0
        d = np.linalg.norm(pos[:, None] - pos[None], axis=-1) + np.eye(len(num)) * 10
        # every H sits 2.05 bohr from some heavy atom; all other pairs >= 2.2 bohr
        for i in np.where(~heavy)[0]:
            assert np.isclose(d[i][heavy].min(), molgen.BOND_H)
        hh = d[np.ix_(heavy, heavy)]
        assert hh.min() >= molgen.MIN_DIST - 1e-9


def test_workload_sizes():
    mols = molgen.c2_batch(64)
    sizes = np.array([len(n) for n, _ in mols])
    assert sizes.min() >= 9 and sizes.max() <= 120
    f = molgen.c3_forces(8)
    assert all(29 <= len(n) <= 60 for n, _ in f)
