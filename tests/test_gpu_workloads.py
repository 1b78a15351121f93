"""Full-size workloads on the GPU against the reference's own results for
every molecule (tests/golden/workload_*_ref.npz, produced by the reference).

Molecules with several self-consistent solutions can end on different
solutions in the reference (Anderson mixing) and in the engine (Broyden
mixing).  For those the test checks that the engine's state is a genuine
fixed point of the reference's equations: the oracle restarted from the
engine's converged potential stays there and reproduces its energy."""
import numpy as np
import pytest
import torch

from dxtb_gb300 import molgen, params
from oracle import gfn1_oracle as go
from tests.helpers import GOLDEN, same_state

pytestmark = pytest.mark.gpu

TIGHT = {"exclude": ["disp"], "maxiter": 300, "x_atol": 1e-10, "x_atol_max": 1e-10}


def pad(mols):
    n = max(len(m[0]) for m in mols)
    num = np.zeros((len(mols), n), dtype=np.int64)
    pos = np.zeros((len(mols), n, 3))
    for i, (a, b) in enumerate(mols):
        num[i, :len(a)] = a
        pos[i, :len(a)] = b
    return num, pos


def shells_of(numbers):
    return sum(len(params.raw()["elements"][str(int(z))]["shells"]) for z in numbers)


def orbital_potential(numbers, vsh):
    out = []
    k = 0
    for z in numbers:
        for sh in params.raw()["elements"][str(int(z))]["shells"]:
            out.extend([vsh[k]] * (2 * sh["l"] + 1))
            k += 1
    return np.array(out)


def run_workload(mols, forces):
    from dxtb_gb300 import GFN1Calculator

    num, pos = pad(mols)
    calc = GFN1Calculator(torch.as_tensor(num), opts=TIGHT)
    import warnings

    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return calc.singlepoint(torch.tensor(pos, device="cuda"), forces=forces)


def check_workload(mols, ref, forces, min_agree):
    res = run_workload(mols, forces)
    e = res.energy.cpu().numpy()
    q = res.charges.cpu().numpy()
    f = -res.gradient.cpu().numpy() if forces else None
    vsh = res.shell_potential
    assert np.array_equal(np.array([len(n) for n, _ in mols]), ref["natom"])
    aoff = np.concatenate([[0], np.cumsum(ref["natom"])])
    soff = np.concatenate([[0], np.cumsum([shells_of(n) for n, _ in mols])])
    stats = {"same": 0, "other_state": 0, "ref_unconverged": 0, "engine_unconverged": 0}
    restarts = 0
    fd_checks = 0
    worst = {"dE": 0.0, "dq": 0.0, "dF": 0.0}
    for k, (num, pos) in enumerate(mols):
        a, b = aoff[k], aoff[k + 1]
        if res.status[k] & 1:
            stats["engine_unconverged"] += 1
            continue
        assert res.status[k] == 0
        if not ref["converged"][k]:
            stats["ref_unconverged"] += 1
            continue
        if same_state(e[k], ref["energy"][k]):
            stats["same"] += 1
            de = abs(e[k] - ref["energy"][k])
            dq = np.abs(q[a:b] - ref["charges"][a:b]).max()
            worst["dE"] = max(worst["dE"], de)
            worst["dq"] = max(worst["dq"], dq)
            assert de < 1e-8, k
            assert dq < 1e-6, k
            if forces:
                # the reference's analytical-gradient forces: same quantity
                dfa = np.abs(f[a:b] - ref["forces_analytical"][a:b]).max()
                worst["dF_analytical"] = max(worst.get("dF_analytical", 0.0), dfa)
                assert dfa < 1e-6, k
                # the reference's default autograd forces: equal up to the
                # Lorentzian broadening of its eigenvector derivative, which
                # matters when the HOMO-LUMO gap is near kT; central finite
                # differences decide those cases
                dfg = np.abs(f[a:b] - ref["forces"][a:b])
                worst["dF"] = max(worst["dF"], dfg.max())
                if dfg.max() >= 1e-6:
                    stats["autograd_outliers"] = stats.get("autograd_outliers", 0) + 1
                    if fd_checks < 3:
                        fd_checks += 1
                        at, x = np.unravel_index(np.argmax(dfg), dfg.shape)
                        # five-point central difference (truncation error O(h^4))
                        # of the oracle energy with the electron count solved
                        # to 1e-13: at the reference's sqrt(eps) Fermi
                        # tolerance the energy carries ~5e-9 Eh of noise,
                        # 5e-6 Eh/bohr after dividing by the step
                        h = 5e-4
                        efd = {}
                        for st in (-2, -1, 1, 2):
                            pp = pos.copy()
                            pp[at, x] += st * h
                            efd[st] = go.singlepoint(num, pp, mixer="broyden", forces=False,
                                                     fermi_thr=1e-13).energy
                        fd = -(8.0 * (efd[1] - efd[-1]) - (efd[2] - efd[-2])) / (12.0 * h)
                        err_engine = abs(f[a + at, x] - fd)
                        err_ref = abs(ref["forces"][a + at, x] - fd)
                        assert err_engine < 1e-6 and err_engine < err_ref, (k, err_engine, err_ref)
        else:
            stats["other_state"] += 1
            if restarts < 2:
                restarts += 1
                v = orbital_potential(num, vsh[soff[k]:soff[k + 1]])
                r = go.singlepoint(num, pos, mixer="broyden", v_init=v, forces=False, maxiter=30)
                assert r.converged and r.iterations <= 40, k
                assert abs(r.energy - e[k]) < 1e-8, k
    print(stats, worst)
    assert stats["same"] >= min_agree * len(mols)
    return stats


def test_batch_workload_512():
    ref = np.load(GOLDEN / "workload_batch_ref.npz")
    check_workload(molgen.c2_batch(512), ref, forces=False, min_agree=0.75)


def test_forces_workload_256():
    ref = np.load(GOLDEN / "workload_forces_ref.npz")
    check_workload(molgen.c3_forces(256), ref, forces=True, min_agree=0.85)
