"""Continuous batching (slot pools) on the GPU: every served result equals
the same molecule's solo single point, whatever else shares the device.

Tolerances as the other parity tests: energies 1e-8 Eh, forces 1e-6
Eh/bohr, charges 1e-7 e.  Molecules enter while others are mid-SCF, leave
when they converge, and their slots are reused."""
import warnings

import numpy as np
import pytest
import torch

from dxtb_gb300 import molgen

pytestmark = pytest.mark.gpu

TIGHT = {"exclude": ["disp"], "maxiter": 300, "x_atol": 1e-10, "x_atol_max": 1e-10}
E_TOL, F_TOL, Q_TOL = 1e-8, 1e-6, 1e-7


def solo(num, pos):
    from dxtb_gb300 import GFN1Calculator

    calc = GFN1Calculator(torch.as_tensor(np.asarray(num)), opts=TIGHT)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return calc.singlepoint(torch.tensor(pos, device="cuda"), forces=True)


def check_against_solo(requests):
    checked = 0
    for r in requests:
        ref = solo(r.numbers, r.positions)
        assert r.status == int(ref.status[0]), r.id
        if r.status != 0:
            continue
        assert abs(r.energy - ref.energy.item()) < E_TOL, r.id
        assert np.abs(r.gradient - ref.gradient.cpu().numpy()).max() < F_TOL, r.id
        assert np.abs(r.charges - ref.charges.cpu().numpy()).max() < Q_TOL, r.id
        checked += 1
    return checked


def test_served_results_equal_solo_runs():
    from dxtb_gb300.serve import Server

    mols = molgen.workload(3, 14, 8, 70, log_uniform=True)
    srv = Server(classes=((24, 3), (70, 3)), opts=TIGHT)
    # a first wave, then the rest while the first is still iterating
    for num, pos in mols[:5]:
        srv.submit(num, pos)
    for _ in range(4):
        srv.step()
    assert not srv.idle
    for num, pos in mols[5:]:
        srv.submit(num, pos)
    done = srv.run_until_idle()
    reqs = sorted(srv.completed, key=lambda r: r.id)
    assert len(reqs) == len(mols) and srv.idle
    # slots were reused: more molecules than slots, and some were admitted
    # after the first molecules had left
    first_done = min(r.t_done for r in reqs)
    assert any(r.t_admit > first_done for r in reqs)
    assert check_against_solo(reqs) >= len(mols) - 1
    assert len(done) <= len(mols)


def test_single_slot_pool_serves_a_queue():
    from dxtb_gb300.serve import Server

    mols = molgen.workload(3, 4, 10, 30, log_uniform=True)
    srv = Server(classes=((30, 1),), opts=TIGHT)
    for num, pos in mols:
        srv.submit(num, pos)
    srv.run_until_idle()
    assert len(srv.completed) == 4
    assert check_against_solo(srv.completed) == 4


def test_oversized_request_is_refused():
    from dxtb_gb300.serve import Server

    srv = Server(classes=((16, 2),), opts=TIGHT)
    num, pos = molgen.grow(30, 7)
    with pytest.raises(ValueError):
        srv.submit(num, pos)


def test_stragglers_leave_their_slots_and_keep_their_results():
    """evict_after = 12 passes: molecules still iterating then move to the
    straggler pool of their class and are solved again there; every result
    still equals the solo single point, and the evicted molecules are the
    ones whose solo SCF needs more passes."""
    from dxtb_gb300.serve import Server

    mols = molgen.workload(3, 10, 8, 60, log_uniform=True)
    srv = Server(classes=((24, 3), (60, 3)), opts=TIGHT, evict_after=12, straggler_share=0.34)
    for num, pos in mols:
        srv.submit(num, pos)
    srv.run_until_idle()
    reqs = sorted(srv.completed, key=lambda r: r.id)
    assert len(reqs) == len(mols) and srv.idle
    assert any(r.evicted for r in reqs)
    assert check_against_solo(reqs) >= len(mols) - 1
    for r in reqs:
        if r.evicted and r.status == 0:
            assert r.iterations + 1 >= 12


def test_small_molecules_in_a_large_class():
    """Molecules far below a class's capacity (here a class of up to 150
    atoms, 600 orbitals, above the on-chip limit of the FP32
    tridiagonalisation) are served correctly, whether the pool's passes
    take the shapes of a full batch or of its tail."""
    from dxtb_gb300.serve import Server

    mols = molgen.workload(3, 6, 10, 60, log_uniform=True)
    srv = Server(classes=((150, 6),), opts=TIGHT)
    for num, pos in mols:
        srv.submit(num, pos)
    srv.run_until_idle()
    assert len(srv.completed) == len(mols)
    assert check_against_solo(srv.completed) >= len(mols) - 1
