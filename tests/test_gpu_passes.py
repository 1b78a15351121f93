"""The two ways the engine runs SCF passes agree, on the GPU.

Without profiling a pass is replayed as a CUDA graph (one graph launch per
pass; the graph of the tail shapes once the iterating molecules fit on the
SMs); with profiling every kernel is launched on its own with timing events
around the stages.  Both enqueue the same kernels with the same launch
shapes, so their energies, charges and iteration counts are bit-identical;
the forces agree to 1e-12 Eh/bohr (the force kernels sum shell-pair terms
into atoms with atomic adds, whose order varies from run to run).  The
launch-shape autotuner only
changes how many warps or threads share a molecule's reductions: results
stay within the parity tolerances (energies 1e-8 Eh, forces 1e-6 Eh/bohr,
charges 1e-7 e)."""
import warnings

import numpy as np
import pytest
import torch

from dxtb_gb300 import molgen

pytestmark = pytest.mark.gpu

TIGHT = {"exclude": ["disp"], "maxiter": 300, "x_atol": 1e-10, "x_atol_max": 1e-10}
E_TOL, F_TOL, Q_TOL = 1e-8, 1e-6, 1e-7


def batch(nmol, lo, hi, seed):
    mols = molgen.workload(seed, nmol, lo, hi, log_uniform=True)
    n = max(len(m[0]) for m in mols)
    num = np.zeros((nmol, n), dtype=np.int64)
    pos = np.zeros((nmol, n, 3))
    for i, (a, b) in enumerate(mols):
        num[i, :len(a)] = a
        pos[i, :len(a)] = b
    return torch.as_tensor(num), torch.tensor(pos, device="cuda")


def run(num, pos, **extra):
    from dxtb_gb300 import GFN1Calculator

    calc = GFN1Calculator(num, opts={**TIGHT, "autotune": False, **extra})
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        return calc, calc.singlepoint(pos, forces=True)


def same(a, b):
    return (torch.equal(a.energy, b.energy) and torch.equal(a.charges, b.charges)
            and np.array_equal(a.iterations, b.iterations) and np.array_equal(a.status, b.status)
            and (a.gradient - b.gradient).abs().max().item() < 1e-12)


@pytest.mark.parametrize("mixed", [True, False])
def test_graph_replay_equals_launch_by_launch(mixed):
    # 200 molecules: more than the SMs, so both pass graphs (all molecules,
    # tail shapes) run before the batch ends
    num, pos = batch(200, 4, 60, 11)
    _, graph = run(num, pos, mixed_precision=mixed)
    _, plain = run(num, pos, mixed_precision=mixed, profile=True)
    assert same(graph, plain)


def test_graph_follows_a_new_workspace_and_new_positions():
    num, pos = batch(40, 4, 40, 12)
    calc, first = run(num, pos)
    # the same plan on moved atoms (a new geometry, the same graphs), then on
    # a new workspace (the graphs are captured again); the old workspace is
    # kept alive so that the new one has another address
    moved_pos = pos + 0.05 * torch.sin(torch.arange(pos.numel(), device="cuda").reshape(pos.shape).double())
    moved_pos = torch.where(num.to("cuda").unsqueeze(-1) > 0, moved_pos, pos)
    plan = next(iter(calc._plans.values()))
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        moved = calc.singlepoint(moved_pos, forces=True)
        old_ws = plan._ws
        plan._ws = None
        again = calc.singlepoint(pos, forces=True)
    assert plan._ws.data_ptr() != old_ws.data_ptr()
    _, moved_fresh = run(num, moved_pos)
    assert same(moved, moved_fresh)
    assert same(again, first)


def test_autotuned_shapes_keep_parity():
    num, pos = batch(64, 4, 90, 13)
    calc, tuned = run(num, pos, autotune=True)
    plan = next(iter(calc._plans.values()))
    assert plan.tuned is not None and len(plan.tuned) == 4
    assert all(w in (8, 16, 32) for w in plan.tuned[:3]) and plan.tuned[3] in (32, 64, 128, 256)
    _, fixed = run(num, pos)
    ok = (tuned.status == 0) & (fixed.status == 0)
    assert ok.sum() >= 60
    counts = (num != 0).sum(-1).numpy()
    ok_atom = torch.as_tensor(np.repeat(ok, counts), device="cuda")
    ok_mol = torch.as_tensor(ok, device="cuda")
    assert (tuned.energy - fixed.energy)[ok_mol].abs().max() < E_TOL
    assert (tuned.gradient - fixed.gradient)[ok_atom].abs().max() < F_TOL
    assert (tuned.charges - fixed.charges)[ok_atom].abs().max() < Q_TOL
