"""Per-molecule status paths, driven by ordinary host inputs only.

A batch mixes normal molecules with molecules that must fail:
* non-finite positions (refused by the geometry kernel: status NONFINITE);
* two coincident atoms (the repulsion energy is infinite: NONFINITE);
* three hydrogens 0.11/0.11/0.08 bohr apart, whose overlap matrix is
  indefinite because the reference drops overlap blocks of atom pairs closer
  than 0.1 bohr (integral/driver/pytorch/impls/overlap.py:147-243):
  CHOLESKY_FAIL, where the reference's Cholesky-reduced eigensolver raises.
Failed molecules return NaN energies, charges and gradients, the calculator
raises as the reference does, and every other molecule of the batch gives
exactly its result when run alone.  The Fermi-level and SCF iteration
limits are options of a call, so they are driven by their own calls: a
Fermi search cut to one Newton step at 5000 K fails
(wavefunction/filling.py:366: RuntimeError), two SCF iterations end
unconverged (SCFConvergenceWarning / SCFConvergenceError).
"""
import warnings

import numpy as np
import pytest
import torch

from dxtb_gb300 import _lib, molgen

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


def calc_for(numbers, **extra):
    from dxtb_gb300 import GFN1Calculator

    return GFN1Calculator(torch.as_tensor(np.asarray(numbers)), opts={**TIGHT, **extra})


def raw_call(calc, positions, forces=True):
    """The engine through torch.ops.gbxtb.singlepoint, returning every
    molecule's result and status (the calculator raises on failures)."""
    from dxtb_gb300 import calculator as cm

    plan = calc._plan(0, None)
    iopts, fopts = cm._pack_options(calc._options(forces))
    rpos = calc._ragged_positions(positions)
    e, q, g, st = cm._ops().singlepoint(plan.handle.value, rpos, plan.workspace(), iopts, fopts)
    return e.cpu().numpy(), q.cpu().numpy(), g.cpu().numpy(), st[:, 0].numpy()


def failing_batch():
    normal = molgen.c2_batch(8)[2:6]
    nan_mol = (normal[0][0].copy(), normal[0][1].copy())
    nan_mol[1][2, 1] = np.nan
    coincident = (normal[1][0].copy(), normal[1][1].copy())
    coincident[1][3] = coincident[1][2]
    h = np.sqrt(0.11 ** 2 - 0.04 ** 2)
    h3 = (np.array([1, 1, 1]), np.array([[0.0, 0.0, 0.0], [0.04, h, 0.0], [0.08, 0.0, 0.0]]))
    mols = [normal[0], nan_mol, normal[1], coincident, normal[2], h3, normal[3]]
    expect = {1: _lib.MOL_NONFINITE, 3: _lib.MOL_NONFINITE, 5: _lib.MOL_CHOLESKY_FAIL}
    return mols, expect


@pytest.mark.parametrize("mixed", [True, False], ids=["mixed", "fp64"])
def test_failures_stay_in_their_molecule(mixed):
    mols, expect = failing_batch()
    num, pos = pad(mols)
    calc = calc_for(num, mixed_precision=mixed)
    p = torch.tensor(pos, device="cuda")
    e, q, g, st = raw_call(calc, p)
    off = np.concatenate([[0], np.cumsum([len(m[0]) for m in mols])])
    for k, (n1, p1) in enumerate(mols):
        a, b = off[k], off[k + 1]
        if k in expect:
            assert st[k] & expect[k], (k, st[k])
            assert np.isnan(e[k]) and np.isnan(q[a:b]).all() and np.isnan(g[a:b]).all(), k
            continue
        assert st[k] == 0, (k, st[k])
        solo = calc_for(n1, mixed_precision=mixed).singlepoint(torch.tensor(p1, device="cuda"), forces=True)
        assert e[k] == solo.energy.item(), k
        assert np.array_equal(q[a:b], solo.charges.cpu().numpy()), k
        assert np.abs(g[a:b] - solo.gradient.cpu().numpy()).max() <= 1e-12, k
    with pytest.raises(RuntimeError):
        calc.singlepoint(p, forces=True)


def test_fermi_failure_raises():
    mols = molgen.c2_batch(8)[2:6]
    num, pos = pad(mols)
    calc = calc_for(num, fermi_etemp=5000.0, fermi_maxiter=1)
    p = torch.tensor(pos, device="cuda")
    e, _, g, st = raw_call(calc, p)
    failed = (st & _lib.MOL_FERMI_FAIL) != 0
    assert failed.any()
    assert np.isnan(e[failed]).all()
    with pytest.raises(RuntimeError, match="Fermi energy failed to converge"):
        calc.get_energy(p)
    # with the default Newton budget the same molecules find their Fermi level
    _, _, _, st2 = raw_call(calc_for(num, fermi_etemp=5000.0), p)
    assert (st2 & _lib.MOL_FERMI_FAIL == 0).all()


def test_two_iterations_end_unconverged():
    from dxtb_gb300 import SCFConvergenceError, SCFConvergenceWarning

    mols = molgen.c2_batch(8)[2:6]
    num, pos = pad(mols)
    p = torch.tensor(pos, device="cuda")
    calc = calc_for(num, maxiter=2)
    e, _, g, st = raw_call(calc, p)
    assert (st == _lib.MOL_NOT_CONVERGED).all()
    assert np.isfinite(e).all() and np.isfinite(g).all()  # the last iterate, as the reference returns
    with pytest.warns(SCFConvergenceWarning):
        calc.get_energy(p)
    with pytest.raises(SCFConvergenceError):
        calc_for(num, maxiter=2, force_convergence=True).get_energy(p)
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        calc_for(num).get_energy(p)


def test_fp64_throughput_probes():
    """The FP64 FMA and FP64 MMA microbenchmarks run and report plausible
    rates (between 10 GFLOP/s and 100 TFLOP/s)."""
    import ctypes as C

    from dxtb_gb300 import _lib

    lib = _lib.load()
    for probe in (lib.gbxtb_fp64_peak, lib.gbxtb_fp64_mma_peak):
        g = C.c_double()
        _lib.check(probe(C.byref(g)))
        assert 1e1 < g.value < 1e5, g.value
