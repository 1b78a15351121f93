"""GPU parity of the CUDA engine against the oracle and the reference's
outputs.  Tolerances: energies 1e-8 Eh, forces 1e-6 Eh/bohr (the bar of the
reference comparison), charges 1e-7 e; integrals 1e-12."""
import warnings

import numpy as np
import pytest
import torch

from dxtb_gb300 import molgen
from oracle import gfn1_oracle as go
from tests.helpers import GOLDEN, load_golden, same_state

pytestmark = pytest.mark.gpu

E_TOL = 1e-8
F_TOL = 1e-6
Q_TOL = 1e-7
TIGHT = {"exclude": ["disp"], "maxiter": 300, "x_atol": 1e-10, "x_atol_max": 1e-10}


def calc_for(numbers, **extra):
    from dxtb_gb300 import GFN1Calculator

    return GFN1Calculator(torch.as_tensor(np.asarray(numbers)), opts={**TIGHT, **extra})


def pad(mols):
    n = max(len(m[0]) for m in mols)
    num = np.zeros((len(mols), n), dtype=np.int64)
    pos = np.zeros((len(mols), n, 3))
    for i, (a, b) in enumerate(mols):
        num[i, :len(a)] = a
        pos[i, :len(a)] = b
    return num, pos


@pytest.mark.parametrize("mol", load_golden("reference_mols.npz") + load_golden("synthetic.npz")[:6],
                         ids=lambda m: m["name"])
def test_integrals_match_oracle(mol):
    num, pos = mol["numbers"], mol["positions"]
    calc = calc_for(num)
    (s, h), = calc.get_integrals(torch.tensor(pos, device="cuda"))
    b = go.Basis(num)
    s_ref = go.overlap(b, pos)
    h_ref = go.core_hamiltonian(b, pos, s_ref, go.coordination_number(num, pos)).h0
    assert np.abs(s.cpu().numpy() - s_ref).max() < 1e-12
    assert np.abs(h.cpu().numpy() - h_ref).max() < 1e-12


@pytest.mark.parametrize("mol", load_golden("reference_mols.npz"), ids=lambda m: m["name"])
def test_reference_molecules(mol):
    """Reference test geometries (incl. the open-shell NO2 and Si/Li
    compounds with d shells) against the reference's energies, charges and
    autograd forces."""
    calc = calc_for(mol["numbers"])
    pos = torch.tensor(mol["positions"], device="cuda")
    res = calc.singlepoint(pos, chrg=mol["charge"], forces=True)
    assert res.status[0] == 0
    assert abs(res.energy.item() - mol["energy"]) < E_TOL
    assert np.abs(res.charges.cpu().numpy() - mol["charges"]).max() < Q_TOL
    assert np.abs(-res.gradient.cpu().numpy() - mol["forces"]).max() < F_TOL


def test_synthetic_molecules_against_reference():
    """The synthetic golden molecules with the reference's own mixer
    (Anderson, every pass in FP64): every molecule ends in the reference's
    state, energies 1e-8 Eh, charges 1e-7 e, forces 1e-6 Eh/bohr of the
    reference's autograd forces.  Where those differ by more (the reference
    differentiates through its unrolled SCF, which is unreliable on slowly
    converging molecules), a five-point finite difference of the energy
    decides, and the engine must be within 1e-6 of it."""
    from tests.helpers import fd_force_component
    from tests.test_gpu_workloads import orbital_potential, shells_of

    mols = load_golden("synthetic.npz")
    num, pos = pad([(m["numbers"], m["positions"]) for m in mols])
    calc = calc_for(num, mixer="anderson", mixed_precision=False)
    res = calc.singlepoint(torch.tensor(pos, device="cuda"), forces=True)
    e = res.energy.cpu().numpy()
    f = -res.gradient.cpu().numpy()
    q = res.charges.cpu().numpy()
    off, soff = 0, 0
    for k, m in enumerate(mols):
        n, ns = len(m["numbers"]), shells_of(m["numbers"])
        assert res.status[k] == 0, m["name"]
        assert abs(e[k] - m["energy"]) < E_TOL, m["name"]
        assert np.abs(q[off:off + n] - m["charges"]).max() < Q_TOL, m["name"]
        df = np.abs(f[off:off + n] - m["forces"])
        if df.max() >= F_TOL:
            at, x = np.unravel_index(np.argmax(df), df.shape)
            v = orbital_potential(m["numbers"], res.shell_potential[soff:soff + ns])
            fd = fd_force_component(m["numbers"], m["positions"], at, x, v)
            assert abs(f[off + at, x] - fd) < F_TOL, (m["name"], f[off + at, x], fd, m["forces"][at, x])
        off += n
        soff += ns


def test_engine_replays_oracle_broyden():
    """Same mixer on both sides: the GPU (every pass in FP64) and the oracle
    follow the same SCF trajectory (iteration counts) and agree to 1e-10 Eh."""
    mols = molgen.c3_forces(4)
    for num, pos in mols:
        calc = calc_for(num, mixed_precision=False)
        res = calc.singlepoint(torch.tensor(pos, device="cuda"), forces=True)
        r = go.singlepoint(num, pos, mixer="broyden")
        assert abs(res.energy.item() - r.energy) < 1e-10
        assert np.abs(-res.gradient.cpu().numpy() - r.forces).max() < 1e-8
        assert abs(int(res.iterations[0]) - r.iterations) <= 2


def test_engine_replays_oracle_anderson():
    """The device Anderson mixer is the reference's (scf/mixer/anderson.py:
    200-317): with every pass in FP64 the engine and the oracle's restatement
    of the reference loop take the same number of SCF iterations and agree
    to 1e-10 Eh, in a batch of molecules of different sizes."""
    # molecules the reference converges in fewer than 150 iterations: far
    # slower ones amplify rounding differences over hundreds of iterations
    ref = np.load(GOLDEN / "workload_batch_ref.npz")
    pick = [k for k in range(40) if ref["converged"][k] and ref["iterations"][k] < 150][:8]
    mols = [molgen.c2_batch(40)[k] for k in pick]
    num, pos = pad(mols)
    calc = calc_for(num, mixer="anderson", mixed_precision=False)
    res = calc.singlepoint(torch.tensor(pos, device="cuda"), forces=True)
    for k, (n1, p1) in enumerate(mols):
        r = go.singlepoint(n1, p1, mixer="anderson", forces=False)
        if not r.converged:
            assert res.status[k] & 1
            continue
        assert res.status[k] == 0
        assert abs(res.energy[k].item() - r.energy) < 1e-10, k
        assert abs(int(res.iterations[k]) - r.iterations) <= 1, (k, int(res.iterations[k]), r.iterations)


def test_simple_mixer_and_options():
    """The simple mixer and the reference's mixing switches (mix_guess,
    damp_dynamic, soft start off) change the path, not the fixed point."""
    num, pos = molgen.c1_single()[0]
    p = torch.tensor(pos, device="cuda")
    e0 = calc_for(num).singlepoint(p).energy.item()
    for extra in ({"mixer": "simple", "damp": 0.2},
                  {"mixer": "anderson", "mix_guess": False},
                  {"mixer": "anderson", "damp_dynamic": True, "damp_soft_start": False},
                  {"mixer": "anderson", "damp_generations": 8, "damp_diagonal_offset": None}):
        res = calc_for(num, **extra).singlepoint(p)
        assert res.status[0] == 0, extra
        assert abs(res.energy.item() - e0) < 1e-10, extra


def test_torch_ops_direct():
    """torch.ops.gbxtb.singlepoint on a plan and forces_backward, and
    torch.autograd.grad through the calculator (which runs both), against
    the oracle."""
    from dxtb_gb300 import calculator as cm

    mols = molgen.c3_forces(3)
    num, pos = pad(mols)
    calc = calc_for(num, mixed_precision=False)
    plan = calc._plan(0, None)
    ops = cm._ops()
    iopts, fopts = cm._pack_options(calc._options(True))
    rpos = calc._ragged_positions(torch.tensor(pos, device="cuda"))
    e, q, state, st = ops.singlepoint(plan.handle.value, rpos, plan.workspace(), iopts, fopts)
    assert st.device.type == "cpu" and (st[:, 0] == 0).all()
    ge = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64, device="cuda")
    g = ops.forces_backward(state, ge, plan.atom_mol)
    off = np.concatenate([[0], np.cumsum([len(m[0]) for m in mols])])
    for k, (n1, p1) in enumerate(mols):
        r = go.singlepoint(n1, p1, mixer="broyden")
        assert abs(e[k].item() - r.energy) < 1e-10
        a, b = off[k], off[k + 1]
        assert np.abs(-state[a:b].cpu().numpy() - r.forces).max() < 1e-8
        assert torch.equal(g[a:b], ge[k] * state[a:b])
    # autograd through the operators, padded layout
    p = torch.tensor(pos, device="cuda", requires_grad=True)
    energy = calc.get_energy(p)
    (grad,) = torch.autograd.grad((energy * ge).sum(), p)
    for k, (n1, p1) in enumerate(mols):
        r = go.singlepoint(n1, p1, mixer="broyden")
        assert np.abs(grad[k, :len(n1)].cpu().numpy() + ge[k].item() * r.forces).max() < 1e-8
        assert (grad[k, len(n1):] == 0).all()


def test_forces_after_energy_reuse_the_scf():
    """get_forces after get_energy on the same positions computes the forces
    from the converged state of that call (gbxtb_forces), with no second
    SCF, and equals a fresh get_forces."""
    mols = molgen.c3_forces(2)
    num, pos = pad(mols)
    calc = calc_for(num)
    p = torch.tensor(pos, device="cuda")
    calc.get_energy(p)
    plan = calc._plan(0, None)
    runs = plan.runs
    f = calc.get_forces(p)
    assert plan.runs == runs
    fresh = calc_for(num).get_forces(p)
    assert torch.allclose(f, fresh, atol=1e-12, rtol=0)
    # other positions: a new SCF
    p2 = p + 0.01
    calc.get_energy(p2)
    assert plan.runs == runs + 1


def test_orbital_charges():
    """get_charges gives orbital-resolved Mulliken charges, as the
    reference's get_charges (calculators/types/abc.py:429-486): they match
    the oracle's per-orbital charges, their sums over each atom's orbitals
    are the atomic charges of singlepoint, and a batch pads them with 0."""
    mols = molgen.c3_forces(2)
    num, pos = pad(mols)
    calc = calc_for(num)
    p = torch.tensor(pos, device="cuda")
    q = calc.get_charges(p).cpu().numpy()
    assert torch.equal(calc.get_mulliken_charges(p).cpu(), torch.as_tensor(q))
    qat = calc.singlepoint(p).charges.cpu().numpy()
    naos = []
    off = 0
    for k, (n1, p1) in enumerate(mols):
        r = go.singlepoint(n1, p1, mixer="broyden", forces=False)
        nao = len(r.charges_orbital)
        naos.append(nao)
        assert np.abs(q[k, :nao] - r.charges_orbital).max() < Q_TOL
        assert np.all(q[k, nao:] == 0.0)
        b = go.Basis(n1)
        sums = np.bincount(b.sh_atom[b.ao_sh], weights=q[k, :nao], minlength=len(n1))
        assert np.abs(sums - qat[off:off + len(n1)]).max() < 1e-12
        off += len(n1)
    assert q.shape == (2, max(naos))
    # a single molecule gives a vector
    q1 = calc_for(mols[0][0]).get_charges(torch.tensor(mols[0][1], device="cuda"))
    assert q1.shape == (naos[0],)


def test_batch_equals_single():
    mols = molgen.c2_batch(6)
    num, pos = pad(mols)
    calc = calc_for(num)
    rb = calc.singlepoint(torch.tensor(pos, device="cuda"), forces=True)
    off = 0
    for k, (n1, p1) in enumerate(mols):
        rs = calc_for(n1).singlepoint(torch.tensor(p1, device="cuda"), forces=True)
        n = len(n1)
        assert rb.energy[k].item() == rs.energy.item()
        assert torch.allclose(rb.gradient[off:off + n], rs.gradient, atol=1e-12, rtol=0)
        off += n


def test_autograd_matches_forces():
    num, pos = molgen.c1_single()[0]
    calc = calc_for(num)
    p = torch.tensor(pos, device="cuda", requires_grad=True)
    e = calc.get_energy(p)
    (g,) = torch.autograd.grad(e, p)
    f = calc.get_forces(torch.tensor(pos, device="cuda"))
    assert torch.allclose(-g, f, atol=1e-12, rtol=0)
    assert e.shape == ()


def test_finite_differences():
    """Central differences (h = 1e-4 bohr) on 8 random atoms of each of four
    perturbed 30-60-atom molecules, every displaced geometry in one batched
    call, within 1e-6 Eh/bohr of the analytic forces.  The electron count is
    solved to 1e-13 (fermi_thresh), since at the default sqrt(eps) the
    energy carries ~1e-8 Eh of noise, 1e-4 Eh/bohr after dividing by h."""
    fine = {"fermi_thresh": 1e-13, "x_atol": 1e-12, "x_atol_max": 1e-12, "mixed_precision": False}
    h = 1e-4
    rng = np.random.default_rng(7)
    geoms, nums, an = [], [], []
    for num, pos in molgen.c3_forces(4):
        f = calc_for(num, **fine).get_forces(torch.tensor(pos, device="cuda")).cpu().numpy()
        atoms = rng.choice(len(num), size=8, replace=False)
        for a in atoms:
            for x in range(3):
                an.append(f[a, x])
                for sgn in (1.0, -1.0):
                    p = pos.copy()
                    p[a, x] += sgn * h
                    geoms.append((num, p))
    nb, pb = pad(geoms)
    e = calc_for(nb, **fine).get_energy(torch.tensor(pb, device="cuda")).cpu().numpy()
    fd = -(e[0::2] - e[1::2]) / (2 * h)
    err = np.abs(fd - np.array(an))
    assert err.max() < 1e-6, err.max()


def test_maxiter_warning_and_error():
    from dxtb_gb300 import SCFConvergenceError, SCFConvergenceWarning

    num, pos = molgen.c1_single()[0]
    calc = calc_for(num, maxiter=2)
    with pytest.warns(SCFConvergenceWarning):
        res = calc.singlepoint(torch.tensor(pos, device="cuda"))
    assert res.status[0] & 1
    calc = calc_for(num, maxiter=2, force_convergence=True)
    with pytest.raises(SCFConvergenceError):
        calc.singlepoint(torch.tensor(pos, device="cuda"))


def test_input_errors():
    from dxtb_gb300 import GFN1Calculator
    from dxtb_gb300._lib import GbxtbError

    with pytest.raises(ValueError):
        GFN1Calculator(torch.tensor([1, 1]), opts={})  # D3 not excluded
    with pytest.raises(ValueError):
        GFN1Calculator(torch.tensor([1.0, 1.0]), opts=TIGHT)
    calc = GFN1Calculator(torch.tensor([1, 1]), opts=TIGHT)
    with pytest.raises(ValueError):
        calc.get_energy(torch.zeros((2, 3), dtype=torch.float32, device="cuda"))
    with pytest.raises(GbxtbError):
        GFN1Calculator(torch.tensor([1, 87]), opts=TIGHT).get_energy(
            torch.tensor([[0.0, 0, 0], [0, 0, 1.4]], dtype=torch.float64, device="cuda"))


def test_charged_and_spin():
    """Cation and explicit spin go through the same path as the reference
    (electron count and alpha/beta split)."""
    num, pos = molgen.c1_single()[0]
    calc = calc_for(num)
    p = torch.tensor(pos, device="cuda")
    res = calc.singlepoint(p, chrg=1.0, spin=1)
    r = go.singlepoint(num, pos, chrg=1.0, spin=1, mixer="broyden", forces=False)
    assert abs(res.energy.item() - r.energy) < 1e-10
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        res2 = calc.singlepoint(p, chrg=2.0)
    r2 = go.singlepoint(num, pos, chrg=2.0, mixer="broyden", forces=False)
    assert abs(res2.energy.item() - r2.energy) < 1e-10


def test_mixed_precision_same_fixed_point():
    """The FP32 passes only move the SCF start: with and without them the
    engine ends on the same fixed point (energies 1e-10 Eh, forces 1e-8)."""
    mols = molgen.c2_batch(8)
    num, pos = pad(mols)
    p = torch.tensor(pos, device="cuda")
    r64 = calc_for(num, mixed_precision=False).singlepoint(p, forces=True)
    r32 = calc_for(num, mixed_precision=True).singlepoint(p, forces=True)
    e64, e32 = r64.energy.cpu().numpy(), r32.energy.cpu().numpy()
    # molecule 1 of the workload has no converging SCF (neither here nor in
    # the reference); the others converge in both modes
    conv = [k for k in range(len(mols)) if r64.status[k] == 0 and r32.status[k] == 0]
    assert len(conv) >= len(mols) - 1
    same = [k for k in conv if same_state(e64[k], e32[k])]
    assert len(same) >= len(conv) - 1
    for k in same:
        assert abs(e64[k] - e32[k]) < 1e-10
    g64, g32 = r64.gradient.cpu().numpy(), r32.gradient.cpu().numpy()
    off = np.concatenate([[0], np.cumsum([len(m[0]) for m in mols])])
    for k in same:
        assert np.abs(g64[off[k]:off[k + 1]] - g32[off[k]:off[k + 1]]).max() < 1e-8


def test_df64_tridiagonalisation_same_fixed_point():
    """FP64 passes with the on-chip cluster tridiagonalisation in double-float
    arithmetic (~48 bits) end on the fixed point of native FP64: every pass
    in FP64, molecules of 150-330 AOs (all on the cluster kernel), energies
    within 1e-10 Eh, forces 1e-8 Eh/bohr, and the same SCF pass counts up to
    one."""
    mols = [molgen.grow(a, 8100 + a) for a in (50, 70, 90, 110)]
    num, pos = pad(mols)
    p = torch.tensor(pos, device="cuda")
    rn = calc_for(num, mixed_precision=False, fp64_tridiag="native").singlepoint(p, forces=True)
    rd = calc_for(num, mixed_precision=False, fp64_tridiag="df64").singlepoint(p, forces=True)
    assert (rn.status == 0).all() and (rd.status == 0).all()
    assert np.abs(rn.energy.cpu().numpy() - rd.energy.cpu().numpy()).max() < 1e-10
    assert np.abs(rn.gradient.cpu().numpy() - rd.gradient.cpu().numpy()).max() < 1e-8
    assert np.abs(rn.iterations - rd.iterations).max() <= 1


def test_large_molecule_against_oracle():
    """A 300-atom molecule (~900 AOs): the block-wise Cholesky over the whole
    GPU, the global-memory lead-in of the on-chip FP32 tridiagonalisation
    and the cluster FP64 passes, against the oracle.  If the engine's mixed
    precision run ends in another SCF state than the oracle, the state must
    be a genuine fixed point of the reference's equations, and the FP64-only
    run (the oracle's own trajectory) must match the oracle."""
    from tests.helpers import restart_energy
    from tests.test_gpu_workloads import orbital_potential

    num, pos = molgen.grow(300, 4253)
    p = torch.tensor(pos, device="cuda")
    r = go.singlepoint(num, pos, mixer="broyden")
    assert r.converged
    res = calc_for(num).singlepoint(p, forces=True)
    assert res.status[0] == 0
    e = res.energy.item()
    if same_state(e, r.energy):
        assert abs(e - r.energy) < E_TOL
        assert np.abs(-res.gradient.cpu().numpy() - r.forces).max() < F_TOL
    else:
        assert abs(e - r.energy) > 1e-4
        conv, it, er = restart_energy(num, pos, orbital_potential(num, res.shell_potential))
        assert conv and it <= 40 and abs(er - e) < E_TOL
    r64 = calc_for(num, mixed_precision=False).singlepoint(p, forces=True)
    assert r64.status[0] == 0
    assert abs(r64.energy.item() - r.energy) < E_TOL
    assert np.abs(-r64.gradient.cpu().numpy() - r.forces).max() < F_TOL


def test_halogenated_molecules_against_reference():
    """Molecules with Br/I halogen-bond donors (tests/golden/halogen.npz,
    produced by the reference): energies 1e-8 Eh, charges 1e-7 e, forces
    1e-6 Eh/bohr.  The halogen-bond term is classical, so switching it off
    (exclude "hal") changes the energy by exactly the reference's term and
    the gradient by exactly its gradient."""
    mols = load_golden("halogen.npz")
    g = np.load(GOLDEN / "halogen.npz")
    num, pos = pad([(m["numbers"], m["positions"]) for m in mols])
    p = torch.tensor(pos, device="cuda")
    res = calc_for(num, mixer="anderson", mixed_precision=False).singlepoint(p, forces=True)
    off_ = calc_for(num, mixer="anderson", mixed_precision=False, exclude=["disp", "hal"]).singlepoint(
        p, forces=True)
    e, q, f = res.energy.cpu().numpy(), res.charges.cpu().numpy(), -res.gradient.cpu().numpy()
    e0, f0 = off_.energy.cpu().numpy(), -off_.gradient.cpu().numpy()
    off = 0
    for k, m in enumerate(mols):
        n = len(m["numbers"])
        assert res.status[k] == 0, m["name"]
        assert abs(e[k] - m["energy"]) < E_TOL, m["name"]
        assert np.abs(q[off:off + n] - m["charges"]).max() < Q_TOL, m["name"]
        assert np.abs(f[off:off + n] - m["forces"]).max() < F_TOL, m["name"]
        assert abs((e[k] - e0[k]) - g["xb_energy"][k]) < 1e-12, m["name"]
        assert np.abs((f0 - f)[off:off + n] - g["xb_gradient"][off:off + n]).max() < 1e-12, m["name"]
        off += n
