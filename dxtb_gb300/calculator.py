"""Drop-in GFN1-xTB calculator on the GB300 engine.

Mirrors the surface of dxtb's calculator
(``dxtb/_src/calculators/gfn1.py:46-70``; ``types/abc.py:88-170``):

    calc = GFN1Calculator(numbers, opts={...}, dtype=torch.float64)
    energy = calc.get_energy(positions)          # (...,)
    forces = calc.get_forces(positions)          # (..., nat, 3) = -dE/dR

``numbers`` is ``(nat,)`` or a padded batch ``(B, nat_max)`` with 0 as
padding (``types/base.py:518-569``); ``positions`` are in bohr with the same
leading shape.  Energies are differentiable: if ``positions.requires_grad``
the engine computes the analytic gradient in the same call and autograd
returns it (``types/autograd.py:82-201``).

All arithmetic runs in the CUDA library ``libgbxtb.so`` (FP64); this module
only converts between the padded torch layout and the engine's ragged
layout, owns device workspaces, and maps status codes onto the reference's
exceptions and warnings (``scf/unrolling/default.py:123-136``,
``wavefunction/filling.py:366``).
"""
from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, params

__all__ = ["GFN1Calculator", "SCFConvergenceWarning", "SCFConvergenceError", "Result"]


class SCFConvergenceWarning(UserWarning):
    """SCF hit ``maxiter`` (reference: typing/exceptions/scf.py)."""


class SCFConvergenceError(RuntimeError):
    """Raised instead of the warning when ``force_convergence`` is set."""


DEFAULT_OPTS = {
    "maxiter": 100,          # constants/defaults.py MAXITER
    "x_atol": 1.0e-4,        # X_ATOL
    "x_atol_max": 1.0e-5,    # X_ATOL_MAX
    "f_atol": 1.0e-4,        # accepted, unused (the potential change decides)
    "fermi_etemp": 300.0,    # FERMI_ETEMP (K)
    "fermi_maxiter": 200,    # FERMI_MAXITER
    "force_convergence": False,
    "exclude": [],
    "guess": "sad",
    "mixer": "broyden",
    "broyden_alpha": 0.3,
    "broyden_memory": 20,
    "verbosity": 0,
    "profile": False,        # per-stage device timings (last_profile)
    "mixed_precision": True,  # FP32 linear algebra in the early SCF passes
    "autotune": "auto",      # tune eigensolver launch shapes on the first call (auto: batches of >= 32)
}
_ACCEPTED_IGNORED = {"scf_mode", "scp_mode", "int_driver", "int_level", "batch_mode", "damp",
                     "damp_init", "mix_guess", "cache_enabled", "timer", "strict", "log_level"}


@dataclass
class Result:
    energy: torch.Tensor          # (B,) total energy per molecule
    charges: torch.Tensor         # ragged Mulliken atomic charges
    gradient: torch.Tensor | None  # ragged dE/dR
    status: np.ndarray
    iterations: np.ndarray
    shell_potential: np.ndarray | None = None  # final shell-resolved potential (host)
    fp32_passes: np.ndarray | None = None      # SCF passes per molecule that ran in FP32


class _Context:
    """Parameter tables uploaded to one CUDA device."""

    _by_device: dict[int, "_Context"] = {}

    def __init__(self, device: int):
        lib = _lib.load()
        t = params.tables()
        self._keep = t
        p = _lib.Params()
        p.max_z = params.MAX_Z
        p.n_shell_records = t.shell_int.shape[0]
        p.elem_shell0 = _lib.ptr(t.elem_shell0, C.c_int32)
        p.elem_nshell = _lib.ptr(t.elem_nshell, C.c_int32)
        p.elem_data = _lib.ptr(t.elem_data, C.c_double)
        p.shell_int = _lib.ptr(t.shell_int, C.c_int32)
        p.shell_data = _lib.ptr(t.shell_data, C.c_double)
        p.kpair = _lib.ptr(t.kpair, C.c_double)
        p.globals = _lib.ptr(t.globals, C.c_double)
        h = C.c_void_p()
        with torch.cuda.device(device):
            _lib.check(lib.gbxtb_ctx_create(C.byref(p), C.byref(h)))
        self.handle = h
        self.device = device

    @classmethod
    def get(cls, device: int) -> "_Context":
        if device not in cls._by_device:
            cls._by_device[device] = cls(device)
        return cls._by_device[device]


class Plan:
    """A planned ragged batch (atom/shell/AO maps on the device)."""

    def __init__(self, ctx: _Context, numbers_ragged: np.ndarray, offsets: np.ndarray,
                 charge: np.ndarray, uhf: np.ndarray | None):
        lib = _lib.load()
        self._lib = lib
        self.nmol = len(offsets) - 1
        self.natom = int(offsets[-1])
        nums = np.ascontiguousarray(numbers_ragged, dtype=np.int32)
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        chg = np.ascontiguousarray(charge, dtype=np.float64)
        u = None if uhf is None else np.ascontiguousarray(uhf, dtype=np.int32)
        h = C.c_void_p()
        ws = C.c_size_t()
        with torch.cuda.device(ctx.device):
            _lib.check(lib.gbxtb_plan_create(
                ctx.handle, self.nmol, _lib.ptr(nums, C.c_int32), _lib.ptr(offs, C.c_int64),
                _lib.ptr(chg, C.c_double), None if u is None else _lib.ptr(u, C.c_int32),
                C.byref(h), C.byref(ws)))
        self.handle = h
        self.ws_bytes = int(ws.value)
        sizes = np.zeros(6, dtype=np.int64)
        _lib.check(lib.gbxtb_plan_sizes(h, _lib.ptr(sizes, C.c_int64)))
        self.sizes = sizes
        self.device = ctx.device
        self._ws: torch.Tensor | None = None
        self.tuned: list | None = None  # autotuned launch shapes, once tuned

    def workspace(self) -> torch.Tensor:
        if self._ws is None:
            self._ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=f"cuda:{self.device}")
        return self._ws

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.handle.value:
                self._lib.gbxtb_plan_destroy(self.handle)
        except Exception:  # pragma: no cover - interpreter shutdown
            pass


class _EnergyFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, positions, calc, chrg, spin):
        res = calc._run(positions.detach(), chrg, spin, forces=True)
        ctx.save_for_backward(calc._pad_vectors(res.gradient))
        return calc._shape_energy(res.energy)

    @staticmethod
    def backward(ctx, grad_e):
        (g,) = ctx.saved_tensors
        return grad_e.unsqueeze(-1).unsqueeze(-1) * g, None, None, None


class GFN1Calculator:
    """GFN1-xTB calculator with dxtb's ``GFN1Calculator`` interface."""

    def __init__(self, numbers: torch.Tensor, *, classical=None, interaction=None, opts=None,
                 device: torch.device | str | None = None, dtype: torch.dtype | None = None,
                 **kwargs):
        if classical or interaction:
            raise NotImplementedError("custom classical/interaction components are not supported")
        if dtype is not None and dtype != torch.float64:
            raise ValueError("the engine computes in float64; pass dtype=torch.float64")
        if numbers.dtype not in (torch.int16, torch.int32, torch.int64):
            raise ValueError(f"numbers must be int16/int32/int64, got {numbers.dtype}")
        if numbers.ndim not in (1, 2):
            raise ValueError("numbers must have shape (nat,) or (B, nat)")
        o = dict(DEFAULT_OPTS)
        for key, val in (opts or {}).items():
            if key in DEFAULT_OPTS:
                o[key] = val
            elif key not in _ACCEPTED_IGNORED:
                raise ValueError(f"unknown option {key!r}")
        excl = set(o["exclude"]) if not isinstance(o["exclude"], str) else {o["exclude"]}
        if "disp" not in excl:
            raise ValueError(
                "D3 dispersion is not available in this engine (its reference data is not "
                "distributed with the model); pass opts={'exclude': ['disp']}"
            )
        if {"es2", "es3", "rep", "scf", "all", "hcore"} & excl:
            raise NotImplementedError(f"excluding {sorted(excl - {'disp', 'halogen'})} is not supported")
        if o["guess"] not in ("sad", "eeq"):
            raise ValueError(f"unknown guess {o['guess']!r}")
        self.opts = o
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device()) if numbers.device.type != "cuda" else numbers.device
        device = torch.device(device)
        if device.type != "cuda":
            raise RuntimeError("the GFN1 engine runs on CUDA devices only")
        self.device = device if device.index is not None else torch.device("cuda", torch.cuda.current_device())
        self.dtype = torch.float64
        self.numbers = numbers.to(self.device)
        self.batched = numbers.ndim == 2
        nh = numbers.detach().cpu().numpy().astype(np.int64)
        nh2 = nh[None, :] if not self.batched else nh
        self._mask_np = nh2 != 0
        counts = self._mask_np.sum(-1)
        if (counts == 0).any():
            raise ValueError("a molecule without atoms in the batch")
        self._counts = counts
        self._offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        self._numbers_ragged = nh2[self._mask_np]
        self._mask = torch.as_tensor(self._mask_np, device=self.device)
        self._ctx = _Context.get(self.device.index)
        self._plans: dict = {}
        self._cache: dict = {}
        self.last_profile: dict = {}

    # ------------------------------------------------------------------ layout
    def _ragged_positions(self, positions: torch.Tensor) -> torch.Tensor:
        if positions.dtype != torch.float64:
            raise ValueError(f"positions must be float64, got {positions.dtype}")
        if positions.device != self.device:
            raise ValueError(f"positions are on {positions.device}, calculator on {self.device}")
        if positions.shape[:-1] != self.numbers.shape or positions.shape[-1] != 3:
            raise ValueError(f"positions {tuple(positions.shape)} do not match numbers {tuple(self.numbers.shape)}")
        pos = positions if self.batched else positions.unsqueeze(0)
        return pos[self._mask].contiguous()

    def _pad_vectors(self, ragged: torch.Tensor) -> torch.Tensor:
        nb, nat = self._mask.shape
        out = torch.zeros((nb, nat, *ragged.shape[1:]), dtype=ragged.dtype, device=ragged.device)
        out[self._mask] = ragged
        return out if self.batched else out[0]

    def _shape_energy(self, e: torch.Tensor) -> torch.Tensor:
        return e if self.batched else e[0]

    def _plan(self, chrg, spin) -> Plan:
        nmol = len(self._counts)
        if isinstance(chrg, torch.Tensor):
            c = chrg.detach().cpu().double().numpy().reshape(-1)
        else:
            if self.batched and chrg != 0:
                raise ValueError("Cannot set charge for batched calculations with a single number; pass a tensor")
            c = np.array([float(chrg)])
        c = np.broadcast_to(c, (nmol,)).copy()
        if spin is None:
            u = None
        else:
            su = spin.detach().cpu().numpy().reshape(-1) if isinstance(spin, torch.Tensor) else np.array([spin])
            u = np.broadcast_to(su.astype(np.int32), (nmol,)).copy()
        key = (tuple(c.tolist()), None if u is None else tuple(u.tolist()))
        if key not in self._plans:
            self._plans[key] = Plan(self._ctx, self._numbers_ragged, self._offsets, c, u)
        return self._plans[key]

    # ------------------------------------------------------------------ engine
    def _options(self, forces: bool) -> _lib.Options:
        o = self.opts
        opt = _lib.Options()
        opt.maxiter = int(o["maxiter"])
        opt.fermi_maxiter = int(o["fermi_maxiter"])
        opt.broyden_memory = int(o["broyden_memory"])
        opt.want_forces = 1 if forces else 0
        opt.x_atol = float(o["x_atol"])
        opt.x_atol_max = float(o["x_atol_max"])
        opt.kt = float(o["fermi_etemp"]) * params.KELVIN2AU
        opt.broyden_alpha = float(o["broyden_alpha"])
        opt.profile = 1 if o["profile"] else 0
        opt.mixed_precision = 1 if o["mixed_precision"] else 0
        return opt

    def _run(self, positions: torch.Tensor, chrg=0, spin=None, forces: bool = False) -> Result:
        lib = _lib.load()
        plan = self._plan(chrg, spin)
        pos = self._ragged_positions(positions)
        dev = self.device
        energy = torch.empty(plan.nmol, dtype=torch.float64, device=dev)
        charges = torch.empty(plan.natom, dtype=torch.float64, device=dev)
        grad = torch.empty((plan.natom, 3), dtype=torch.float64, device=dev) if forces else None
        ws = plan.workspace()
        opt = self._options(forces)
        stream = torch.cuda.current_stream(dev).cuda_stream
        tune = self.opts["autotune"]
        if plan.tuned is None and (tune is True or (tune == "auto" and plan.nmol >= 32)):
            choice = np.zeros(4, dtype=np.int32)
            with torch.cuda.device(dev):
                _lib.check(lib.gbxtb_plan_autotune(plan.handle, C.byref(opt), pos.data_ptr(), ws.data_ptr(),
                                                   plan.ws_bytes, stream, _lib.ptr(choice, C.c_int32)))
            plan.tuned = choice.tolist()
        with torch.cuda.device(dev):
            _lib.check(lib.gbxtb_singlepoint(
                plan.handle, C.byref(opt), pos.data_ptr(), energy.data_ptr(), charges.data_ptr(),
                grad.data_ptr() if grad is not None else None, ws.data_ptr(), plan.ws_bytes, stream))
        status = np.zeros(plan.nmol, dtype=np.int32)
        iters = np.zeros(plan.nmol, dtype=np.int32)
        _lib.check(lib.gbxtb_get_status(plan.handle, _lib.ptr(status, C.c_int32), _lib.ptr(iters, C.c_int32)))
        p32 = np.zeros(plan.nmol, dtype=np.int32)
        _lib.check(lib.gbxtb_get_fp32_passes(plan.handle, _lib.ptr(p32, C.c_int32)))
        vsh = np.zeros(int(plan.sizes[2]), dtype=np.float64)
        _lib.check(lib.gbxtb_get_shell_potential(plan.handle, _lib.ptr(vsh, C.c_double)))
        ms = np.zeros(len(_lib.PROF_CLASSES), dtype=np.float64)
        nl = np.zeros(len(_lib.PROF_CLASSES), dtype=np.int64)
        tot = C.c_int64()
        _lib.check(lib.gbxtb_get_profile(plan.handle, _lib.ptr(ms, C.c_double), _lib.ptr(nl, C.c_int64),
                                         C.byref(tot)))
        self.last_profile = {"ms": dict(zip(_lib.PROF_CLASSES, ms.tolist())),
                             "launches": dict(zip(_lib.PROF_CLASSES, nl.tolist())),
                             "total_launches": int(tot.value)}
        self._raise_on_status(status)
        return Result(energy=energy, charges=charges, gradient=grad, status=status, iterations=iters,
                      shell_potential=vsh, fp32_passes=p32)

    def _raise_on_status(self, status: np.ndarray) -> None:
        if (status & _lib.MOL_FERMI_FAIL).any():
            raise RuntimeError("Fermi energy failed to converge.")
        if (status & _lib.MOL_CHOLESKY_FAIL).any():
            raise RuntimeError("overlap matrix is not positive definite (atoms too close?)")
        if (status & _lib.MOL_NONFINITE).any():
            raise RuntimeError("non-finite values in the SCF (check the geometry)")
        if (status & _lib.MOL_NOT_CONVERGED).any():
            msg = (f"SCF does not converge after {self.opts['maxiter']} cycles for "
                   f"{int((status & _lib.MOL_NOT_CONVERGED).astype(bool).sum())} molecule(s).")
            if self.opts["force_convergence"]:
                raise SCFConvergenceError(msg)
            warnings.warn(msg, SCFConvergenceWarning, stacklevel=3)

    # ------------------------------------------------------------------ public
    def singlepoint(self, positions: torch.Tensor, chrg=0, spin=None, forces: bool = False) -> Result:
        """Engine call returning energies, charges, gradient (ragged) and status."""
        return self._run(positions, chrg, spin, forces)

    def get_energy(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        if positions.requires_grad:
            return _EnergyFunction.apply(positions, self, chrg, spin)
        key = ("energy", positions.data_ptr(), positions._version, str(chrg), str(spin))
        if key not in self._cache:
            self._cache = {key: self._shape_energy(self._run(positions, chrg, spin).energy)}
        return self._cache[key]

    def get_forces(self, positions: torch.Tensor, chrg=0, spin=None, grad_mode: str = "autograd",
                   **kwargs) -> torch.Tensor:
        if grad_mode not in ("autograd", "backward", "functorch", "row", "analytical"):
            raise ValueError(f"unknown grad_mode {grad_mode!r}")
        res = self._run(positions.detach(), chrg, spin, forces=True)
        return -self._pad_vectors(res.gradient)

    def get_potential_energy(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        """Alias of ``get_energy`` (``calculators/types/abc.py:101-109``)."""
        return self.get_energy(positions, chrg, spin, **kwargs)

    def get_charges(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        """Orbital-resolved Mulliken charges, shape ``(..., nao)`` with
        padded orbitals set to 0, as ``get_charges`` of the reference
        (``calculators/types/abc.py:429-486``).  Their sums over each
        atom's orbitals are the atomic charges of ``singlepoint``."""
        lib = _lib.load()
        self._run(positions.detach(), chrg, spin)
        plan = self._plan(chrg, spin)
        q = np.zeros(int(plan.sizes[3]))
        _lib.check(lib.gbxtb_get_orbital_charges(plan.handle, _lib.ptr(q, C.c_double)))
        return torch.as_tensor(self._pad_orbitals(q), device=self.device)

    def get_mulliken_charges(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        """Alias of ``get_charges`` (``calculators/types/abc.py:488-495``)."""
        return self.get_charges(positions, chrg, spin, **kwargs)

    def get_iterations(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        """SCF iterations as a 0-d tensor (``calculators/types/abc.py:497-508``;
        the reference stores the count of its SCF loop, which for a batch
        runs until the last molecule is done: here the largest count of the
        batch)."""
        res = self._run(positions.detach(), chrg, spin)
        return torch.tensor(int(np.max(res.iterations)), device=self.device)

    def get_implemented_properties(self) -> list[str]:
        return sorted(["charges", "energy", "forces", "iterations"])

    def _orbital_counts(self) -> np.ndarray:
        if not hasattr(self, "_nao_per_mol"):
            elems = params.raw()["elements"]
            nao_z = {int(z): sum(2 * sh["l"] + 1 for sh in elems[str(int(z))]["shells"])
                     for z in np.unique(self._numbers_ragged)}
            per_atom = np.array([nao_z[int(z)] for z in self._numbers_ragged], dtype=np.int64)
            self._nao_per_mol = np.array([per_atom[self._offsets[m]:self._offsets[m + 1]].sum()
                                          for m in range(len(self._counts))], dtype=np.int64)
        return self._nao_per_mol

    def _pad_orbitals(self, ragged: np.ndarray) -> np.ndarray:
        """Ragged per-orbital values (plan order) -> ``(B, nao_max)``
        padded with zeros, or ``(nao,)`` for a single molecule."""
        counts = self._orbital_counts()
        if len(ragged) != int(counts.sum()):
            raise ValueError(f"{len(ragged)} orbital values for {int(counts.sum())} orbitals")
        out = np.zeros((len(counts), int(counts.max())))
        off = 0
        for m, n in enumerate(counts):
            out[m, :n] = ragged[off:off + n]
            off += n
        return out if self.batched else out[0]

    def get_integrals(self, positions: torch.Tensor, chrg=0, spin=None):
        """Overlap and core Hamiltonian of every molecule, as a list of
        (nao, nao) tensors."""
        lib = _lib.load()
        plan = self._plan(chrg, spin)
        pos = self._ragged_positions(positions.detach())
        nmat = int(plan.sizes[4])
        s = torch.empty(nmat, dtype=torch.float64, device=self.device)
        h = torch.empty(nmat, dtype=torch.float64, device=self.device)
        ws = plan.workspace()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        with torch.cuda.device(self.device):
            _lib.check(lib.gbxtb_integrals(plan.handle, pos.data_ptr(), s.data_ptr(), h.data_ptr(),
                                           ws.data_ptr(), plan.ws_bytes, stream))
        out = []
        off = 0
        nums = self._numbers_ragged
        for m in range(plan.nmol):
            z = nums[self._offsets[m]:self._offsets[m + 1]]
            n = sum(sum(2 * s_["l"] + 1 for s_ in params.raw()["elements"][str(int(x))]["shells"]) for x in z)
            out.append((s[off:off + n * n].view(n, n), h[off:off + n * n].view(n, n)))
            off += n * n
        return out

    def reset(self) -> None:
        self._cache = {}
