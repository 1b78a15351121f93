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
    "f_atol": 1.0e-4,        # F_ATOL: read only by the reference's implicit and single-shot SCF
                             # modes, not by its default full mode; accepted, unused
    "fermi_etemp": 300.0,    # FERMI_ETEMP (K)
    "fermi_maxiter": 200,    # FERMI_MAXITER
    "fermi_thresh": None,    # FERMI_THRESH (None: sqrt of machine epsilon)
    "force_convergence": False,
    "exclude": [],
    "guess": "sad",
    # "broyden": the engine's modified Broyden (Johnson 1988); "anderson": the
    # reference's Anderson mixer step for step (what its default full-mode SCF
    # runs, scf/unrolling/base.py:81-99); "simple": linear mixing
    "mixer": "broyden",
    "broyden_alpha": 0.2,    # fastest of 0.1-0.5 on the 512-molecule workload, and the closest to the reference
    "broyden_memory": 20,
    # Broyden/simple: a molecule still iterating after this many passes is
    # solved again from the guess with the reference's Anderson mixer (FP64),
    # so that it follows the reference's own SCF; 0: never
    "anderson_restart": 0,
    "damp": 0.5,                    # DAMP
    "damp_init": 0.1,               # DAMP_INIT
    "damp_generations": 5,          # DAMP_GENERATIONS
    "damp_diagonal_offset": 0.01,   # DAMP_DIAGONAL_OFFSET (None: no rescaling)
    "damp_soft_start": True,        # DAMP_SOFT_START
    "damp_dynamic": False,          # DAMP_DYNAMIC
    "damp_dynamic_factor": 0.99,    # DAMP_DYNAMIC_FACTOR
    "mix_guess": True,              # MIX_GUESS
    "scp_mode": "potential",        # SCP_MODE: the potential is the mixed quantity
    "verbosity": 0,
    "profile": False,        # per-stage device timings (last_profile)
    "mixed_precision": True,  # FP32 linear algebra in the early SCF passes
    # FP64 passes of the on-chip cluster tridiagonalisation: "auto" (double-
    # float pairs on the FP32 pipe with mixed_precision, native FP64
    # without), "native" or "df64"
    "fp64_tridiag": "auto",
    "autotune": "auto",      # tune eigensolver launch shapes on the first call (auto: batches of >= 32)
}
# Options of the reference that do not change the numbers this engine
# computes: the SCF mode only decides how the reference tracks gradients
# through its SCF (the fixed point and the forces are the same), the
# integral driver and level only how it evaluates the same integrals, the
# batch mode how it pads, and the rest are logging and caching switches.
_ACCEPTED_IGNORED = {"scf_mode", "int_driver", "int_level", "batch_mode", "cache_enabled", "timer",
                     "strict", "log_level"}
_SCP_MODES = {"potential"}
_FP64_TRIDIAG = {"auto": 0, "native": 1, "df64": 2}


@dataclass
class Result:
    energy: torch.Tensor          # (B,) total energy per molecule
    charges: torch.Tensor         # ragged Mulliken atomic charges
    gradient: torch.Tensor | None  # ragged dE/dR
    status: np.ndarray
    iterations: np.ndarray
    shell_potential: np.ndarray | None = None  # final shell-resolved potential (host)
    fp32_passes: np.ndarray | None = None      # SCF passes per molecule that ran in FP32
    atom_mol: torch.Tensor | None = None       # molecule of each ragged atom (device)


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
        counts = np.diff(offs)
        self.atom_mol = torch.as_tensor(np.repeat(np.arange(self.nmol), counts), device=f"cuda:{ctx.device}")
        self.runs = 0  # singlepoint calls made; the workspace holds the state of the last

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


_OPS_LOADED = False


def _ops():
    """``torch.ops.gbxtb`` (``csrc/torch_ops.cpp``), loaded once; raises if the
    operator library has not been built."""
    global _OPS_LOADED
    if not _OPS_LOADED:
        from . import build

        path = build.torch_ops_path()
        if not path.exists():
            raise _lib.GbxtbError(
                f"{path.name} is not built; run `python -m dxtb_gb300.build` (the torch operators of the "
                "CUDA engine are required, there is no CPU fallback)")
        _lib.load()
        torch.ops.load_library(str(path))
        _register_fakes()
        _OPS_LOADED = True
    return torch.ops.gbxtb


def _register_fakes() -> None:
    """Shape functions of the operators, so that FX tracing and
    ``torch.compile`` can see through them without running the engine."""
    lib = _lib.load()

    def sizes(plan: int) -> np.ndarray:
        out = np.zeros(6, dtype=np.int64)
        _lib.check(lib.gbxtb_plan_sizes(C.c_void_p(plan), _lib.ptr(out, C.c_int64)))
        return out

    @torch.library.register_fake("gbxtb::singlepoint")
    def _singlepoint_fake(plan, positions, workspace, iopts, fopts):
        nmol, natom = (int(x) for x in sizes(plan)[:2])
        want = bool(iopts[3])
        return (positions.new_empty((nmol,)), positions.new_empty((natom,)),
                positions.new_empty((natom, 3) if want else (0,)),
                torch.empty((nmol, 2), dtype=torch.int32, device="cpu"))

    @torch.library.register_fake("gbxtb::forces_backward")
    def _forces_backward_fake(state, grad_energy, atom_mol):
        return torch.empty_like(state)


def _pack_options(o: _lib.Options) -> tuple[list[int], list[float]]:
    """The option vectors of ``gbxtb::singlepoint`` (order in torch_ops.cpp)."""
    iopts = [o.maxiter, o.fermi_maxiter, o.broyden_memory, o.want_forces, o.profile, o.mixed_precision,
             o.mixer, o.generations, o.soft_start, o.mix_guess, o.damp_dynamic, o.no_halogen, o.restart_at,
             o.fp64_split]
    fopts = [o.x_atol, o.x_atol_max, o.kt, o.broyden_alpha, o.damp, o.damp_init, o.diagonal_offset,
             o.damp_dynamic_factor, o.fermi_thresh]
    return [int(x) for x in iopts], [float(x) for x in fopts]


class _EnergyFunction(torch.autograd.Function):
    """Energies of a plan's molecules as a differentiable function of the
    ragged positions: the forward runs ``gbxtb::singlepoint`` with the
    adjoint kernels, the backward ``gbxtb::forces_backward``
    (reference: ``calculators/types/autograd.py:82-201``)."""

    @staticmethod
    def forward(ctx, positions_ragged, calc, chrg, spin):
        res = calc._run(positions_ragged.detach(), chrg, spin, forces=True, ragged=True)
        ctx.save_for_backward(res.gradient, res.atom_mol)
        return res.energy

    @staticmethod
    def backward(ctx, grad_e):
        state, atom_mol = ctx.saved_tensors
        return _ops().forces_backward(state, grad_e.contiguous(), atom_mol), None, None, None


def resolve_opts(opts: dict | None) -> dict:
    """The reference's option dict (``calculators/config/main.py:86-156``)
    merged with the defaults and checked: options this engine cannot honour
    raise instead of being dropped."""
    o = dict(DEFAULT_OPTS)
    for key, val in (opts or {}).items():
        if key in DEFAULT_OPTS:
            o[key] = val
        elif key not in _ACCEPTED_IGNORED:
            raise ValueError(f"unknown option {key!r}")
    if str(o["mixer"]).lower() not in _lib.MIXERS:
        raise ValueError(f"unknown mixer {o['mixer']!r}; choose one of {sorted(_lib.MIXERS)}")
    if str(o["scp_mode"]).lower() not in _SCP_MODES:
        raise NotImplementedError(
            f"scp_mode {o['scp_mode']!r}: the engine mixes the potential (scp_mode='potential'), "
            "which can reach another SCF solution than mixing charges or the Fock matrix")
    excl = set(o["exclude"]) if not isinstance(o["exclude"], str) else {o["exclude"]}
    if "disp" not in excl:
        raise ValueError(
            "D3 dispersion is not available in this engine (its reference data is not "
            "distributed with the model); pass opts={'exclude': ['disp']}"
        )
    # "hal" switches the halogen-bond term off; "aes2" and "d4sc" name GFN2
    # terms that GFN1 does not have (types/base.py:594-651)
    unsupported = excl - {"disp", "hal", "aes2", "d4sc"}
    if unsupported:
        raise NotImplementedError(f"excluding {sorted(unsupported)} is not supported")
    o["exclude"] = sorted(excl)
    if o["guess"] == "eeq":
        raise ValueError(
            "the EEQ guess needs the tad-multicharge EEQ parameters, which are not distributed with "
            "the model; use guess='sad' (it changes the SCF start, not the converged result)")
    if o["guess"] != "sad":
        raise ValueError(f"unknown guess {o['guess']!r}")
    if not 1 <= int(o["damp_generations"]) <= 28:
        raise ValueError("damp_generations must be in 1..28")
    if not 1 <= int(o["broyden_memory"]) <= 29:
        raise ValueError("broyden_memory must be in 1..29")
    if int(o["anderson_restart"]) < 0:
        raise ValueError("anderson_restart must be >= 0")
    if str(o["fp64_tridiag"]).lower() not in _FP64_TRIDIAG:
        raise ValueError(f"fp64_tridiag must be one of {sorted(_FP64_TRIDIAG)}")
    return o


def engine_options(o: dict, forces: bool) -> _lib.Options:
    """``gbxtb_options`` of a resolved option dict."""
    opt = _lib.default_options()
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
    opt.mixer = _lib.MIXERS[str(o["mixer"]).lower()]
    opt.generations = int(o["damp_generations"])
    opt.damp = float(o["damp"])
    opt.damp_init = float(o["damp_init"])
    off = o["damp_diagonal_offset"]
    opt.diagonal_offset = -1.0 if off is None else float(off)
    opt.soft_start = 1 if o["damp_soft_start"] else 0
    opt.mix_guess = 1 if o["mix_guess"] else 0
    opt.damp_dynamic = 1 if o["damp_dynamic"] else 0
    opt.damp_dynamic_factor = float(o["damp_dynamic_factor"])
    opt.fermi_thresh = 0.0 if o["fermi_thresh"] is None else float(o["fermi_thresh"])
    opt.no_halogen = 1 if "hal" in o["exclude"] else 0
    opt.restart_at = int(o["anderson_restart"])
    opt.fp64_split = _FP64_TRIDIAG[str(o["fp64_tridiag"]).lower()]
    return opt


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
        o = resolve_opts(opts)
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
        return engine_options(self.opts, forces)

    def _run(self, positions: torch.Tensor, chrg=0, spin=None, forces: bool = False,
             ragged: bool = False) -> Result:
        """One engine call through ``torch.ops.gbxtb.singlepoint``.
        ``positions`` are padded like ``numbers`` or, with ``ragged``, the
        ragged ``(natoms, 3)`` positions of the plan."""
        lib = _lib.load()
        ops = _ops()
        plan = self._plan(chrg, spin)
        pos = self._check_ragged(positions) if ragged else self._ragged_positions(positions)
        dev = self.device
        ws = plan.workspace()
        opt = self._options(forces)
        tune = self.opts["autotune"]
        if plan.tuned is None and (tune is True or (tune == "auto" and plan.nmol >= 32)):
            choice = np.zeros(4, dtype=np.int32)
            stream = torch.cuda.current_stream(dev).cuda_stream
            with torch.cuda.device(dev):
                _lib.check(lib.gbxtb_plan_autotune(plan.handle, C.byref(opt), pos.data_ptr(), ws.data_ptr(),
                                                   plan.ws_bytes, stream, _lib.ptr(choice, C.c_int32)))
            plan.tuned = choice.tolist()
        iopts, fopts = _pack_options(opt)
        energy, charges, state, st = ops.singlepoint(plan.handle.value, pos, ws, iopts, fopts)
        plan.runs += 1
        status = st[:, 0].numpy().astype(np.int32)
        iters = st[:, 1].numpy().astype(np.int32)
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
        return Result(energy=energy, charges=charges, gradient=state if forces else None, status=status,
                      iterations=iters, shell_potential=vsh, fp32_passes=p32, atom_mol=plan.atom_mol)

    def _check_ragged(self, pos: torch.Tensor) -> torch.Tensor:
        if pos.dtype != torch.float64 or pos.device != self.device:
            raise ValueError("ragged positions must be float64 on the calculator's device")
        if pos.shape != (int(self._offsets[-1]), 3):
            raise ValueError(f"ragged positions must have shape ({int(self._offsets[-1])}, 3)")
        return pos.contiguous()

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

    def _key(self, positions: torch.Tensor, chrg, spin) -> tuple:
        return (positions.data_ptr(), positions._version, tuple(positions.shape), str(chrg), str(spin))

    def get_energy(self, positions: torch.Tensor, chrg=0, spin=None, **kwargs) -> torch.Tensor:
        if positions.requires_grad:
            ragged = self._ragged_positions(positions)  # differentiable gather
            return self._shape_energy(_EnergyFunction.apply(ragged, self, chrg, spin))
        key = self._key(positions, chrg, spin)
        hit = self._cache.get("energy")
        if hit is None or hit[0] != key:
            res = self._run(positions, chrg, spin)
            plan = self._plan(chrg, spin)
            self._cache = {"energy": (key, res, plan, plan.runs)}
            hit = self._cache["energy"]
        return self._shape_energy(hit[1].energy)

    def get_forces(self, positions: torch.Tensor, chrg=0, spin=None, grad_mode: str = "autograd",
                   **kwargs) -> torch.Tensor:
        """Forces -dE/dR.  After ``get_energy`` on the same positions the
        gradient comes from that call's converged state (``gbxtb_forces``),
        without a second SCF."""
        if grad_mode not in ("autograd", "backward", "functorch", "row", "analytical"):
            raise ValueError(f"unknown grad_mode {grad_mode!r}")
        key = self._key(positions, chrg, spin)
        hit = self._cache.get("energy")
        if hit is not None and hit[0] == key:
            _, res, plan, runs = hit
            if res.gradient is None and plan.runs == runs:
                lib = _lib.load()
                grad = torch.empty((plan.natom, 3), dtype=torch.float64, device=self.device)
                pos = self._ragged_positions(positions.detach())
                stream = torch.cuda.current_stream(self.device).cuda_stream
                ws = plan.workspace()
                with torch.cuda.device(self.device):
                    _lib.check(lib.gbxtb_forces(plan.handle, pos.data_ptr(), grad.data_ptr(), ws.data_ptr(),
                                                plan.ws_bytes, stream))
                res.gradient = grad
            if res.gradient is not None:
                return -self._pad_vectors(res.gradient)
        res = self._run(positions.detach(), chrg, spin, forces=True)
        plan = self._plan(chrg, spin)
        self._cache = {"energy": (key, res, plan, plan.runs)}
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
