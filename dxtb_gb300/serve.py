"""Continuous batching of GFN1-xTB single points with forces.

A ``Server`` keeps one slot pool (``gbxtb_pool_*`` in ``include/gbxtb.h``)
per molecule-size class on the GPU.  Requests are queued on submission and
admitted into a free slot of the smallest class that fits them, between any
two SCF passes; every ``step`` runs one SCF pass for every molecule on the
device (the pools of the size classes on their own CUDA streams, so their
work overlaps), computes the forces of the molecules that converged, and
hands their results back.  Converged molecules leave at once and their slots
take the next requests, so requests that arrive while others are on the GPU
join the running batch instead of waiting for it to drain.

Slot counts follow a device-memory budget: a slot of capacity N AOs holds
its molecule's SCF state (about 14 N^2 doubles).  A molecule goes to the
smallest class whose atom, shell and orbital capacity it fits; one that fits
no class is refused at submission.

Stragglers: with ``evict_after`` set, a molecule still iterating after that
many passes leaves its slot (``gbxtb_pool_evict``) when a queued request
waits for a slot of its class, and is solved again from the start in a
small pool of the same class reserved for such molecules.
A fresh SCF of the same molecule takes the same path, so its result is the
one it would have had; the main slots stop being held for up to ``maxiter``
passes by molecules that converge slowly or not at all.

Per molecule the result is the single point of
``dxtb_gb300.GFN1Calculator`` (the reference's ``get_energy`` /
``get_forces``, ``calculators/types/energy.py:78-402``,
``types/autograd.py:82-201``); the reference itself has no serving form.
"""
from __future__ import annotations

import ctypes as C
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, params
from .calculator import _Context, engine_options, resolve_opts

__all__ = ["Server", "Request", "size_class_capacity", "molecule_size"]

# (max atoms, share of the memory budget) of the default size classes
DEFAULT_CLASSES = ((32, 0.15), (100, 0.25), (200, 0.3), (400, 0.3))


def size_class_capacity(max_atoms: int) -> tuple[int, int]:
    """Shells and AOs reserved for a slot of ``max_atoms`` atoms: enough for
    molecules of elements with s and p valence shells (H-Ne and the heavier
    main-group elements without d shells: two shells, at most four AOs per
    atom); larger molecules go to a larger class."""
    return 2 * max_atoms, 4 * max_atoms


def molecule_size(numbers) -> tuple[int, int]:
    """(shells, AOs) of a molecule."""
    elems = params.raw()["elements"]
    nsh = nao = 0
    for z in np.asarray(numbers).tolist():
        el = elems.get(str(int(z)))
        if el is None:
            raise ValueError(f"atomic number {z} has no GFN1 parameters")
        nsh += len(el["shells"])
        nao += sum(2 * s["l"] + 1 for s in el["shells"])
    return nsh, nao


def slot_bytes(max_atoms: int) -> int:
    nsh, nao = size_class_capacity(max_atoms)
    # workspace: 8 + 5 matrices of nao^2 doubles, the shell-pair Coulomb
    # matrix, mixer history and vectors
    return 8 * (13 * nao * nao + nsh * nsh + 60 * nsh + 20 * nao) + 64 * max_atoms


@dataclass
class Request:
    id: int
    numbers: np.ndarray
    positions: np.ndarray
    charge: float = 0.0
    spin: int | None = None
    t_submit: float = 0.0
    t_admit: float | None = None
    t_done: float | None = None
    energy: float | None = None
    gradient: np.ndarray | None = None
    charges: np.ndarray | None = None
    status: int | None = None
    iterations: int | None = None
    size_class: int | None = None
    passes: int = 0        # SCF passes run in its current slot
    evicted: bool = False  # moved to a straggler pool
    dims: tuple[int, int] | None = None  # (shells, AOs)

    @property
    def latency(self) -> float | None:
        return None if self.t_done is None else self.t_done - self.t_submit


class _Pool:
    """One size class: a ``gbxtb_pool`` and its stream."""

    def __init__(self, ctx: _Context, opts: _lib.Options, max_atoms: int, nslots: int, device: int,
                 priority: int = 0):
        self.lib = _lib.load()
        self.max_atoms = max_atoms
        self.nslots = nslots
        nsh, nao = size_class_capacity(max_atoms)
        self.cap_sh, self.cap_ao = nsh, nao
        h = C.c_void_p()
        nbytes = C.c_size_t()
        with torch.cuda.device(device):
            _lib.check(self.lib.gbxtb_pool_create(ctx.handle, C.byref(opts), nslots, max_atoms, nsh, nao,
                                                  C.byref(h), C.byref(nbytes)))
            # smaller size classes get higher stream priority: when SMs free
            # up, their short passes go before the long passes of large
            # molecules, which keeps the latency of small requests low
            self.stream = torch.cuda.Stream(device, priority=priority)
        self.handle = h
        self.device_bytes = int(nbytes.value)
        self.requests: dict[int, Request] = {}  # slot -> request
        self._ended = np.zeros(nslots, dtype=np.int32)
        self.launched = False

    def free(self) -> int:
        return int(self.lib.gbxtb_pool_free_slots(self.handle))

    def fits(self, req: Request) -> bool:
        if req.dims is None:
            req.dims = molecule_size(req.numbers)
        nsh, nao = req.dims
        return len(req.numbers) <= self.max_atoms and nsh <= self.cap_sh and nao <= self.cap_ao

    def evict(self, slot: int) -> Request:
        """Take the molecule of `slot` out (between steps) and return its request."""
        _lib.check(self.lib.gbxtb_pool_evict(self.handle, int(slot), C.c_void_p(self.stream.cuda_stream)))
        return self.requests.pop(slot)

    def admit(self, req: Request) -> bool:
        num = np.ascontiguousarray(req.numbers, dtype=np.int32)
        pos = np.ascontiguousarray(req.positions, dtype=np.float64)
        slot = C.c_int32()
        rc = self.lib.gbxtb_pool_admit(self.handle, len(num), _lib.ptr(num, C.c_int32), _lib.ptr(pos, C.c_double),
                                       float(req.charge), -1 if req.spin is None else int(req.spin),
                                       C.byref(slot))
        if rc == -4:  # GBXTB_ERR_WORKSPACE: does not fit (or no free slot)
            return False
        _lib.check(rc)
        self.requests[slot.value] = req
        return True

    def launch(self) -> None:
        _lib.check(self.lib.gbxtb_pool_step_launch(self.handle, C.c_void_p(self.stream.cuda_stream)))
        self.launched = True

    def ready(self) -> bool:
        rc = self.lib.gbxtb_pool_step_poll(self.handle)
        if rc < 0:
            _lib.check(rc)
        return rc == 1

    def finish(self) -> list[Request]:
        n = C.c_int32()
        it = C.c_int32()
        _lib.check(self.lib.gbxtb_pool_step_finish(self.handle, _lib.ptr(self._ended, C.c_int32), C.byref(n),
                                                   C.byref(it)))
        self.launched = False
        self.iterating = it.value
        done = []
        for k in range(n.value):
            slot = int(self._ended[k])
            req = self.requests.pop(slot)
            nat = len(req.numbers)
            e = np.zeros(1)
            q = np.zeros(nat)
            g = np.zeros((nat, 3))
            st = C.c_int32()
            its = C.c_int32()
            _lib.check(self.lib.gbxtb_pool_result(self.handle, slot, _lib.ptr(e, C.c_double), _lib.ptr(q, C.c_double),
                                                  _lib.ptr(g, C.c_double), C.byref(st), C.byref(its)))
            req.energy, req.charges, req.gradient = float(e[0]), q, g
            req.status, req.iterations = int(st.value), int(its.value)
            done.append(req)
        return done

    @property
    def busy(self) -> bool:
        return bool(self.requests)

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.handle.value:
                self.lib.gbxtb_pool_destroy(self.handle)
        except Exception:  # pragma: no cover - interpreter shutdown
            pass


class Server:
    """Continuous-batching GFN1 single points with forces on one GPU.

    ``classes``: ``(max_atoms, nslots)`` pairs, or ``(max_atoms, share)``
    pairs with ``share`` < 1 of a ``memory_gb`` device-memory budget.
    ``opts``: calculator options (``dxtb_gb300.calculator.DEFAULT_OPTS``)."""

    def __init__(self, classes=DEFAULT_CLASSES, opts: dict | None = None, memory_gb: float = 16.0,
                 device: int | None = None, max_slots: int = 512, evict_after: int | None = None,
                 straggler_share: float = 0.15):
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        o = resolve_opts(opts)
        if o["profile"]:
            raise ValueError("profiling is not available for served requests")
        opt = engine_options(o, forces=True)
        self.opts = o
        ctx = _Context.get(device)
        self.evict_after = evict_after
        self.pools: list[_Pool] = []
        self.slow: list[_Pool] = []  # straggler pools, one per class (with evict_after)
        for rank, (max_atoms, amount) in enumerate(sorted(classes)):
            amount = float(amount)
            if amount < 1:
                nslots = int(amount * memory_gb * 1e9 // slot_bytes(max_atoms))
            else:
                nslots = int(amount)
            nslots = max(1, min(max_slots, nslots))
            nslow = max(1, int(round(straggler_share * nslots))) if evict_after else 0
            # priority -1 (high) for the two smallest classes, 0 (normal) for the rest
            prio = -1 if rank <= 1 else 0
            self.pools.append(_Pool(ctx, opt, int(max_atoms), max(1, nslots - nslow), device, priority=prio))
            if nslow:
                self.slow.append(_Pool(ctx, opt, int(max_atoms), nslow, device, priority=prio))
        self.queue: deque[Request] = deque()
        self.slow_queue: deque[Request] = deque()
        self.completed: list[Request] = []
        self._next_id = 0
        self.steps = 0

    @property
    def device_bytes(self) -> int:
        return sum(p.device_bytes for p in self.pools + self.slow)

    def submit(self, numbers, positions, charge: float = 0.0, spin: int | None = None,
               t_submit: float | None = None) -> Request:
        """Queue one single point (host arrays; positions in bohr)."""
        num = np.asarray(numbers)
        nsh, nao = molecule_size(num)
        big = self.pools[-1]
        if len(num) > big.max_atoms or nsh > big.cap_sh or nao > big.cap_ao:
            raise ValueError(f"molecule with {len(num)} atoms, {nsh} shells and {nao} orbitals exceeds the "
                             f"largest size class ({big.max_atoms} atoms, {big.cap_sh} shells, {big.cap_ao} orbitals)")
        req = Request(self._next_id, num, np.asarray(positions, dtype=np.float64), float(charge), spin,
                      time.perf_counter() if t_submit is None else t_submit, dims=(nsh, nao))
        self._next_id += 1
        self.queue.append(req)
        return req

    def submit_file(self, path, t_submit: float | None = None) -> Request:
        """Queue one single point read from a ``coord`` or ``xyz`` file, with
        the charge and unpaired electrons of the ``.CHRG`` / ``.UHF`` files
        beside it (``dxtb_gb300.io.read_molecule``)."""
        from .io import read_molecule

        mol = read_molecule(path)
        return self.submit(mol["numbers"], mol["positions"], mol["charge"], mol["uhf"], t_submit)

    def _admit(self) -> None:
        for queue, pools in ((self.queue, self.pools), (self.slow_queue, self.slow)):
            waiting = deque()
            while queue:
                req = queue.popleft()
                placed = False
                for c, pool in enumerate(pools):
                    if pool.fits(req) and pool.free() > 0 and pool.admit(req):
                        if req.t_admit is None:
                            req.t_admit = time.perf_counter()
                        req.size_class = c
                        req.passes = 0
                        placed = True
                        break
                if not placed:
                    waiting.append(req)
            queue.extend(waiting)

    def _evict_stragglers(self, pool: "_Pool") -> None:
        """After a finished step of a main pool: molecules that have run
        evict_after passes there move to the straggler pools, but only as
        many as queued requests that fit this pool need slots beyond its
        free ones, longest-running first.  A molecule with nothing waiting
        for its slot keeps it (an evicted molecule starts again from the
        guess, so eviction without a waiting request only costs passes)."""
        for req in pool.requests.values():
            req.passes += 1
        if not self.evict_after:
            return
        # queued requests that the next admission leaves waiting and that
        # this pool could take (admission places a request in the first
        # class that fits it and has a free slot)
        free = [p.free() for p in self.pools]
        need = 0
        for r in self.queue:
            c = next((c for c, p in enumerate(self.pools) if free[c] > 0 and p.fits(r)), None)
            if c is not None:
                free[c] -= 1
            elif pool.fits(r):
                need += 1
        if need <= 0:
            return
        slow = sorted(((req.passes, slot) for slot, req in pool.requests.items() if req.passes >= self.evict_after),
                      reverse=True)
        for _, slot in slow[:need]:
            req = pool.evict(slot)
            req.evicted = True
            self.slow_queue.append(req)

    def step(self, wait: bool = True) -> list[Request]:
        """Advance every pool at its own pace: collect the pools whose step
        has completed, admit queued requests into free slots, and launch the
        next step of every idle pool that holds molecules (the size classes
        overlap on their streams; a pool of small molecules does not wait
        for the slow passes of large ones).  Returns the requests that
        completed.  ``wait``: block until at least one pool's step ends
        when every busy pool is still running."""
        done = []
        while True:
            for p in self.pools + self.slow:
                if p.launched and p.ready():
                    done.extend(p.finish())
                    if self.evict_after and p in self.pools:
                        self._evict_stragglers(p)
            self._admit()
            for p in self.pools + self.slow:
                if not p.launched and p.busy:
                    p.launch()
                    self.steps += 1
            if done or not wait or not any(p.launched for p in self.pools + self.slow):
                break
            time.sleep(5e-5)
        now = time.perf_counter()
        for r in done:
            r.t_done = now
        self.completed.extend(done)
        return done

    @property
    def idle(self) -> bool:
        return (not self.queue and not self.slow_queue
                and not any(p.busy or p.launched for p in self.pools + self.slow))

    def run_until_idle(self, max_steps: int = 100000) -> list[Request]:
        out = []
        for _ in range(max_steps):
            if self.idle:
                break
            out.extend(self.step())
        return out


def latency_summary(requests) -> dict:
    lat = np.array([r.latency for r in requests if r.latency is not None])
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None}
    return {"p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3)}
