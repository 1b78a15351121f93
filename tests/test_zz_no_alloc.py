"""gbxtb_singlepoint_noalloc against gbxtb_singlepoint, through the C ABI.

The no-allocation entry point is for callers that cannot call cudaMalloc
when they compute (a memory pool that must not grow, a real-time loop, a
plugin callback handed only a stream).  It uses a fixed device array inside
the library as scratch instead of a caller workspace.  Two calls in a row
must give the results of the workspace entry point within the parity
tolerances of the other GPU tests, and plans larger than the array must be
refused with a clear error.

This file is named to be collected last; it builds its own context and
plans, so it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from dxtb_gb300 import molgen

pytestmark = pytest.mark.gpu

E_TOL = 1e-8
F_TOL = 1e-6
Q_TOL = 1e-7


def small_batch():
    """The 20-atom single-point molecule and the small molecules of the
    10-120-atom batch workload (a plan that fits the fixed scratch)."""
    mols = molgen.c1_single() + [m for m in molgen.c2_batch(64) if len(m[0]) <= 30][:5]
    return mols


def make_plan(mols):
    from dxtb_gb300.calculator import Plan, _Context

    ctx = _Context.get(torch.cuda.current_device())
    nums = np.concatenate([m[0] for m in mols]).astype(np.int32)
    offs = np.concatenate([[0], np.cumsum([len(m[0]) for m in mols])]).astype(np.int64)
    return Plan(ctx, nums, offs, np.zeros(len(mols)), None)


def options(profile=0):
    from dxtb_gb300 import _lib

    o = _lib.default_options()
    o.maxiter, o.want_forces = 300, 1
    o.x_atol, o.x_atol_max = 1e-10, 1e-10
    o.mixer = _lib.MIXER_BROYDEN
    o.profile = profile
    o.mixed_precision = 1
    return o


def outputs(plan):
    dev = torch.device("cuda", torch.cuda.current_device())
    return (torch.full((plan.nmol,), np.nan, dtype=torch.float64, device=dev),
            torch.full((plan.natom,), np.nan, dtype=torch.float64, device=dev),
            torch.full((plan.natom, 3), np.nan, dtype=torch.float64, device=dev))


def test_noalloc_matches_workspace_entry_point():
    from dxtb_gb300 import _lib

    lib = _lib.load()
    mols = small_batch()
    plan = make_plan(mols)
    assert plan.ws_bytes <= _lib.NOALLOC_SCRATCH_BYTES
    pos = torch.tensor(np.concatenate([m[1] for m in mols]), device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    opt = options()

    # the existing entry point with a caller workspace
    e0, q0, g0 = outputs(plan)
    ws = plan.workspace()
    _lib.check(lib.gbxtb_singlepoint(plan.handle, C.byref(opt), pos.data_ptr(), e0.data_ptr(), q0.data_ptr(),
                                     g0.data_ptr(), ws.data_ptr(), plan.ws_bytes, stream))
    st = np.zeros(plan.nmol, dtype=np.int32)
    _lib.check(lib.gbxtb_get_status(plan.handle, _lib.ptr(st, C.c_int32), None))
    assert (st == 0).all()

    # two calls in a row without a workspace; the first one on this plan
    # after the workspace call above instantiates the plan's pass graphs for
    # the fixed scratch, the second must take no device memory at all
    for call in range(2):
        e1, q1, g1 = outputs(plan)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        _lib.check(lib.gbxtb_singlepoint_noalloc(plan.handle, C.byref(opt), pos.data_ptr(), e1.data_ptr(),
                                                 q1.data_ptr(), g1.data_ptr(), stream))
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free0
        st = np.zeros(plan.nmol, dtype=np.int32)
        _lib.check(lib.gbxtb_get_status(plan.handle, _lib.ptr(st, C.c_int32), None))
        assert (st == 0).all()
        assert torch.isfinite(e1).all() and torch.isfinite(g1).all()
        assert (e1 - e0).abs().max().item() < E_TOL
        assert (q1 - q0).abs().max().item() < Q_TOL
        assert (g1 - g0).abs().max().item() < F_TOL


def test_noalloc_refuses_oversized_plans_and_profiling():
    from dxtb_gb300 import _lib

    lib = _lib.load()
    big = make_plan(molgen.c2_batch(64))
    assert big.ws_bytes > _lib.NOALLOC_SCRATCH_BYTES
    e, q, g = outputs(big)
    pos = torch.zeros((big.natom, 3), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.gbxtb_singlepoint_noalloc(big.handle, C.byref(options()), pos.data_ptr(), e.data_ptr(),
                                       q.data_ptr(), g.data_ptr(), stream)
    assert rc == -4  # GBXTB_ERR_WORKSPACE
    assert b"bytes of scratch" in lib.gbxtb_last_error()
    small = make_plan(small_batch())
    rc = lib.gbxtb_singlepoint_noalloc(small.handle, C.byref(options(profile=1)), pos.data_ptr(), e.data_ptr(),
                                       q.data_ptr(), g.data_ptr(), stream)
    assert rc == -1  # GBXTB_ERR_ARG
    assert torch.isnan(e).all()  # nothing ran


def test_noalloc_refuses_a_plan_of_another_device():
    """The scratch is the current device's array: a plan made on another
    device is refused before anything runs."""
    if torch.cuda.device_count() < 2:
        pytest.skip("needs two GPUs")
    from dxtb_gb300 import _lib

    lib = _lib.load()
    with torch.cuda.device(1):
        plan = make_plan(small_batch())
    with torch.cuda.device(0):
        e, q, g = outputs(plan)
        pos = torch.zeros((plan.natom, 3), dtype=torch.float64, device="cuda:0")
        rc = lib.gbxtb_singlepoint_noalloc(plan.handle, C.byref(options()), pos.data_ptr(), e.data_ptr(),
                                           q.data_ptr(), g.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == -1  # GBXTB_ERR_ARG
    assert b"not the device of the plan" in lib.gbxtb_last_error()
