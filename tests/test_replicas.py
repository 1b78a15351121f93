"""The multi-GPU host path on CPU: two gloo ranks, as ``bench.py --gpus 2``
runs them (one process per GPU, molecule shards, no collective on the data
path, the whole-job time is the maximum over ranks)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from dxtb_gb300 import replicas


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mols = replicas.batch_shard(rank, 16)
        sizes = [len(a) for a, _ in mols]
        first = mols[0][1][:2].ravel().tolist()
        # a rank-dependent "time": the job takes as long as the slowest rank
        t = replicas.max_over_ranks(1.0 + rank, world)
        dist.barrier()
        out[rank] = (sizes, first, t, replicas.whole_job_rate(16, world, 3, t))
    finally:
        dist.destroy_process_group()


def test_two_ranks_shard_and_time():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
        res = dict(out)
    (s0, p0, t0, v0), (s1, p1, t1, v1) = res[0], res[1]
    # every rank has its own molecules; rank 0 has the single-GPU workload
    assert p0 != p1
    assert s0 == [len(a) for a, _ in replicas.batch_shard(0, 16)]
    assert all(10 <= n <= 120 for n in s0 + s1)
    # both ranks report the slowest rank's time and the same whole-job rate
    assert t0 == t1 == 2.0
    assert v0 == v1 == pytest.approx(16 * 2 * 3 / 2.0)


def test_single_rank_needs_no_process_group():
    assert replicas.max_over_ranks(3.5, 1) == 3.5
    assert replicas.whole_job_rate(512, 1, 3, 1.5) == pytest.approx(1024.0)
    with pytest.raises(ValueError):
        replicas.whole_job_rate(1, 1, 1, 0.0)


def test_shards_are_disjoint_and_deterministic():
    a = replicas.batch_shard(1, 8)
    b = replicas.batch_shard(1, 8)
    c = replicas.batch_shard(2, 8)
    for (na, pa), (nb, pb) in zip(a, b):
        assert np.array_equal(na, nb) and np.array_equal(pa, pb)
    assert any(len(x[0]) != len(y[0]) or not np.allclose(x[1][:1], y[1][:1]) for x, y in zip(a, c))
