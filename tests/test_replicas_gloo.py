"""The N-GPU bookkeeping of bench.py (replicas: one process per GPU, independent jobs, the
slowest rank's time) on CPU with two gloo ranks over 127.0.0.1."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from slater_stoch_gb300.replicas import job_seed, max_over_ranks, whole_job_throughput


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        per_rank_ms = [2100.0, 2175.0][rank]  # the ranks' summed step times differ
        dist.barrier()
        ms = max_over_ranks(per_rank_ms, world, dist, "cpu") / 3
        out[rank] = (ms, whole_job_throughput(61776, world, ms * 1e-3), job_seed(1, rank))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    ms0, v0, s0 = res[0]
    ms1, v1, s1 = res[1]
    assert ms0 == ms1 == pytest.approx(2175.0 / 3)
    assert v0 == v1 == pytest.approx(2 * 61776 / (2175.0 / 3 * 1e-3))
    assert s0 != s1  # independent walker streams


def test_single_rank_is_identity():
    assert max_over_ranks(5.0, 1) == 5.0
    assert whole_job_throughput(100, 1, 2.0) == 50.0


def _lost_rank(rank, world, port, out):
    import datetime
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=datetime.timedelta(seconds=10))
    if rank == 1:
        os._exit(0)  # the rank leaves between steps, before the timing reduction
    try:
        max_over_ranks(1.0, world, dist, "cpu")
        out[rank] = "no error"
    except Exception as e:  # the lost peer surfaces as an error, not a hang
        out[rank] = "error: " + type(e).__name__


def test_lost_rank_is_reported():
    """A rank that exits between steps: the surviving rank's next collective ends with an error
    (peer closed or the 10 s process-group timeout) instead of hanging."""
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_lost_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        assert all(p.exitcode is not None for p in procs)
        res = dict(out)
    assert res.get(0, "").startswith("error")
