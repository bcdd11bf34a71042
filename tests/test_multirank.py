"""The N>1 path of bench.py on CPU: world-size-2 gloo ranks.

The workload does not shard (every rank runs an independent replica), so the
only cross-rank step is the timing reduction: the slowest rank's time, and
the whole-job rate = all ranks' units / that time.
"""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    m = bench.max_over_ranks(times[rank])
    rate = bench.whole_job_rate(900, 3, world, m)
    out[rank] = (m, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_timing_reduction():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    times = [120.0, 150.0]
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, times, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        m, rate = out[r]
        assert m == 150.0
        assert rate == pytest.approx(2 * 900 * 3 / 0.150)


def test_single_process_is_identity():
    import bench
    assert bench.max_over_ranks(12.5) == 12.5
