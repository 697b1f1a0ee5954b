"""The multi-GPU form of bench.py is replicas only: every rank times its own
copy of the workload, the job's time is the maximum over ranks and the value
counts every rank's particles.  Checked here on CPU with two gloo ranks
(127.0.0.1 rendezvous): the all-reduce takes the slowest rank's time, and the
aggregate value follows from it."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = [120.0, 135.5][rank]  # rank 1 is the slow replica
    ms = bench.max_over_ranks(local_ms, world, torch.device("cpu"))
    out[rank] = (ms, bench.replica_value(65536, 30, ms / 1e3, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        ms, value = res[r]
        assert ms == 135.5
        assert value == pytest.approx(2 * 65536 * 30 / 0.1355)


def test_single_rank_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1, None) == 3.5
    assert bench.replica_value(100, 10, 2.0, 1) == 500.0
