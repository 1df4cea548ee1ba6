"""The N-GPU bench path runs N independent replicas (the path is not sharded
across GPUs here): the barrier and the max-over-ranks timing, exercised with
two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    dist.barrier()
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world)
    value = bench.whole_job_value(1000, 4, ms, world)
    out.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [15.0, 15.0]
    # two replicas of 1000 DOF x 3 stages x 4 steps in 15 ms
    assert got[0][2] == pytest.approx(2 * 1000 * 3 * 4 / 0.015)
