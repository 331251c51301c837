"""Multi-GPU is replicas only: N independent syntheses, no collective on the data path.  The
one cross-rank step of bench.py -- the whole-job rate from the slowest rank -- is checked here
with world_size-2 gloo process groups on the CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as tdist
    tdist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, value = bench.replica_rate(10.0 + 5.0 * rank, world, "cpu", tdist)
    tdist.barrier()
    q.put((rank, ms, value))
    tdist.destroy_process_group()


def test_replica_rate_takes_the_slowest_rank():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, value in out:
        assert ms == 15.0  # the slower rank's step time
        assert value == pytest.approx(2 * 1000.0 / 15.0)


def test_replica_rate_single_process():
    import bench
    assert bench.replica_rate(20.0, 1, "cpu") == (20.0, 50.0)
