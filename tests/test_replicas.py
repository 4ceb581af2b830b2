"""CPU test of the multi-GPU replica path (world_size 2, gloo): the timed
region's barrier, the max-over-ranks time and the whole-job rate that
bench.py reports for N > 1."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from exactclosure_gb300 import replicas

    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = replicas.world()
    dist.barrier()
    t = replicas.slowest(1.0 + rank)  # rank 1 is the slowest
    rate = replicas.job_rate(1000.0, t, w)
    q.put((r, w, lr, t, rate))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_rate():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, w, lr, t, rate in out:
        assert w == 2 and lr == r
        assert t == pytest.approx(2.0)
        assert rate == pytest.approx(1000.0 * 2 / 2.0)


def test_single_process_identity():
    from exactclosure_gb300 import replicas

    assert replicas.slowest(3.5) == 3.5
    assert replicas.job_rate(10.0, 2.0, 1) == 5.0
