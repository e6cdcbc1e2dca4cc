"""Multi-rank handling of the benchmark on CPU: two gloo ranks agree on the
timed region and reduce (max time, summed work), as N GPU replicas do."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    from unsflow2d_gb300 import replicas
    dist = replicas.init("gloo")
    replicas.barrier(dist)
    units, secs = replicas.reduce_timing(dist, units=1000.0 * (rank + 1), seconds=0.5 + rank, device="cpu")
    q.put((rank, units, secs))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timing():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(world))
    for _, units, secs in got:
        assert units == pytest.approx(3000.0) and secs == pytest.approx(1.5)


def test_single_process_is_a_no_op():
    from unsflow2d_gb300 import replicas
    assert replicas.reduce_timing(None, 10.0, 2.0) == (10.0, 2.0)
