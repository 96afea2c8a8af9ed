"""Multi-rank path of the benchmark (replicas only: no data-path collective):
two gloo ranks on CPU synchronise and combine their timings."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    from muphfasa_gb300 import replicas
    dist = replicas.init("gloo")
    replicas.barrier(dist)
    t = replicas.max_over_ranks(dist, 1.0 + rank)
    cells = replicas.sum_over_ranks(dist, 1000.0 * (rank + 1))
    q.put((rank, t, cells))
    dist.destroy_process_group()


def test_two_rank_timing_combination():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 3000.0), (1, 2.0, 3000.0)]


def test_single_rank_is_identity():
    from muphfasa_gb300 import replicas
    assert replicas.init() is None or int(os.environ.get("WORLD_SIZE", "1")) > 1
    assert replicas.max_over_ranks(None, 3.5) == 3.5
    assert replicas.sum_over_ranks(None, 2.0) == 2.0
