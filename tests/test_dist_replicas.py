"""The multi-rank path of bench.py (replicas: one image per rank, no
collective on the data path): barrier and max-over-ranks timing on two gloo
ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, ws, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(ws), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), BENCH_BACKEND="gloo")
    import bench
    w, r, _ = bench.dist_setup()
    bench.barrier(w)
    my_ms = 10.0 + 5.0 * r  # rank 1 is the slower replica
    ms = bench.allmax(w, my_ms)
    q.put((r, w, ms, bench.replica_value(w, 3, 1000, ms)))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_replicas_max_over_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(60)
        assert p.exitcode == 0
    for r, w, ms, value in out:
        assert w == 2 and ms == 15.0
        assert value == pytest.approx(2 * 3 * 1000 / 0.015 / 1e6)
