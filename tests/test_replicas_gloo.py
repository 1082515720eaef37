"""Multi-GPU runs of the projection are independent replicas (the reference
builds the whole system on every rank): bench.py only needs a barrier and
the max-over-ranks of the timed total.  Checked here with two gloo ranks on
the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import sys
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist = bench.init_dist(world)
    bench.barrier(dist)
    v = bench.allreduce_max(dist, float(rank + 1) * 1.5)
    out.put((rank, v, bench.dist_env()))
    bench.barrier(dist)
    dist.destroy_process_group()


def test_replica_timing_is_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, v, env in res:
        assert v == 3.0
        assert env == (2, rank, rank)
