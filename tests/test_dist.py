"""The multi-GPU form is replicas only (independent solves per rank, no
data-path collective).  This checks bench.py's host logic for N > 1 with a
world-size-2 gloo group on CPU: rendezvous, barrier, max-over-ranks timing
and the whole-job value."""
import multiprocessing as mp
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    r, w, local, pg = bench.dist_setup(world)
    bench.barrier(pg)
    ms = 100.0 * (rank + 1)                 # rank 1 is the slow one
    mx = bench.allmax(pg, ms)
    q.put((r, w, mx, bench.replica_value(w, 20, mx)))
    pg.destroy_process_group()


def test_replicas_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, mx, val in out:
        assert w == 2 and mx == 200.0
        assert val == pytest.approx(2 * 20 / 0.2)
