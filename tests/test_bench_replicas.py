"""bench.py's replica mode (N > 1 under torchrun) on CPU: two gloo ranks.

Each rank steps its own DEMs (weak scaling), so the whole job's figure is the
cells of all ranks over the slowest rank's time.  The ranks read RANK /
WORLD_SIZE / LOCAL_RANK from the environment the way torchrun sets them, join
one process group over 127.0.0.1 and reduce through the same helpers the
timed region uses.  No GPU is touched.
"""
import multiprocessing as mp
import os
import socket

import pytest

pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    try:
        import bench
        r, w, local = bench.dist_env()
        dist = bench.init_dist(w, local, backend="gloo")
        # rank 1 is the slower replica and steps twice the cells
        value, ms_max, cells_all = bench.whole_job(dist, cells=1000 * (r + 1), steps=10, ms=50.0 + 25.0 * r)
        bench.barrier(dist)
        dist.destroy_process_group()
        q.put((r, w, local, value, ms_max, cells_all))
    except Exception as e:  # reported to the parent
        q.put(("error", repr(e)))


def test_two_gloo_replicas_report_the_whole_job():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(x[0] != "error" for x in res), res
    for r, w, local, value, ms_max, cells_all in res:
        assert w == 2 and local == r
        assert ms_max == 75.0 and cells_all == 3000.0  # max over ranks, sum over ranks
        assert value == pytest.approx(3000.0 * 10 / 0.075)


def test_single_process_needs_no_group():
    import bench
    assert bench.init_dist(1, 0) is None
    assert bench.whole_job(None, cells=500, steps=4, ms=20.0) == (500 * 4 / 0.02, 20.0, 500)
