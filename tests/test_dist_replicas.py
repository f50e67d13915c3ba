"""The multi-process bench path on the CPU: two gloo ranks run the host logic that
`bench.py --gpus N` runs under torchrun (rank discovery, slowest-rank time, whole-job rate).

The engine's single simulation does not shard: each rank runs an independent replica, and
the only collective is the max of the timings, outside the data path.
"""
import multiprocessing as mp
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    r, w, local, pg = bench.dist_setup(0, backend="gloo")
    ms_local = 100.0 + 50.0 * r  # rank 1 is the slow one
    ms = bench.rank_max(pg, ms_local)
    rate = bench.job_rate(1e9, w, ms)
    q.put((r, w, local, ms, rate))
    pg.barrier()
    pg.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_rank():
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
    assert [o[0] for o in out] == [0, 1] and all(o[1] == 2 for o in out)
    for r, w, local, ms, rate in out:
        assert local == r
        assert ms == 150.0  # both ranks see the slowest rank's time
        assert rate == pytest.approx(2e9 / 0.150 / 1e9)  # all ranks' units over that time


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench

    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    assert bench.dist_setup(1)[1:] == (1, 0, None)
    assert bench.rank_max(None, 3.5) == 3.5
    assert bench.job_rate(1e9, 1, 1000.0) == pytest.approx(1.0)
