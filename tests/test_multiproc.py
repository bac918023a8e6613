"""The N > 1 path of bench.py on CPU: two gloo ranks run the replica
harness (barrier, max of the per-rank times, sum of the per-rank bins) that
bench.py uses on GPUs, and one rank that raises is reported on the host
without a hang."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out, fail_rank):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    d = bench.Dist(world, rank, backend="gloo")
    try:
        if rank == fail_rank:
            raise RuntimeError("injected failure on rank %d" % rank)
        d.barrier()
        t = 1.0 + rank          # rank-local elapsed seconds
        bins = 1e9 * (rank + 1)  # rank-local bin-updates
        tmax = d.max(t)
        ball = d.sum(bins)
        out[rank] = (tmax, ball, ball / tmax)
        d.barrier()
    finally:
        d.close()


def test_replica_aggregation_two_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    manager = mp.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, out, -1)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        tmax, ball, v = out[r]
        assert tmax == 2.0 and ball == 3e9 and v == 1.5e9
    import bench

    assert bench.aggregate([1e9, 2e9], [1.0, 2.0]) == 1.5e9


def test_failed_rank_is_reported():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    manager = mp.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, out, 1)) for r in range(2)]
    for p in procs:
        p.start()
    procs[1].join(60)
    assert procs[1].exitcode != 0          # the failing rank exits with an error
    procs[0].join(5)
    if procs[0].is_alive():                # the survivor would wait in the barrier:
        procs[0].terminate()               # the host ends it (no GPU involved)
        procs[0].join(30)
    assert 1 not in out
