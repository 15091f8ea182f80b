"""The multi-process path of bench.py on CPU: two gloo ranks, each a
replica, the slowest rank's time and the whole-job rate."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    r, w, local, dist = bench.dist_setup(backend="gloo")
    bench.barrier(dist)
    t = bench.max_over_ranks(dist, 1.0 + rank)   # rank 1 is the slower one
    rate = bench.replica_rate(w, 100, 10, t)
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, t, rate))


def test_two_gloo_ranks_take_the_slowest_time():
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
    assert [o[0] for o in out] == [0, 1]
    for r, w, t, rate in out:
        assert w == 2 and t == 2.0
        assert rate == 2 * 100 * 10 / 2.0


def test_single_process_has_no_group():
    import bench
    r, w, local, dist = bench.dist_setup()
    assert (r, w, dist) == (0, 1, None)
    assert bench.max_over_ranks(None, 3.5) == 3.5
