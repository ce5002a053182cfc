"""The N>1 path of bench.py (independent replicas, one per GPU) on CPU: two
gloo ranks check the barrier, the max-over-ranks time and the summed work."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "WORLD_SIZE": str(world),
                       "RANK": str(rank), "LOCAL_RANK": str(rank), "PF_DIST_BACKEND": "gloo"})
    import bench
    r, w, local, dist = bench.dist_init(world)
    try:
        bench.barrier(dist)
        t = bench.dist_max(dist, local, 1.0 + rank)        # rank times 1.0 and 2.0 s
        units = bench.dist_sum(dist, local, 1000 * (rank + 1))
        q.put((r, w, t, units, units / t))
    finally:
        dist.destroy_process_group()


def test_two_replicas_aggregate_with_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for r, w, t, units, value in out:
        assert w == 2
        assert t == 2.0                  # the slowest rank's time
        assert units == 3000             # both ranks' work
        assert value == 1500.0           # whole-job throughput
