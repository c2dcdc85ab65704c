"""bench.py's multi-rank path on the CPU: two gloo ranks through the same
set-up, barrier and max-over-ranks timing that torchrun runs use on GPUs
(replicas only: no collective on the data path)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), SMPC_DIST_BACKEND="gloo")
    sys.path.insert(0, ROOT)
    import bench
    w, r, _, dist = bench.dist_setup(None)
    bench.barrier(dist)
    ms = bench.max_over_ranks(dist, 10.0 + r)  # rank 1 is the slower one
    value = bench.job_value(1000, 5, w, ms)
    bench.barrier(dist)
    dist.destroy_process_group()
    q.put((r, w, ms, value))


def test_two_gloo_ranks_time_by_the_slowest():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, ms, value in out:
        assert w == 2 and ms == 11.0
        assert value == pytest.approx(1000 * 5 * 2 / 0.011)  # whole job over the slowest rank
