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


def test_reference_arm_line():
    # the reference arm on the host cores: the oracle's restatement on every
    # replica of the workload, warm-up honoured, one JSON line with the keys
    # the contract names
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--workload", "single_star_20", "--steps", "2", "--warmup", "3"],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["steps"] == 2 and line["warmup"] == 3
    assert line["config"]["replicas"] == 1 and line["config"]["particles"] == 80121
    assert line["value"] > 0 and line["e2e"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
