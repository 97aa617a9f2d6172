"""The bench's multi-rank path on CPU: world size 2 over gloo (replicas: each rank steps its
own system, the job's time is the slowest rank's, the rate counts every rank's units), and the
reference arm's rule that only rank 0 runs and prints."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench._barrier(dist)
        t = bench._max_over_ranks(1.5 * (rank + 1), dist)  # rank 1 is the slower one
        rate = bench.aggregate_rate(world, 1000, 10, t)
        q.put((rank, t, rate))
        bench._barrier(dist)
    finally:
        dist.destroy_process_group()


def test_two_ranks_over_gloo():
    import torch.multiprocessing as mp
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
    # both ranks see the slowest rank's time; the rate is both ranks' units over it
    assert [t for _, t, _ in out] == [3.0, 3.0]
    assert all(abs(rate - 2 * 1000 * 10 / 3.0) < 1e-9 for _, _, rate in out)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""  # only rank 0 prints the line


def test_aggregate_rate_is_weak_scaling():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.aggregate_rate(1, 2_621_440, 50, 0.0315)
    assert bench.aggregate_rate(4, 2_621_440, 50, 0.0315) == pytest.approx(4 * one)


def test_reference_arm_line_contract():
    """The reference arm's one JSON line on rank 0: the reference's CPU path (its own cpp/ step
    loop where it was compiled here, else the oracle port) on a bounded sample, with the
    line's own metric, its cpu_baseline and an e2e without copies."""
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--cpu-sample", "20000"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "MPCD fluid particle-steps/s"
    assert d["unit"] == "particle-steps/s" and d["higher_is_better"] is True and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "20000 fluid particles" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
