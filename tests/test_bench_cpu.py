"""The benchmark's multi-rank plumbing on CPU (gloo, world size 2).

bench.py runs one independent replica per GPU under torchrun (the path has
no exchange step); ranks meet only to take the slowest rank's timings and to
let rank 0 print the single JSON line.  These tests cover that host logic
without a GPU: the max-over-ranks reduction under gloo with two processes,
the whole-job rate, and the reference arm's rank behaviour (rank 0 prints
one line, other ranks exit 0 silently)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r: step 10 + r ms, sweep 5 - r ms, e2e 1.5 s on every rank
        got = bench.max_over_ranks([10.0 + rank, 5.0 - rank, 1.5], world, "cpu")
        dist.barrier()
        out.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [11.0, 5.0, 1.5]


def test_job_rate_counts_every_replica():
    sys.path.insert(0, ROOT)
    import bench
    one = bench.job_rate(1, 2048 * 1024, 1000, 0.5)
    assert one == pytest.approx(2048 * 1024 * 1000 / 0.5 / 1e9)
    assert bench.job_rate(4, 2048 * 1024, 1000, 0.5) == pytest.approx(4 * one)


def _reference_arm(rank, world):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
               MASTER_ADDR="127.0.0.1")
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                           "--gpus", str(world), "--steps", "1", "--warmup", "3"],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_prints_on_rank_0_only():
    p1 = _reference_arm(1, 2)
    assert p1.returncode == 0, p1.stderr
    assert p1.stdout.strip() == ""
    p0 = _reference_arm(0, 2)
    assert p0.returncode == 0, p0.stderr
    lines = [ln for ln in p0.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == line["metric"]
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_both_arms_report_the_same_config():
    """The reference arm and the GPU arm describe the workload with the same
    `config` dict (the arithmetic each runs is the line's own `precision`
    key), so the two lines compare like for like."""
    sys.path.insert(0, ROOT)
    import bench
    w = bench.workload()
    cfg = bench.config_json(w)
    assert cfg == bench.config_json(bench.workload())
    assert "precision" not in cfg and "l2" not in cfg
    assert (cfg["n_x"], cfg["n_y"], cfg["scheme"], cfg["riemann"], cfg["boundary"]) == \
        (2048, 1024, "MUSCL", "HLLC", "IDWBaseGFM")
