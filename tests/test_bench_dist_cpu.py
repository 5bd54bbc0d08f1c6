"""The bench's multi-rank path on CPU: the cross-rank reduction over two gloo
ranks, and the reference arm launched as two ranks by torch.distributed.run
(rank 0 alone works and prints one line; the other exits 0)."""

from __future__ import annotations

import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_worker(rank, world, port, out):
    sys.path.insert(0, str(ROOT))
    import bench

    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                                         rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
        value = bench.whole_job_gvu_s(world, 3, 2e9, slowest)
        out.put((rank, slowest, value))
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    # both ranks see the slower rank's 15 ms; 2 ranks x 3 steps x 2e9 updates / 15 ms
    assert [g[1] for g in got] == [15.0, 15.0]
    assert abs(got[0][2] - 2 * 3 * 2e9 / 0.015 / 1e9) < 1e-9
    assert got[0][2] == got[1][2]


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(7.5, 1, torch.device("cpu")) == 7.5
    assert bench.whole_job_gvu_s(1, 1, 1e9, 1000.0) == 1.0


def test_reference_arm_as_two_ranks_prints_one_line():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node",
           "2", "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--size", "16", "--angles", "8", "--steps",
           "1", "--warmup", "1"]
    res = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_metric_and_l2_note_follow_the_configuration():
    """The headline configuration keeps the published metric's name; other
    sizes name their own, and the L2 note says whether the inputs exceed L2
    (the steps are not separated by an L2 flush)."""
    import argparse

    sys.path.insert(0, str(ROOT))
    import bench

    head = argparse.Namespace(size=512, angles=192)
    assert bench.metric_name(head) == bench.METRIC
    small = argparse.Namespace(size=128, angles=192)
    assert "128³/192" in bench.metric_name(small)
    assert bench.metric_name(small) != bench.METRIC
    assert bench.l2_note(512**3 * 4, 192 * 512 * 512 * 4).startswith("inputs larger than L2")
    assert "warm-L2" in bench.l2_note(128**3 * 4, 192 * 128 * 128 * 4)
    # one input below L2 is enough for the warm-L2 label
    assert "warm-L2" in bench.l2_note(512**3 * 4, 8 * 512 * 512 * 4)
