"""The bench's multi-process path on CPU: torchrun with two gloo ranks runs the reference arm (rank 0 alone
prints one JSON line; rank 1 exits 0 without work), and the max-over-ranks helper reduces across ranks."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_two_ranks_gloo():
    pytest.importorskip("torch")
    env = dict(os.environ, OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2", "--master-addr",
           "127.0.0.1", "--master-port", "29611", os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--size", "4", "--rves", "2", "--steps", "1", "--warmup", "1", "--cpu-sample-rves", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "homogenizations/s"
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0


WORKER = r"""
import os, sys, json
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank = dist.get_rank()
v = bench.max_over_ranks(dist, float(rank + 1) * 2.5, dist.get_world_size())
with open(os.path.join({out!r}, f"rank{{rank}}.json"), "w") as f:
    json.dump({{"rank": rank, "max": v}}, f)
dist.destroy_process_group()
"""


def test_max_over_ranks_gloo(tmp_path):
    pytest.importorskip("torch")
    w = tmp_path / "w.py"
    w.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2", "--master-addr",
           "127.0.0.1", "--master-port", "29612", str(w)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    # each rank writes its own file: two processes printing to one pipe may interleave their lines
    vals = [json.load(open(tmp_path / f"rank{k}.json"))["max"] for k in range(2)]
    assert vals == [5.0, 5.0]
