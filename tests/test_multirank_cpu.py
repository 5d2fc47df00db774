"""The N > 1 path on CPU (gloo, world size 2): the front end of one diagram is
not sharded, so N GPUs run N independent replicas; what crosses ranks is only
the timing reduction (max over ranks) and the barriers around the timed
region. These tests run that host logic with two gloo ranks, and the
reference arm under torchrun, where rank 0 alone works and prints."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys
sys.path.insert(0, {root!r})
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
ws, rank, _ = bench.dist_env()
bench.barrier(ws)
v = bench.max_over_ranks(float(rank + 1) * 10.0, ws)
with open(os.path.join({out!r}, "rank%d.txt" % rank), "w") as f:   # one file per rank: no interleaving
    f.write("RESULT %d %d %r\n" % (rank, ws, v))
dist.destroy_process_group()
"""


def _torchrun(args, timeout=600):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(29500 + os.getpid() % 1000)] + args
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, env=env, cwd=ROOT)


def test_max_over_ranks_and_barrier_gloo(tmp_path):
    w = tmp_path / "worker.py"
    w.write_text(WORKER.format(root=ROOT, out=str(tmp_path)))
    r = _torchrun([str(w)])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [(tmp_path / f"rank{q}.txt").read_text().split() for q in range(2)]
    assert len(lines) == 2
    assert all(float(ln[3]) == 20.0 and ln[2] == "2" for ln in lines)


def test_reference_arm_under_torchrun_prints_one_line():
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                   "--cpu-sample", "40", "--points", "2000"])
    assert r.returncode == 0, r.stderr[-2000:]
    out = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(out) == 1
    d = json.loads(out[0])
    assert d["impl"] == "reference" and d["metric"] == "diagrams/s" and d["value"] > 0
    kind = "reference" if os.path.exists(os.path.join(ROOT, "oracle", "_ref", "refbench")) else "port"
    assert d["cpu_baseline"]["kind"] == kind and d["e2e"]["h2d_bytes_per_step"] == 0


def test_backend_string():
    sys.path.insert(0, ROOT)
    import bench
    # GPU arm on a GPU host: the timing reduction's host tensor must reach gloo,
    # which a plain "nccl" group would not have
    assert bench.pg_backend("gb300", True) == "cpu:gloo,cuda:nccl"
    assert bench.pg_backend("reference", True) == "gloo"
    assert bench.pg_backend("gb300", False) == "gloo"
