"""The CLI drop-in: exact-text diagrams of the reference CLI on hand-checkable
inputs (GPU), and the error paths (exit code 2, 'turbotops: <message>'),
which need no GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = json.load(open(os.path.join(ROOT, "tests", "golden", "cli_cases.json")))


def cli(*args, stdin=None):
    return subprocess.run([sys.executable, "-m", "turbotops_gb300", *args], capture_output=True, text=True,
                          cwd=ROOT, timeout=300)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[" ".join(c["args"]) or "default" for c in CASES])
def test_cli_golden_diagrams(case, tmp_path):
    p = tmp_path / "in.txt"
    p.write_text(case["input"])
    r = cli("run", str(p), *case["args"], "--quiet")
    assert r.returncode == 0, r.stderr
    assert r.stdout == case["stdout"]


@pytest.mark.gpu
def test_cli_bom_bin_and_output_file(tmp_path):
    import numpy as np
    sq = CASES[0]
    p = tmp_path / "bom.txt"
    p.write_bytes(b"\xef\xbb\xbf" + sq["input"].encode())
    out = tmp_path / "o.txt"
    r = cli("run", str(p), "--maxdim", "1", "--output", str(out))
    assert r.returncode == 0 and out.read_text() == sq["stdout"]
    b = tmp_path / "sq.bin"
    np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32).tofile(b)
    r = cli("run", str(b), "--dim", "2", "--maxdim", "1", "--quiet")
    assert r.returncode == 0 and r.stdout == sq["stdout"]


def test_cli_version_and_usage():
    r = cli("--version")
    assert r.returncode == 0 and r.stdout.startswith("turbotops 0.1.0")
    r = cli()
    assert r.returncode == 2 and "usage" in r.stderr


@pytest.mark.parametrize("args,msg", [
    (["run"], "missing <input>"),
    (["run", "/nonexistent/x.txt"], "cannot open"),
    (["run", "X.bin"], "--dim is required"),
    (["bogus"], "unknown command"),
])
def test_cli_errors_exit_2(args, msg):
    r = cli(*args)
    assert r.returncode == 2 and msg in r.stderr and r.stderr.startswith("turbotops: ")


def test_cli_rejects_bad_rows_metric_and_flags(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("0 0\n1 0 2\n")
    r = cli("run", str(p))
    assert r.returncode == 2 and "inconsistent row length" in r.stderr
    q = tmp_path / "ok.txt"
    q.write_text("0 0\n1 0\n")
    r = cli("run", str(q), "--metric", "cosine")
    assert r.returncode == 2 and "metric: unknown 'cosine'" in r.stderr
    r = cli("run", str(q), "--frobnicate")
    assert r.returncode == 2 and "unknown option" in r.stderr
    r = cli("run", str(q), "--graph", "star")
    assert r.returncode == 2 and "--graph must be full or knn" in r.stderr
    r = cli("run", str(q), "--mode", "sideways")
    assert r.returncode == 2 and "mode must be auto, boundary or coboundary" in r.stderr
