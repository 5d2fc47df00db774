"""The CLI drop-in: exact-text diagrams of the reference CLI on hand-checkable
inputs (GPU), and the error paths (exit code 2, 'turbotops: <message>'),
which need no GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ALL_CASES = json.load(open(os.path.join(ROOT, "tests", "golden", "cli_cases.json")))
CASES = [c for c in ALL_CASES if "rc" not in c]
ERR_CASES = [c for c in ALL_CASES if "rc" in c]


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
@pytest.mark.parametrize("case", ERR_CASES, ids=[c["input"].split()[-2] for c in ERR_CASES])
def test_cli_golden_errors(case, tmp_path):
    """Inputs the reference CLI rejects: same exit code, same message (the
    points are read on the device)."""
    p = tmp_path / "in.txt"
    p.write_text(case["input"])
    r = cli("run", str(p), *case["args"], "--quiet")
    assert r.returncode == case["rc"] and r.stderr == case["stderr"], r.stderr


def test_coordinates_parse_like_strtof():
    """One rounding from the text to float32 (the host's strtof), not a double
    parse rounded again; hex floats accepted; Python-only spellings rejected."""
    import numpy as np
    from turbotops_gb300.cli import CliError, _parse_f32
    bits = lambda t: int(np.float32(_parse_f32(t, "coordinate")).view(np.uint32))
    assert bits("1.0000000596046447753906250001") == 0x3F800001
    assert float(np.float32(float("1.0000000596046447753906250001"))) == 1.0   # what double-then-float gives
    assert _parse_f32("0x1.8p1", "coordinate") == 3.0
    for bad in ["1_000", "1.5x", "", "0x"]:
        with pytest.raises(CliError):
            _parse_f32(bad, "coordinate")


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


@pytest.mark.gpu
def test_cli_rejects_bad_rows_and_metric(tmp_path):
    p = tmp_path / "bad.txt"
    p.write_text("0 0\n1 0 2\n")
    r = cli("run", str(p))
    assert r.returncode == 2 and r.stderr == f"turbotops: {p}: inconsistent row length at point 1\n"
    q = tmp_path / "ok.txt"
    q.write_text("0 0\n1 0\n")
    r = cli("run", str(q), "--metric", "cosine")
    assert r.returncode == 2 and "metric: unknown 'cosine'" in r.stderr


def test_cli_rejects_flags(tmp_path):
    """Option errors come before the input is read (no GPU needed)."""
    q = tmp_path / "ok.txt"
    q.write_text("0 0\n1 0\n")
    r = cli("run", str(q), "--frobnicate")
    assert r.returncode == 2 and "unknown option" in r.stderr
    r = cli("run", str(q), "--graph", "star")
    assert r.returncode == 2 and "--graph must be full or knn" in r.stderr
    r = cli("run", str(q), "--mode", "sideways")
    assert r.returncode == 2 and "mode must be auto, boundary or coboundary" in r.stderr


@pytest.mark.parametrize("text,msg", [
    ("0 1\n", "in.txt:1: expected 'i j w'"),
    ("0 1 1\n1 2 -1\n", "in.txt:2: bad weight"),
    ("0 1 nan\n", "in.txt:1: bad weight"),
    ("0 x 1\n", "bad vertex 'x'"),
    ("0 1 w\n", "bad weight 'w'"),
    ("0 4294967295 1\n", "vertex id too large"),
    ("# nothing\n3 3 1\n", "in.txt: no vertices (empty edge list?)"),
])
def test_cli_edges_errors_exit_2(text, msg, tmp_path):
    """Edge-list input errors (src/turbotops.cpp:173-205, :879-882), before any GPU work."""
    p = tmp_path / "in.txt"
    p.write_text(text)
    r = cli("run", str(p), "--edges")
    assert r.returncode == 2 and r.stderr.startswith("turbotops: ") and msg in r.stderr, r.stderr


def test_symmetric_rows_matches_reference_ingestion():
    """Both directions of every entry, self loops dropped, the smallest weight of a
    repeated (row, column), rows sorted: checked against a direct restatement of
    the reference's per-row vectors (python/turbotops_ext.cpp:82-98)."""
    import numpy as np
    from turbotops_gb300.api import symmetric_rows
    rng = np.random.default_rng(5)
    n = 60
    i = rng.integers(0, n, 900)
    j = rng.integers(0, n, 900)
    w = rng.integers(0, 8, 900).astype(np.float32) * np.float32(0.5)
    rp, ci, ww = symmetric_rows(i, j, w, n)
    rows = [[] for _ in range(n)]
    for a, b, d in zip(i, j, w):
        if a == b:
            continue
        rows[a].append((int(b), float(d)))
        rows[b].append((int(a), float(d)))
    exp_rp, exp_ci, exp_w = [0], [], []
    for r in rows:
        r.sort()
        seen = set()
        for b, d in r:
            if b in seen:
                continue
            seen.add(b)
            exp_ci.append(b)
            exp_w.append(d)
        exp_rp.append(len(exp_ci))
    assert rp.tolist() == exp_rp and ci.tolist() == exp_ci and ww.tolist() == exp_w
