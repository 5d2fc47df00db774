"""Whole diagrams of the benchmark workloads at full size, byte for byte.

Each case runs the product's public API (turbotops_gb300.persistence: GPU
front end, host reduction) on the seeded full-size points and compares the
SHA-256 of the canonical diagram text (the CLI's '%u %.9g %.9g' lines in
(dim, birth, death) order, src/turbotops.cpp:208-230) with the text the
unmodified reference CLI printed for the same points (tests/golden/
diagrams.json; L1, L2 and L-inf diagrams are host-independent). The
per-dimension bar counts are compared first so a mismatch says where. The
lp:1.5 diagram of the kNN workload comes from the reference built on this
box's aarch64 host (tests/golden/configs_a64.json)."""
import hashlib
import json
import os

import pytest

from golden_io import cli_kwargs, workload_points

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DIAGRAMS = json.load(open(os.path.join(ROOT, "tests", "golden", "diagrams.json")))
# lp:1.5: the reference built on this machine's aarch64 host
DIAGRAMS.update({k: v for k, v in json.load(open(os.path.join(ROOT, "tests", "golden", "configs_a64.json"))).items()
                 if "sha256" in v})


def _check(name, case):
    from turbotops_gb300 import api
    x = workload_points(name)
    assert x.shape == (case["n"], case["dim"])
    dgms, info = api.persistence(x, **cli_kwargs(case["args"]))
    text = api.format_diagram(dgms)
    counts = {}
    for line in text.splitlines():
        counts[line.split(" ", 1)[0]] = counts.get(line.split(" ", 1)[0], 0) + 1
    assert counts == case["bars"], (counts, case["bars"])
    assert hashlib.sha256(text.encode()).hexdigest() == case["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(DIAGRAMS))
def test_full_size_diagram(name):
    _check(name, DIAGRAMS[name])
