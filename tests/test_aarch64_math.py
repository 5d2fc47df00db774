"""The oracle's model of the reference's non-integer Lp arithmetic
(oracle/aarch64_math.h) against the real thing on this host: glibc's powf
(every x of the ranges an lp:1.5 distance feeds it, plus random pairs) and,
on aarch64, the FRECPE instruction (every float) and SIMDe's NEON rcp_ps
sequence. No GPU involved."""
from __future__ import annotations

import os
import platform
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("a64") / "amc")
    subprocess.run(["g++", "-O2", "-std=c++20", "-ffp-contract=off", "-I" + os.path.join(ROOT, "oracle"),
                    "-o", exe, os.path.join(HERE, "aarch64_math_check.cpp"), "-pthread"], check=True)
    return exe


def _run(exe: str, mode: str) -> dict[str, tuple[int, int, str]]:
    out = subprocess.run([exe, mode], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        f = line.split(" ", 3)
        if f[1] == "skipped":
            continue
        res[f[0]] = (int(f[1]), int(f[2]), f[3] if len(f) > 3 else "")
    return res


def test_restatement_matches_host(checker):
    res = _run(checker, "quick")
    assert res["powf_root_1.5"][0] == 5 << 23   # every float in [1, 32)
    if platform.machine() == "aarch64":
        assert res["frecpe"][0] == 1 << 32
    for name, (tested, bad, first) in res.items():
        assert tested > 0, name
        assert bad == 0, f"{name}: {bad} of {tested} differ ({first})"
