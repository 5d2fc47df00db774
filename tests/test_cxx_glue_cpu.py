"""CPU check of the C++ glue's RedZeD hand-over (include/turbotops_gb300.hpp):
the reference's unmodified RedZeD engine takes its edge list from the glue's
build_edges overload and, given the reference's own list, reproduces the
reference's diagrams bar for bar; and the leftover-coface predicate answered
from precomputed bits (as the device computes them) agrees with the engine's
own scan on every edge it is asked about. Needs the reference's installed copy
(baseline/_ref); no GPU and no library call."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")


def test_redzed_takes_the_prebuilt_edge_list(tmp_path):
    if not os.path.isdir(os.path.join(REF, "include", "turbotops")):
        pytest.skip("the reference's installed copy (baseline/_ref) is absent")
    exe = str(tmp_path / "glue_cpu")
    subprocess.run(["g++", "-std=c++20", "-O1", "-Wno-unused-parameter", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(REF, "include"), "-isystem", os.path.join(REF, "third_party"), "-isystem",
                    os.path.join(REF, "third_party", "simde"), os.path.join(ROOT, "tests", "cxx_glue_cpu_check.cpp"),
                    "-o", exe, "-pthread"], check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == "ok 12", r.stdout + r.stderr
