"""The C++ boundary compiled for real: tests/cxx_boundary_check.cpp includes
the unmodified reference headers (the reference's installed copy in
baseline/_ref) and include/turbotops_gb300.hpp, links the CUDA library, and
compares the GB300 glue with the reference's own persistence / knn_graph /
mst::h0 results and exception messages on the same inputs."""
import os
import subprocess

import pytest

from turbotops_gb300 import build

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "baseline", "_ref")


def test_cxx_glue_matches_the_reference(tmp_path):
    if not os.path.isdir(os.path.join(REF, "include", "turbotops")):
        pytest.skip("the reference's installed copy (baseline/_ref) is absent")
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path / "cxx_boundary_check")
    subprocess.run(["g++", "-std=c++20", "-O2", "-march=native", "-Wno-unused-parameter",
                    "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(REF, "include"),
                    "-isystem", os.path.join(REF, "third_party"), "-isystem",
                    os.path.join(REF, "third_party", "simde"), os.path.join(ROOT, "tests", "cxx_boundary_check.cpp"),
                    "-o", exe, "-L" + libdir, "-lturbotops_gb300", "-Wl,-rpath," + libdir, "-pthread"],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
    assert int(r.stdout.split()[1]) >= 30
