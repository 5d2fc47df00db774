"""In-tree build of libturbotops_gb300.so for sm_103a (GB300).

Every translation unit under csrc/ is compiled by nvcc in parallel with one
``-gencode arch=compute_103a,code=sm_103a`` and linked into
``turbotops_gb300/_lib/libturbotops_gb300.so``. No cmake, no torch extension
machinery: the library is plain C-ABI and is loaded with ctypes.

    python -m turbotops_gb300.build [--force] [-j N]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libturbotops_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the GB300 library cannot be built")


def flags(extra_debug: bool = False) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing",
                "-I" + os.path.join(ROOT, "include"), "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
    if extra_debug:
        f += ["-DTT_DEVICE_CHECKS=1"]
    return f


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _digest() -> str:
    h = hashlib.sha256()
    for f in sources() + sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
                                + glob.glob(os.path.join(ROOT, "include", "*.h"))):
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    h.update(" ".join(flags()).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _compile(src: str, obj: str) -> None:
    cmd = [nvcc()] + flags() + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    stamp = os.path.join(OUT, "build.stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == dig:
        return LIB
    objs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        futs = []
        for s in sources():
            o = os.path.join(OUT, os.path.basename(s) + ".o")
            objs.append(o)
            futs.append(ex.submit(_compile, s, o))
        for f in futs:
            f.result()
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(dig)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-j", type=int, default=None)
    a = ap.parse_args()
    build(a.force, a.j, verbose=True)
