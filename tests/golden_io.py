"""Load the committed golden fixtures (generated by tests/golden/make_golden.py)."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def cases(prefix: str):
    out = []
    for f in sorted(glob.glob(os.path.join(GOLDEN, prefix + "_*.npz"))):
        z = np.load(f)
        d = {k: z[k] for k in z.files}
        d["metric"] = str(d["metric"])
        d["params"] = json.loads(str(d["params"]))
        d["name"] = os.path.basename(f)[:-4]
        out.append(d)
    return out


def ids(cs):
    return [c["name"] for c in cs]


def thr_of(s: str) -> float:
    return float("inf") if s == "inf" else float(np.float32(s))


def canonical(bars):
    """CLI canonical order (src/turbotops.cpp write_diagram): (dim, birth, death)."""
    t = np.asarray(bars, np.float32).reshape(-1, 3)
    order = np.lexsort((t[:, 2], t[:, 1], t[:, 0]))
    return t[order]
