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


def workload_points(name: str):
    """The seeded points of a full-size workload named in diagrams.json
    (tests/golden/make_golden.py diagram_cases)."""
    from turbotops_gb300 import synth
    if name.startswith("torus1000"):
        return synth.torus()
    if name.startswith("lattice3000"):
        return synth.lattice()
    if name.startswith("gmm100k"):
        return synth.gmm()
    if name.startswith("gmm150k"):
        return synth.gmm(150_000, seed=6)
    if name.startswith("batch"):
        return synth.circle_batch()[int(name[5:name.index("_")])]
    if name.startswith("circle"):
        return synth.circles()[int(name[6:name.index("_")])]
    raise KeyError(name)


def cli_kwargs(args: list) -> dict:
    """`turbotops run` flags -> turbotops_gb300.persistence keyword arguments."""
    kw, it = {}, iter(args)
    for a in it:
        v = next(it)
        if a == "--maxdim":
            kw["maxdim"] = int(v)
        elif a == "--metric":
            kw["metric"] = v
        elif a == "--graph":
            kw["graph"] = v
        elif a == "-k":
            kw["k"] = int(v)
        elif a == "--threshold":
            kw["threshold"] = thr_of(v)
        else:
            raise KeyError(a)
    return kw
