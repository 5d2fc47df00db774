"""Generate the golden fixtures in this folder from the reference itself.

Runs ``oracle/_ref/refprobe`` and ``oracle/_ref/turbotops`` (the unmodified
reference compiled by ``make -C oracle install-ref ref`` from its installed
copy) on seeded clouds and stores each stage's raw outputs as ``.npz``, or the
canonical diagram text's SHA-256 for the full-size workloads. The tests only
read the committed fixtures; they never run this script.

    python tests/golden/make_golden.py              # small fixtures (seconds)
    python tests/golden/make_golden.py --configs    # + checksums of the full workloads' front ends
    python tests/golden/make_golden.py --diagrams   # whole diagrams of the full workloads (minutes)
    python tests/golden/make_golden.py --a64 DIR    # aarch64-host Lp fixtures (run on that host)
    python tests/golden/make_golden.py --higher     # diagrams above the benchmark dimensions
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import platform
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from turbotops_gb300 import synth  # noqa: E402

PROBE = os.path.join(ROOT, "oracle", "_ref", "refprobe")
CLI = os.path.join(ROOT, "oracle", "_ref", "turbotops")


def probe(stage: str, x: np.ndarray, metric: str, *extra: str) -> dict[str, np.ndarray]:
    n, dim = x.shape
    with tempfile.TemporaryDirectory() as td:
        pts = os.path.join(td, "p.bin")
        np.ascontiguousarray(x, np.float32).tofile(pts)
        pre = os.path.join(td, "o")
        subprocess.run([PROBE, stage, pts, str(n), str(dim), metric, *extra, pre], check=True)
        out = {}
        types = {"mat": np.float32, "encl": np.float32, "eidx": np.uint64, "ed": np.float32,
                 "app": np.uint8, "cidx": np.uint64, "cd": np.float32, "h0": np.float32,
                 "emi": np.uint64, "emd": np.float32, "emf": np.uint8, "thr": np.float32,
                 "piv": np.uint64, "c2idx": np.uint64, "c2d": np.float32, "app2n": np.uint64,
                 "ids": np.uint32, "rp": np.uint64, "ci": np.uint32, "w": np.float32,
                 "rd": np.float32, "rv": np.int32, "bars": np.float32}
        for f in os.listdir(td):
            if f.startswith("o."):
                key = f[2:]
                out[key] = np.fromfile(os.path.join(td, f), dtype=types[key])
        return out


def save(name: str, x: np.ndarray, metric: str, stage: str, params: dict, res: dict) -> None:
    np.savez_compressed(os.path.join(HERE, name + ".npz"), x=x, metric=np.array(metric),
                        stage=np.array(stage), params=np.array(json.dumps(params)), **res)


def small() -> None:
    clouds = {
        "u3": synth.uniform(200, 3, 11),
        "g17": synth.gauss(150, 17, 12),
        "g32": synth.gauss(120, 32, 13),
        "g9": synth.gauss(140, 9, 14),
        "grid4": synth.grid(300, 4, 6, 15),
        "torus": synth.torus(240, 16),
        # the first cloud of the topological-loss workload: its H1 columns
        # take thousands of additions in the host reduction
        "circle": synth.circles()[0],
        # C(600, 4) > 2^32: the host reduction of dimension 2 keeps wide
        # (64-bit index + diameter) queue entries
        "torus600": synth.torus(600, 17),
    }
    # dense distance matrices + enclosing radius, every metric path
    for cname in ["u3", "g17", "g32", "g9", "grid4"]:
        for metric in ["l2", "l1", "linf", "lp:3", "lp:1.5"]:
            x = clouds[cname]
            save(f"dense_{cname}_{metric.replace(':', '')}", x, metric, "dense", {},
                 probe("dense", x, metric))
    # dim0 (sorted edges, apparent flags, columns, H0, emergent probe) and assemble
    for cname, metric, thr in [("torus", "l2", "inf"), ("grid4", "l1", "inf"),
                               ("grid4", "linf", "inf"), ("u3", "l2", "0.3"),
                               ("grid4", "l2", "2.5")]:
        x = clouds[cname]
        tag = f"{cname}_{metric}_{thr.replace('.', 'p')}"
        save(f"asm_{tag}", x, metric, "asm", {"thr": thr}, probe("asm", x, metric, thr))
    # kNN lists, kNN graph, radius graph
    knn_cases = [("g9", "l2", 7), ("g9", "l1", 7), ("g9", "linf", 5), ("grid4", "l1", 6),
                 ("g32", "l2", 15), ("u3", "lp3", 6)]
    for cname, metric, k in knn_cases:
        x = clouds[cname]
        m = "lp:3" if metric == "lp3" else metric
        save(f"knn_{cname}_{metric}_{k}", x, m, "knn", {"k": k}, probe("knng", x, m, str(k)) |
             probe("knn", x, m, str(k)))
    for cname, metric, tau in [("u3", "l2", "0.2"), ("u3", "l1", "0.3"), ("grid4", "linf", "2"),
                               ("g9", "l2", "3.0")]:
        x = clouds[cname]
        save(f"radius_{cname}_{metric}", x, metric, "radius", {"tau": tau},
             probe("radius", x, metric, tau))
    # H0 via MST (complete graph)
    for cname, metric, thr in [("u3", "l2", "inf"), ("g32", "l2", "inf"), ("grid4", "l1", "inf"),
                               ("g9", "linf", "1.0")]:
        x = clouds[cname]
        save(f"mst_{cname}_{metric}", x, metric, "mst", {"thr": thr}, probe("mst", x, metric, thr))
    # RedZeD edge lists (dense and kNN graph) and sparse dim0
    for cname, metric in [("grid4", "l1"), ("u3", "l2")]:
        x = clouds[cname]
        save(f"rzd_{cname}_{metric}", x, metric, "rzd", {}, probe("rzd", x, metric))
    for cname, metric, k in [("g9", "l2", 8), ("grid4", "l1", 6)]:
        x = clouds[cname]
        save(f"rzs_{cname}_{metric}", x, metric, "rzs", {"k": k},
             probe("rzs", x, metric, str(k)) | {"knn_" + a: b for a, b in probe("knng", x, metric, str(k)).items()})
        save(f"sdim0_{cname}_{metric}", x, metric, "sdim0", {"k": k},
             probe("sdim0", x, metric, str(k)) | {"g_" + a: b for a, b in probe("knng", x, metric, str(k)).items()})
    # full diagrams (tops::persistence, dense, canonical order is applied by tests)
    for cname, metric, maxdim in [("torus", "l2", 2), ("grid4", "l1", 2), ("u3", "l2", 1),
                                  ("grid4", "linf", 1), ("circle", "l2", 1), ("torus600", "l2", 2)]:
        x = clouds[cname]
        save(f"bars_{cname}_{metric}_{maxdim}", x, metric, "bars", {"maxdim": maxdim},
             probe("bars", x, metric, str(maxdim)))


def sha(*arrs: np.ndarray) -> str:
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def configs() -> None:
    """Checksums of the full benchmark workloads' front-end outputs."""
    res = {}
    x = synth.torus()
    r = probe("asm", x, "l2", "inf")
    res["torus1000_l2"] = {"thr": float(r["thr"][0]), "edges": int(r["eidx"].size),
                           "edges_sha": sha(r["eidx"], r["ed"]), "app_sha": sha(r["app"]),
                           "app": int(r["app"].sum()), "cols": int(r["cidx"].size),
                           "cols_sha": sha(r["cidx"], r["cd"]), "h0_sha": sha(r["h0"]),
                           "piv_sha": sha(r["piv"]), "c2": int(r["c2idx"].size),
                           "c2_sha": sha(r["c2idx"], r["c2d"]), "app2": int(r["app2n"][0])}
    np.savez_compressed(os.path.join(HERE, "cfg_torus1000_piv.npz"), piv=r["piv"])
    for metric in ["linf", "l1"]:
        x = synth.lattice()
        r = probe("asm", x, metric, "inf")
        res[f"lattice3000_{metric}"] = {
            "thr": float(r["thr"][0]), "edges": int(r["eidx"].size),
            "edges_sha": sha(r["eidx"], r["ed"]), "app_sha": sha(r["app"]), "app": int(r["app"].sum()),
            "cols": int(r["cidx"].size), "cols_sha": sha(r["cidx"], r["cd"]), "h0_sha": sha(r["h0"]),
            "piv_sha": sha(r["piv"]), "c2": int(r["c2idx"].size), "c2_sha": sha(r["c2idx"], r["c2d"]),
            "app2": int(r["app2n"][0])}
        np.savez_compressed(os.path.join(HERE, f"cfg_lattice3000_{metric}_piv.npz"), piv=r["piv"])
        print(metric, res[f"lattice3000_{metric}"], flush=True)
    x = synth.gmm()
    r = probe("knng", x, "l2", "15") | probe("knn", x, "l2", "15")
    s = probe("rzs", x, "l2", "15")
    res["gmm100k_l2_k15"] = {"ids_sha": sha(r["ids"]), "nnz": int(r["ci"].size),
                             "csr_sha": sha(r["rp"], r["ci"], r["w"]), "rz_sha": sha(s["rd"], s["rv"])}
    with open(os.path.join(HERE, "configs.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)


def cli_cases() -> None:
    """Exact-text diagrams of the reference CLI on small hand-checkable inputs."""
    inputs = {"sq": "0 0\n1 0\n1 1\n0 1\n", "tri": "0 0\n1 0\n0 1\n",
              # weighted edge lists (--edges): a 4-cycle with one chord; repeated edges, a self
              # loop, a comment and comma separators; a 6-cycle (one H1 bar that never dies)
              "ecyc": "0 1 1\n1 2 1\n2 3 1\n3 0 1\n0 2 1.5\n",
              "edup": "0 1 2\n1 0 1\n1 2 1\n2 0 3\n3 3 0\n# comment\n2,3,0.5\n0\t3\t2.5\n",
              "ehex": "0 1 1\n1 2 1\n2 3 1\n3 4 1\n4 5 1\n5 0 1\n",
              # coordinates strtof reads differently from a double parse rounded to
              # float: a near-midpoint decimal (one rounding: 1 + 2^-23), hex floats,
              # an underscore digit separator (an error for strtof)
              "mid": "0 0\n1.0000000596046447753906250001 0\n0 1\n",
              "hexf": "0x0p0 0\n0x1.8p1 0\n0 0x1p-1\n0x1.4p1 0x1.8p0\n",
              "under": "0 0\n1_000 0\n"}
    runs = [("sq", ["--maxdim", "1"]), ("sq", ["--maxdim", "1", "--metric", "l1"]),
            ("sq", ["--maxdim", "1", "--metric", "linf"]), ("sq", ["--maxdim", "1", "--metric", "lp:3"]),
            ("sq", ["--maxdim", "1", "--threshold", "1"]), ("tri", []),
            ("sq", ["--graph", "knn", "-k", "2", "--maxdim", "1"]), ("sq", ["--maxdim", "2"]),
            ("ecyc", ["--edges", "--maxdim", "1"]), ("ecyc", ["--edges", "--maxdim", "1", "--threshold", "1"]),
            ("edup", ["--edges", "--maxdim", "1"]), ("ehex", ["--edges", "--maxdim", "1"]),
            ("ehex", ["--edges"]), ("mid", ["--maxdim", "1"]), ("hexf", ["--maxdim", "1"]),
            ("under", []),
            # make_dense's memory budget: 4 points need 24 bytes of lower triangle
            ("sq", ["--maxdim", "1", "--memory-budget", "16"]), ("sq", ["--maxdim", "1", "--memory-budget", "24"]),
            ("sq", ["--maxdim", "0", "--memory-budget", "16"]), ("sq", ["--memory-budget", "0.5k"]),
            ("sq", ["--memory-budget", "1x"]), ("sq", ["--memory-budget", "0"])]
    out = []
    with tempfile.TemporaryDirectory() as td:
        for name, text in inputs.items():
            with open(os.path.join(td, name + ".txt"), "w") as f:
                f.write(text)
        for name, args in runs:
            r = subprocess.run([CLI, "run", os.path.join(td, name + ".txt"), *args, "--quiet"],
                               capture_output=True, text=True)
            case = {"input": inputs[name], "args": args, "stdout": r.stdout}
            if r.returncode:
                case["rc"] = r.returncode
                case["stderr"] = r.stderr.replace(td + os.sep, "")
            out.append(case)
    with open(os.path.join(HERE, "cli_cases.json"), "w") as f:
        json.dump(out, f, indent=1)


def graph_bars() -> None:
    """Whole diagrams of kNN-graph complexes from the reference CLI (``--graph
    knn``, points as .bin): the CSR path of the host reduction is checked
    against them. Saved as gbars_<name>.npz (x, metric, params, bars)."""
    runs = [("circle400_l2_k8", synth.circles(1, 400, 0.1, 21)[0], "l2", 8, "inf"),
            ("gauss300_l1_k10", synth.gauss(300, 5, 22), "l1", 10, "inf"),
            ("grid200_linf_k6", synth.grid(200, 3, 6, 23), "linf", 6, "inf"),
            ("uniform500_l2_k12_t0p15", synth.uniform(500, 3, 24), "l2", 12, "0.15")]
    with tempfile.TemporaryDirectory() as td:
        for name, x, metric, k, thr in runs:
            pts = os.path.join(td, "p.bin")
            np.ascontiguousarray(x, np.float32).tofile(pts)
            r = subprocess.run([CLI, "run", pts, "--dim", str(x.shape[1]), "--graph", "knn", "-k", str(k),
                                "--metric", metric, "--maxdim", "1", "--threshold", thr, "--quiet"],
                               check=True, capture_output=True, text=True)
            bars = np.array([[float(t) for t in line.split()] for line in r.stdout.splitlines()],
                            np.float64).astype(np.float32).reshape(-1, 3)
            np.savez_compressed(os.path.join(HERE, f"gbars_{name}.npz"), x=x, metric=np.array(metric),
                                stage=np.array("gbars"), params=np.array(json.dumps({"k": k, "thr": thr})),
                                bars=bars)


def higher_dims() -> None:
    """Diagrams beyond the benchmark's dimensions: dense full Rips up to
    maxdim 3 and 4 (tops::persistence, refprobe "bars"), and flag complexes of
    kNN and radius graphs up to maxdim 3 (the CLI, --graph knn / --threshold)."""
    for name, x, metric, maxdim in [("u70", synth.uniform(70, 3, 41), "l2", 3),
                                    ("g50", synth.gauss(50, 4, 42), "l1", 4),
                                    ("torus150", synth.torus(150, 43), "l2", 3),
                                    ("grid60", synth.grid(60, 3, 4, 44), "linf", 3)]:
        save(f"bars_{name}_{metric}_{maxdim}", x, metric, "bars", {"maxdim": maxdim},
             probe("bars", x, metric, str(maxdim)))
    runs = [("knn400_l2_k10_d2", synth.circles(1, 400, 0.2, 45)[0], "l2", ["--graph", "knn", "-k", "10"], 2),
            ("knn200_l1_k8_d3", synth.gauss(200, 3, 46), "l1", ["--graph", "knn", "-k", "8"], 3),
            ("radius300_l2_t0p3_d2", synth.uniform(300, 3, 47), "l2", ["--threshold", "0.3"], 2),
            ("radius120_linf_t1_d3", synth.grid(120, 3, 5, 48), "linf", ["--threshold", "1"], 3)]
    with tempfile.TemporaryDirectory() as td:
        for name, x, metric, args, maxdim in runs:
            pts = os.path.join(td, "p.bin")
            np.ascontiguousarray(x, np.float32).tofile(pts)
            r = subprocess.run([CLI, "run", pts, "--dim", str(x.shape[1]), *args, "--metric", metric, "--maxdim",
                                str(maxdim), "--quiet"], check=True, capture_output=True, text=True)
            bars = np.array([[float(t) for t in line.split()] for line in r.stdout.splitlines()],
                            np.float64).astype(np.float32).reshape(-1, 3)
            np.savez_compressed(os.path.join(HERE, f"hbars_{name}.npz"), x=x, metric=np.array(metric),
                                stage=np.array("hbars"),
                                params=np.array(json.dumps({"args": args, "maxdim": maxdim})),
                                bars=bars, text=np.array(r.stdout))


def cli_text(x: np.ndarray, *args: str) -> tuple[str, float]:
    """The reference CLI's canonical diagram text for the points x (.bin input)."""
    with tempfile.TemporaryDirectory() as td:
        pts = os.path.join(td, "p.bin")
        np.ascontiguousarray(x, np.float32).tofile(pts)
        t0 = time.perf_counter()
        r = subprocess.run([CLI, "run", pts, "--dim", str(x.shape[1]), *args, "--quiet"], check=True,
                           capture_output=True, text=True)
        return r.stdout, time.perf_counter() - t0


def text_summary(text: str) -> dict:
    counts: dict[str, int] = {}
    for line in text.splitlines():
        d = line.split(" ", 1)[0]
        counts[d] = counts.get(d, 0) + 1
    return {"sha256": hashlib.sha256(text.encode()).hexdigest(), "bars": counts}


# Whole diagrams of the benchmark workloads at full size: (name, points,
# CLI arguments). The reference's text for L1, L2 and L-inf is the same on
# every host (exact lane-order arithmetic), so these are generated wherever
# the reference builds; the lp:1.5 ones depend on the host and come from a64().
def diagram_cases() -> list[tuple[str, np.ndarray, list[str]]]:
    cases = [("torus1000_l2_maxdim2", synth.torus(), ["--maxdim", "2"]),
             ("lattice3000_linf_maxdim2", synth.lattice(), ["--maxdim", "2", "--metric", "linf"]),
             ("lattice3000_l1_maxdim2", synth.lattice(), ["--maxdim", "2", "--metric", "l1"]),
             ("gmm100k_knn15_l2_maxdim1", synth.gmm(), ["--graph", "knn", "-k", "15", "--maxdim", "1"]),
             ("gmm100k_l2_maxdim0", synth.gmm(), ["--maxdim", "0"]),
             # above 131072 points: edge indices wider than the packed 33-bit key field
             ("gmm150k_knn15_l2_maxdim1", synth.gmm(150_000, seed=6), ["--graph", "knn", "-k", "15", "--maxdim", "1"]),
             ("gmm150k_l2_maxdim0", synth.gmm(150_000, seed=6), ["--maxdim", "0"])]
    for i, c in enumerate(synth.circle_batch()[:8]):
        cases.append((f"batch{i}_l2_maxdim1", c, ["--maxdim", "1"]))
    for i, c in enumerate(synth.circles()[:8]):
        cases.append((f"circle{i}_l2_maxdim1", c, ["--maxdim", "1"]))
    return cases


def diagrams(only: str | None = None) -> None:
    path = os.path.join(HERE, "diagrams.json")
    res = json.load(open(path)) if os.path.exists(path) else {}
    for name, x, args in diagram_cases():
        if only and only not in name:
            continue
        text, secs = cli_text(x, *args)
        res[name] = {"args": args, "n": int(x.shape[0]), "dim": int(x.shape[1]), **text_summary(text),
                     "reference_seconds": round(secs, 2), "host": platform.machine()}
        print(name, res[name], flush=True)
        with open(path, "w") as f:
            json.dump(res, f, indent=1, sort_keys=True)


def a64(out: str) -> None:
    """Non-integer Lp fixtures from the reference built on an aarch64 host (the
    GB300 machine's Grace CPU): its distance bits depend on the host's reciprocal
    estimate and libm, so these are generated there and committed as
    *_a64.npz, plus the full-size lp:1.5 workload's checksums and diagram."""
    if platform.machine() != "aarch64":
        sys.exit("a64 fixtures must be generated on an aarch64 host")
    global HERE
    os.makedirs(out, exist_ok=True)
    home, HERE = HERE, out
    clouds = {"u3": synth.uniform(200, 3, 11), "g17": synth.gauss(150, 17, 12), "g32": synth.gauss(120, 32, 13),
              "g9": synth.gauss(140, 9, 14), "grid4": synth.grid(300, 4, 6, 15), "g8": synth.gauss(130, 8, 16),
              "g40": synth.gauss(100, 40, 17)}
    for cname, x in clouds.items():
        for metric in ["lp:1.5", "lp:2.5", "lp:12", "lp:1.1"]:
            save(f"dense_{cname}_{metric.replace(':', '')}_a64", x, metric, "dense", {}, probe("dense", x, metric))
    for cname, metric, k in [("g9", "lp:1.5", 7), ("g32", "lp:1.5", 15), ("u3", "lp:2.5", 6),
                             ("g17", "lp:1.1", 9)]:
        x = clouds[cname]
        tag = metric.replace(":", "")
        save(f"knn_{cname}_{tag}_{k}_a64", x, metric, "knn", {"k": k},
             probe("knng", x, metric, str(k)) | probe("knn", x, metric, str(k)))
    for cname, metric in [("g9", "lp:1.5"), ("u3", "lp:2.5")]:
        x = clouds[cname]
        save(f"mst_{cname}_{metric.replace(':', '')}_a64", x, metric, "mst", {"thr": "inf"},
             probe("mst", x, metric, "inf"))
    for cname, metric, maxdim in [("u3", "lp:1.5", 1), ("g9", "lp:2.5", 2)]:
        x = clouds[cname]
        save(f"bars_{cname}_{metric.replace(':', '')}_{maxdim}_a64", x, metric, "bars", {"maxdim": maxdim},
             probe("bars", x, metric, str(maxdim)))
    HERE = home
    # the full-size lp:1.5 kNN workload
    x = synth.gmm()
    r = probe("knng", x, "lp:1.5", "15") | probe("knn", x, "lp:1.5", "15")
    res = {"gmm100k_lp1.5_k15": {"ids_sha": sha(r["ids"]), "nnz": int(r["ci"].size),
                                 "csr_sha": sha(r["rp"], r["ci"], r["w"])}}
    text, secs = cli_text(x, "--graph", "knn", "-k", "15", "--maxdim", "1", "--metric", "lp:1.5")
    res["gmm100k_knn15_lp1.5_maxdim1"] = {"args": ["--graph", "knn", "-k", "15", "--maxdim", "1", "--metric",
                                                   "lp:1.5"], "n": 100000, "dim": 32, **text_summary(text),
                                          "reference_seconds": round(secs, 2), "host": platform.machine()}
    with open(os.path.join(out, "configs_a64.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", action="store_true", help="+ checksums of the full workloads' front ends")
    ap.add_argument("--diagrams", nargs="?", const="", default=None,
                    help="whole diagrams of the full workloads (optionally only names containing this)")
    ap.add_argument("--a64", metavar="DIR", help="only the aarch64 Lp fixtures, written to DIR")
    ap.add_argument("--higher", action="store_true", help="only the higher-dimension diagrams")
    ap.add_argument("--cli", action="store_true", help="only the CLI text cases")
    a = ap.parse_args()
    if not os.path.exists(PROBE):
        sys.exit("build the reference first: make -C oracle install-ref ref")
    if a.a64:
        a64(a.a64)
    elif a.higher:
        higher_dims()
    elif a.cli:
        cli_cases()
    elif a.diagrams is not None:
        diagrams(a.diagrams or None)
    else:
        small()
        cli_cases()
        graph_bars()
        if a.configs:
            configs()
