"""Front-end benchmark on one GB300 (see --help).

Workload (default): the symmetric kNN flag complex of 100,000 float32 points in
R^32 drawn from a mixture of 16 isotropic Gaussians (centres ~ N(0, 4I),
sigma 1, seed 3), k = 15, L2, maxdim 1 — the front end of one diagram:
exact kNN lists -> symmetric kNN graph (CSR) -> filtration sort of its edges
-> apparent/emergent-pair scan -> Borůvka H0 -> dim-1 columns. A "step" is
one such front end; the metric is front ends (diagrams) per second.

  value  device-resident input, CUDA events on the library's stream around
         each step, L2 flushed (a 512 MB write) between steps outside the
         events, mean over the timed steps, max over ranks
  e2e    the same front end through the host-buffer C-ABI call
         (tt_knn_front_h): host points in, CSR + H0 + columns out, copies
         inside the timed region
  roofline   the dominant stage (exact kNN lists: tile order + k_knn_tc), timed
             alone; tensor work counted over the Gram tiles actually computed
  cpu_baseline   the reference's own front end on the host cores (two whole
         front ends), or the oracle port on a sample where it did not build

--impl reference runs only the CPU arm on rank 0 and prints its line: the
unmodified reference (compiled on this host by build() from its installed copy
in baseline/_ref, oracle/_ref/refbench) runs its own knn_lists_exact ->
knn_graph -> Reducer::dim0 on the whole cloud every step, on every host
thread; where the reference did not build, the oracle port on a bounded
sample stands in.
Multi-GPU: independent replicas per rank (weak scaling, no collective).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "diagrams/s"
N, DIM, K, MAXDIM, METRIC_NAME = 100_000, 32, 15, 1, "l2"


def peaks() -> tuple[dict, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def pg_backend(impl: str, cuda: bool) -> str:
    """The process group's backends: host tensors (the timing reduction) go
    to gloo, device tensors to NCCL; the CPU arm and CPU-only hosts use gloo
    alone (NCCL cannot be created without a GPU)."""
    return "cpu:gloo,cuda:nccl" if cuda and impl != "reference" else "gloo"


def max_over_ranks(v: float, ws: int) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)   # host tensor: reduced by the gloo backend
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------------------
# CPU arm: the reference itself (oracle/_ref/refbench, compiled on this host
# from the reference's installed copy), else the oracle port.
# ----------------------------------------------------------------------------
REFBENCH = os.path.join(ROOT, "oracle", "_ref", "refbench")


def ref_bench(stage: str, x, metric: str, k: int, maxdim: int, warmup: int, steps: int,
              threads: int = 0) -> dict:
    """Runs the unmodified reference's own functions for `stage` (see
    oracle/refbench.cpp) on the points x on the host cores and returns its
    JSON: per-step seconds and mean seconds per phase."""
    import tempfile

    import numpy as np
    with tempfile.TemporaryDirectory() as td:
        pts = os.path.join(td, "p.bin")
        np.ascontiguousarray(x, np.float32).tofile(pts)
        r = subprocess.run([REFBENCH, stage, pts, str(x.shape[0]), str(x.shape[1]), metric, str(k), str(maxdim),
                            str(warmup), str(steps), str(threads)], check=True, capture_output=True, text=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_front_seconds(x, sample: int, threads: int) -> tuple[float, dict]:
    """Seconds for one whole front end on the host, from a bounded sample."""
    import numpy as np

    from oracle import oracle as O
    n = x.shape[0]
    t0 = time.perf_counter()
    ids_s = O.knn_rows(x, METRIC_NAME, K, 0, sample, threads)
    t_knn = (time.perf_counter() - t0) * (n / sample)
    # graph + dim0 at full size need the full lists: use the device's lists'
    # shape (n x k) with the sampled rows' cost already measured; the graph
    # and dim0 stages are timed on a sub-cloud of the same density and scaled
    # by edge count.
    sub = min(n, 20_000)
    xs = np.ascontiguousarray(x[:sub])
    ids = O.knn_rows(xs, METRIC_NAME, K, 0, sub, threads)
    t1 = time.perf_counter()
    rp, ci, w = O.knn_graph(xs, METRIC_NAME, ids)
    t_graph = (time.perf_counter() - t1) * (n / sub)
    t2 = time.perf_counter()
    O.dim0(csr=(rp, ci, w), n=sub, maxdim=MAXDIM)
    t_dim0 = (time.perf_counter() - t2) * (n / sub)
    del ids_s
    return t_knn + t_graph + t_dim0, {"knn_s": t_knn, "graph_s": t_graph, "dim0_s": t_dim0}


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    from turbotops_gb300 import synth
    x = synth.gmm(N, DIM)
    threads = os.cpu_count() or 1
    if os.path.exists(REFBENCH):
        r = ref_bench("knnfront", x, METRIC_NAME, K, MAXDIM, args.warmup, args.steps)
        sec = statistics.mean(r["steps_s"])
        value = 1.0 / sec
        sample = f"the whole {N}-point front end every step (no sampling)"
        line = {"metric": METRIC, "value": value, "unit": "diagrams/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"knn-complex front end, gmm {N}x{DIM}, k={K}, {METRIC_NAME}, "
                                       f"maxdim {MAXDIM}",
                           "stages": "knn_lists_exact -> knn_graph -> Reducer<u64, SparseComplex>::dim0"},
                "impl": "reference",
                "cpu_baseline": {"value": value, "unit": "diagrams/s", "cores": r["threads"], "kind": "reference",
                                 "sample": sample, **{k: round(v, 4) for k, v in r["phases_s"].items()}},
                "e2e": {"value": value, "unit": "diagrams/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    from oracle import oracle as O
    O.lib()
    sample = args.cpu_sample
    for _ in range(args.warmup):
        cpu_front_seconds(x, max(sample // 4, threads), threads)
    times = []
    detail = {}
    for _ in range(args.steps):
        s, detail = cpu_front_seconds(x, sample, threads)
        times.append(s)
    sec = statistics.mean(times)
    value = 1.0 / sec
    line = {"metric": METRIC, "value": value, "unit": "diagrams/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"knn-complex front end, gmm {N}x{DIM}, k={K}, {METRIC_NAME}, maxdim {MAXDIM}",
                       "sample": f"{sample} kNN queries of {N}, graph+dim0 on a 20000-point sub-cloud, "
                                 f"scaled to the whole cloud"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "diagrams/s", "cores": threads, "kind": "port",
                             "sample": f"{sample} of {N} kNN queries (+ graph/dim0 on 20000 points), scaled",
                             **{k: round(v, 4) for k, v in detail.items()}},
            "e2e": {"value": value, "unit": "diagrams/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------
# GPU arm.
# ----------------------------------------------------------------------------
def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch

    from turbotops_gb300 import capi, synth
    from turbotops_gb300.capi import Context, KnnFrontOut

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x_h = synth.gmm(N, DIM)
    x = torch.from_numpy(x_h).to(dev)
    ctx = Context(local)
    L = ctx.L
    kind, p = capi.metric_parse(METRIC_NAME)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        out = KnnFrontOut()
        ctx.check(L.tt_knn_front(ctx.h, x.data_ptr(), N, DIM, kind, p, K, MAXDIM, C.byref(out)))
        return out

    for _ in range(args.warmup):
        out = step()
    torch.cuda.synchronize()
    nnz, ncols = out.graph.nnz, out.dim0.columns

    # ---- value: device-timed steps
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    clocks.start()
    launches0 = ctx.launches
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    launches = ctx.launches - launches0
    barrier(ws)
    clk = clocks.stop()
    ms_step = max_over_ranks(statistics.mean(ms), ws)

    # ---- e2e: host buffers through the C-ABI
    xp = torch.from_numpy(x_h).pin_memory()
    rp_h = torch.empty(N + 1, dtype=torch.int64).pin_memory()
    col_h = torch.empty(nnz + 16, dtype=torch.int32).pin_memory()
    w_h = torch.empty(nnz + 16, dtype=torch.float32).pin_memory()
    h0_h = torch.empty(N, dtype=torch.float32).pin_memory()
    ci_h = torch.empty(ncols + 16, dtype=torch.int64).pin_memory()
    cd_h = torch.empty(ncols + 16, dtype=torch.float32).pin_memory()
    cf_h = torch.empty(ncols + 16, dtype=torch.int64).pin_memory()
    ca_h = torch.empty(ncols + 16, dtype=torch.uint8).pin_memory()
    u64 = C.c_uint64
    cnt = [u64() for _ in range(5)]

    def e2e_step():
        ctx.check(L.tt_knn_front_h(ctx.h, xp.data_ptr(), N, DIM, kind, p, K, MAXDIM, rp_h.data_ptr(),
                                   col_h.data_ptr(), w_h.data_ptr(), nnz + 16, C.byref(cnt[0]), h0_h.data_ptr(),
                                   C.byref(cnt[1]), C.byref(cnt[2]), ci_h.data_ptr(), cd_h.data_ptr(),
                                   cf_h.data_ptr(), ca_h.data_ptr(), ncols + 16, C.byref(cnt[3]),
                                   C.byref(cnt[4])))

    for _ in range(2):
        e2e_step()
    e2e_ms = []
    for _ in range(max(3, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_step_ms = max_over_ranks(statistics.mean(e2e_ms), ws)
    h2d = N * DIM * 4
    d2h = (N + 1) * 8 + cnt[0].value * 8 + cnt[1].value * 4 + cnt[3].value * 21

    # ---- roofline of the dominant kernel: the exact kNN all-pairs scan alone
    ids = torch.empty((N, K), dtype=torch.int32, device=dev)
    dd = torch.empty((N, K), dtype=torch.float32, device=dev)
    ko = C.c_uint32()
    kms = []
    for r in range(args.warmup + args.steps):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.check(L.tt_knn(ctx.h, x.data_ptr(), N, DIM, kind, p, K, ids.data_ptr(), dd.data_ptr(), C.byref(ko)))
        e1.record(stream)
        e1.synchronize()
        if r >= args.warmup:
            kms.append(e0.elapsed_time(e1))
    knn_ms = statistics.mean(kms)
    evals = int(L.tt_ctx_filter_evals(ctx.h))
    tiles = int(L.tt_ctx_filter_tiles(ctx.h))
    tc_path = evals > 0
    kernel_name = ("k_knn_tc (tile-ordered tcgen05 TF32 Gram filter, exact lane-ordered recompute of the survivors)"
                   if tc_path else "k_scan<L2, 32, KnnOp<16>> (exact kNN all-pairs scan)")
    pk, pk_src = peaks()
    ntiles = (N + 127) // 128
    # tensor work actually issued: 128 x 128 x 32 Gram tiles the pruning kept
    gram_flops = 2.0 * 128 * 128 * DIM * (tiles if tc_path else ntiles * ntiles)
    achieved = gram_flops / (knn_ms * 1e-3) / 1e12
    fp32_ops = N * N * (3.0 * DIM)            # sub + mul/fma + add per coordinate, exhaustive exact path
    traffic = None
    tf = os.path.join(ROOT, "profiles", "knn_tc_l2_dim32.md")
    if tc_path and os.path.exists(tf):
        # DRAM bytes of one k_knn_tc launch, from one ncu capture of this
        # workload (the summary's "traffic:" line)
        import re
        with open(tf) as f:
            mt = re.search(r"^traffic: dram_bytes_per_launch=(\d+) points=(\d+) dim=(\d+) k=(\d+)", f.read(), re.M)
        if mt and (int(mt.group(2)), int(mt.group(3)), int(mt.group(4))) == (N, DIM, K):
            traffic = int(mt.group(1))

    # ---- CPU baseline (rank 0, N=1 only): the reference's own front end
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        if os.path.exists(REFBENCH):
            r = ref_bench("knnfront", x_h, METRIC_NAME, K, MAXDIM, 0, 2)
            sec = statistics.mean(r["steps_s"])
            cpu = {"value": 1.0 / sec, "unit": "diagrams/s", "cores": r["threads"], "kind": "reference",
                   "sample": f"2 whole front ends of the {N}-point cloud, all host threads",
                   **{k: round(v, 4) for k, v in r["phases_s"].items()}}
        else:
            s, det = cpu_front_seconds(x_h, args.cpu_sample, threads)
            cpu = {"value": 1.0 / s, "unit": "diagrams/s", "cores": threads, "kind": "port",
                   "sample": f"{args.cpu_sample} of {N} kNN queries on all host threads (+ graph/dim0 on a "
                             f"20000-point sub-cloud), scaled to the whole front end",
                   **{k: round(v, 4) for k, v in det.items()}}

    extras = {}
    if rank == 0 and not args.no_extras:
        extras["batch"] = batch_block(ctx, dev)
        extras["topo"] = topo_block(dev)
        extras["legs"] = legs_block(local, args.all_legs, not args.no_cpu)
        extras["batch_diagrams"] = batch_diagrams_block(args.all_legs, not args.no_cpu)

    value = ws * 1000.0 / ms_step
    line = {
        "metric": METRIC, "value": value, "unit": "diagrams/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"knn-complex front end, gmm {N}x{DIM}, k={K}, {METRIC_NAME}, maxdim {MAXDIM}",
                   "edges": int(out.dim0.edges), "columns": int(ncols), "nnz": int(nnz),
                   "l2": "flushed between steps (512 MB write)", "parallelism": f"replicas x{ws}"},
        "e2e": {"value": ws * 1000.0 / e2e_step_ms, "unit": "diagrams/s", "ms_per_step": e2e_step_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": achieved / pk["bf16_tflops"], "traffic": traffic,
                     "kernel": kernel_name, "gram_tiles": tiles, "gram_tiles_exhaustive": ntiles * ntiles,
                     "exact_evaluations": evals,
                     "exact_fraction_of_pairs": evals / float(N) / float(N),
                     "stage_ms": knn_ms, "peak_source": pk_src,
                     "exhaustive_equivalent_tflops": 2.0 * N * N * DIM / (knn_ms * 1e-3) / 1e12,
                     "fp32_exact_ops_per_s": fp32_ops / (knn_ms * 1e-3)},
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
        "other_workloads": extras,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def legs_block(index: int, all_legs: bool, with_reference: bool, reps: int = 3) -> dict:
    """The other benchmark workloads end to end through the public API
    (turbotops_gb300.persistence: host points in, whole diagram out — GPU
    front end plus host reduction), each beside the unmodified reference's
    own time for the same workload on this host's cores (one run of
    oracle/_ref/refbench), with the SM clocks sampled during our runs.
    Default: the 1000-point torus (maxdim 2), the 100k kNN complex (L2 and
    lp:1.5, maxdim 1), its complete-graph H0 (maxdim 0); --all-legs adds the
    3000-point lattice under L-inf (maxdim 2, ~80 s for the reference)."""
    import numpy as np  # noqa: F401

    from turbotops_gb300 import api, synth
    legs = [("torus1000 full Rips l2 maxdim 2", synth.torus(), dict(maxdim=2), ("dense", "l2", 15, 2)),
            ("gmm100k knn k=15 l2 maxdim 1", synth.gmm(), dict(maxdim=1, graph="knn", k=15),
             ("knnwhole", "l2", 15, 1)),
            ("gmm100k knn k=15 lp:1.5 maxdim 1", synth.gmm(), dict(maxdim=1, graph="knn", k=15, metric="lp:1.5"),
             ("knnwhole", "lp:1.5", 15, 1)),
            ("gmm100k complete-graph H0 l2 (maxdim 0)", synth.gmm(), dict(maxdim=0), ("mst", "l2", 15, 0))]
    if all_legs:
        legs.append(("lattice3000 full Rips linf maxdim 2", synth.lattice(), dict(maxdim=2, metric="linf"),
                     ("dense", "linf", 15, 2)))
    out = {}
    for name, x, kw, ref in legs:
        api.persistence(x, **kw)   # warm-up (buffers, kernels)
        clocks = Clocks(index)
        clocks.start()
        ts, bars = [], 0
        for _ in range(reps):
            t0 = time.perf_counter()
            dgms, _ = api.persistence(x, **kw)
            ts.append(time.perf_counter() - t0)
            bars = sum(len(g) for g in dgms)
        clk = clocks.stop()
        leg = {"seconds": statistics.mean(ts), "diagrams_per_s": 1.0 / statistics.mean(ts), "bars": bars,
               "steps": reps, "clocks": clk}
        if with_reference and os.path.exists(REFBENCH):
            r = ref_bench(ref[0], x, ref[1], ref[2], ref[3], 0, 1)
            leg["reference"] = {"seconds": r["steps_s"][0], "cores": r["threads"], "stage": ref[0],
                                "bars": r["check"], "same_bar_count": r["check"] == bars}
            leg["speedup"] = r["steps_s"][0] / leg["seconds"]
        out[name] = leg
    return out


BATCH_DRIVER = os.path.join(ROOT, "turbotops_gb300", "_lib", "batch_diagrams")


def batch_diagrams_block(all_legs: bool, with_reference: bool, reps: int = 2) -> dict:
    """Whole diagrams of the batched workloads through the C++ drop-in
    (turbotops_gb300/cxx/batch_diagrams.cpp: include/turbotops_gb300.hpp
    compiled inside the reference's include tree — one batched GPU front end,
    then the reference's RedZeD engine per cloud on every host thread),
    beside the reference's own tops::persistence called once per cloud on a
    sample of the clouds (every 16th of the 512; every cloud of the 64 circles;
    --all-legs: every cloud), whose diagrams must be identical."""
    import tempfile

    import numpy as np

    from turbotops_gb300 import synth
    if not os.path.exists(BATCH_DRIVER):
        return {"unavailable": "the C++ drop-in's driver was not built (the reference's installed copy is absent)"}
    out = {}
    for name, clouds, stride in [("512 circle / figure-eight clouds (64..2048 points, seed 4), l2, maxdim 1",
                                  synth.circle_batch(), 1 if all_legs else 16),
                                 ("64 noisy circles x 512 points (seed 5), l2, maxdim 1", synth.circles(), 1)]:
        with tempfile.TemporaryDirectory() as td:
            f = os.path.join(td, "c.bin")
            with open(f, "wb") as fh:
                np.array([len(clouds), clouds[0].shape[1]], np.uint32).tofile(fh)
                np.array([c.shape[0] for c in clouds], np.uint32).tofile(fh)
                np.concatenate(clouds).astype(np.float32).tofile(fh)
            r = subprocess.run([BATCH_DRIVER, f, "l2", "1", str(reps), str(stride if with_reference else 0), "0"],
                               capture_output=True, text=True)
        if r.returncode != 0:
            out[name] = {"error": (r.stdout + r.stderr)[-300:]}
            continue
        d = json.loads(r.stdout.strip().splitlines()[-1])
        d["diagrams_per_s"] = d["clouds"] / d["batch_s"]
        if d["reference_clouds"]:
            d["reference_diagrams_per_s"] = d["reference_clouds"] / d["reference_s"]
            d["speedup"] = d["diagrams_per_s"] / d["reference_diagrams_per_s"]
            d["reference_sample"] = (f"tops::persistence on {d['reference_clouds']} of {d['clouds']} clouds "
                                     f"(every {stride}th), one after another as its callers run it")
        out[name] = d
    return out


def batch_block(ctx, dev, reps: int = 5) -> dict:
    """The batched form (512 circle / figure-eight clouds of 64..2048 points,
    seed 4): one CUDA-graph replay of the batched dense front end vs the plain
    per-cloud GPU path (tt_dense_distances + tt_redzed_edges per cloud)."""
    import numpy as np
    import torch

    from turbotops_gb300 import capi, ops, synth
    clouds = synth.circle_batch()
    sizes = [c.shape[0] for c in clouds]
    b = ops.DenseBatch(ctx, sizes, 3, "l2", use_graph=True)
    b.load(torch.from_numpy(np.concatenate(clouds)).to(dev))
    b.run()   # capture
    out = capi.BatchOut()
    ctx.check(ctx.L.tt_batch_result(b.h, C.byref(out)))
    tr, tc_, ns, fc = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_int()
    tms = (C.c_float * 8)()
    ctx.check(ctx.L.tt_batch_tuning(b.h, C.byref(tr), C.byref(tc_), tms, C.byref(ns), C.byref(fc)))
    tuning = {"tile": [tr.value, tc_.value], "from_cache": bool(fc.value),
              "candidates_ms": {"x".join(map(str, s)): round(tms[i], 4)
                                for i, s in enumerate([(32, 32), (64, 64), (96, 96)][:ns.value])}}
    bs = torch.cuda.ExternalStream(out.stream, device=dev)
    ms = []
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(bs)
        b.run(wait=False)
        e1.record(bs)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    batch_ms = statistics.mean(ms)
    r = b.result()
    edges = int(r["edge_offset"][-1].item())
    b.close()
    # plain per-cloud path
    xs = [torch.from_numpy(c).to(dev) for c in clouds]
    kind, p = capi.metric_parse("l2")
    nmax = max(sizes)
    mat = torch.empty(nmax * nmax, dtype=torch.float32, device=dev)
    dd = torch.empty(nmax * (nmax - 1) // 2 + 1, dtype=torch.float32, device=dev)
    vv = torch.empty(nmax * (nmax - 1) + 2, dtype=torch.int32, device=dev)
    enc = C.c_float()
    cnt = C.c_uint64()

    def plain():
        for x in xs:
            n = x.shape[0]
            ctx.check(ctx.L.tt_dense_distances(ctx.h, x.data_ptr(), n, 3, kind, p, mat.data_ptr(), C.byref(enc)))
            ctx.check(ctx.L.tt_redzed_edges(ctx.h, mat.data_ptr(), None, None, None, n, enc.value, dd.data_ptr(),
                                            vv.data_ptr(), dd.numel(), C.byref(cnt)))
        torch.cuda.synchronize()

    plain()
    t0 = time.perf_counter()
    plain()
    plain_ms = (time.perf_counter() - t0) * 1e3
    pairs = sum(n * (n - 1) // 2 for n in sizes)
    return {"workload": "512 clouds (circle / figure-eight, 64..2048 points, R^3, seed 4), L2: distances, "
                        "enclosing radii, RedZeD edge lists", "clouds": len(sizes), "points": int(sum(sizes)),
            "pairs": pairs, "kept_edges": edges, "batched_graph_ms": batch_ms,
            "batched_diagrams_per_s": len(sizes) * 1000.0 / batch_ms, "per_cloud_ms": plain_ms,
            "per_cloud_diagrams_per_s": len(sizes) * 1000.0 / plain_ms,
            "batched_over_per_cloud": plain_ms / batch_ms,
            "hbm_bytes_written_matrices": 4 * sum(n * n for n in sizes), "autotuner": tuning,
            "hbm": batch_traffic(sizes, edges, batch_ms)}


def batch_traffic(sizes, edges: int, ms: float) -> dict:
    """Algorithmic HBM bytes of one batched run: the matrices written (4 B a
    pair, full layout) and their lower triangles read twice (count, keys),
    the kept keys written once and moved by the stable radix passes of every
    cloud's keys over their 31 distance bits (read for the histogram, read
    and written by the scatter: 24 B an edge a pass; 8-bit digits, four
    passes), the edge list emitted (8 B key read, 12 B written)."""
    pk, src = peaks()
    mat = 4 * sum(n * n for n in sizes)
    tri = 4 * sum(n * (n - 1) // 2 for n in sizes)
    passes = -(-31 // 8)
    b = mat + 2 * tri + 8 * edges + passes * 24 * edges + 20 * edges
    gbs = b / (ms * 1e-3) / 1e9
    return {"algorithmic_bytes": b, "radix_passes": passes, "achieved_gbs": gbs, "peak_gbs": pk["hbm_gbs"],
            "frac": gbs / pk["hbm_gbs"], "peak_source": src}


def topo_block(dev, reps: int = 2) -> dict:
    """The differentiable form: loss = sum over 64 noisy circles (512 points,
    sigma 0.1, seed 5) of -sum(top-4 H1 persistence) + sum(H0 death^2);
    a step = forward + hand-written adjoint backward. Batched: all clouds in
    one call (the clouds' host reductions spread over every core) vs the
    plain per-cloud path (one cloud per call, its reduction given every
    core), both over all 64 clouds."""
    import numpy as np
    import torch

    from turbotops_gb300 import synth, topo
    clouds = synth.circles()
    sizes = [c.shape[0] for c in clouds]
    x = torch.from_numpy(np.concatenate(clouds)).to(dev)

    def batched_step():
        xx = x.clone().requires_grad_(True)
        topo.topo_loss(xx, sizes).backward()
        torch.cuda.synchronize()
        return xx.grad

    batched_step()
    t0 = time.perf_counter()
    for _ in range(reps):
        batched_step()
    bt = (time.perf_counter() - t0) / reps

    def plain_step(q):
        xq = torch.from_numpy(clouds[q]).to(dev).requires_grad_(True)
        topo.topo_loss(xq, [sizes[q]]).backward()
        torch.cuda.synchronize()

    plain_step(0)
    t0 = time.perf_counter()
    for q in range(len(clouds)):
        plain_step(q)
    pt = time.perf_counter() - t0
    return {"workload": "topo loss fwd+bwd, 64 noisy circles x 512 points (R^3, sigma 0.1, seed 5), L2, maxdim 1",
            "batched_s_per_step": bt, "batched_steps_per_s": 1.0 / bt,
            "per_cloud_s_per_step": pt, "per_cloud_steps_per_s": 1.0 / pt,
            "per_cloud": "all 64 clouds, one call each, every host thread for its reduction",
            "host_threads": os.cpu_count(), "batched_over_per_cloud": pt / bt}


def batch_only(count: int) -> int:
    """The batched front end alone (first `count` of the 512 clouds): one
    capture with the autotuner's pick, then three timed graph replays; prints
    one line with their device times. For profiling runs."""
    import numpy as np
    import torch

    from turbotops_gb300 import capi, ops, synth
    from turbotops_gb300.capi import Context
    dev = torch.device("cuda", 0)
    ctx = Context(0)
    clouds = synth.circle_batch()[:count]
    b = ops.DenseBatch(ctx, [c.shape[0] for c in clouds], 3, "l2", use_graph=True)
    b.load(torch.from_numpy(np.concatenate(clouds)).to(dev))
    b.run()
    out = capi.BatchOut()
    ctx.check(ctx.L.tt_batch_result(b.h, C.byref(out)))
    bs = torch.cuda.ExternalStream(out.stream, device=dev)
    ms = []
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(bs)
        b.run(wait=False)
        e1.record(bs)
        e1.synchronize()
        ms.append(round(e0.elapsed_time(e1), 3))
    b.close()
    print(json.dumps({"batch_clouds": count, "replay_ms": ms}))
    return 0


def stage_only(stage: str, n: int, dim: int, steps: int, warmup: int) -> int:
    """One stage alone, timed with CUDA events on the context's stream (the
    default stream), for profiling runs: `dense` is make_dense + the enclosing
    radius of n Gaussian points in R^dim (an n x n float32 matrix written once:
    larger than L2 from n = 6,000, so no flush is needed), `mst` the
    complete-graph H0 deaths of the n x 32 Gaussian mixture. Prints one line."""
    import torch

    from turbotops_gb300 import capi, ops, synth
    from turbotops_gb300.capi import Context
    dev = torch.device("cuda", 0)
    ctx = Context(0)
    stream = torch.cuda.current_stream(dev)
    x = torch.from_numpy(synth.gauss(n, dim, 1) if stage == "dense" else synth.gmm(n, 32)).to(dev)
    if stage == "dense":   # the allocation-free entry point: no host round trip inside the timed region
        mat = torch.empty((n, n), dtype=torch.float32, device=dev)
        radius = torch.empty(1, dtype=torch.float32, device=dev)
        kind, p = capi.metric_parse("l2")

        def run():
            st = ctx.L.tt_dense_distances_static(x.data_ptr(), n, dim, kind, p, mat.data_ptr(), radius.data_ptr(),
                                                 C.c_void_p(stream.cuda_stream))
            if st:
                raise RuntimeError(ctx.L.tt_last_error(None).decode())
    else:
        def run():
            return ops.mst_deaths(ctx, x)
    ms = []
    for r in range(warmup + steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        run()
        e1.record(stream)
        e1.synchronize()
        if r >= warmup:
            ms.append(e0.elapsed_time(e1))
    t = statistics.mean(ms)
    line = {"stage": stage, "points": n, "dim": dim if stage == "dense" else 32, "ms": round(t, 4)}
    if stage == "dense":
        nbytes = 4 * n * n + 4 * n * dim   # the matrix written, the points read
        pk, src = peaks()
        line.update({"algorithmic_bytes": nbytes, "achieved_gbs": round(nbytes / t / 1e6, 1),
                     "peak_gbs": pk["hbm_gbs"], "frac": round(nbytes / t / 1e6 / pk["hbm_gbs"], 3),
                     "peak_source": src})
    print(json.dumps(line))
    return 0


def main():
    global N
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-sample", type=int, default=8000, help="kNN queries timed on the host")
    ap.add_argument("--points", "--n", dest="n", type=int, default=N,
                    help="points (smaller only for profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched / differentiable blocks")
    ap.add_argument("--all-legs", action="store_true", help="also the lattice workload among the other legs")
    ap.add_argument("--batch-only", type=int, metavar="CLOUDS", default=0,
                    help="profiling: only the batched front end on the first CLOUDS clouds (3 graph replays)")
    ap.add_argument("--stage", choices=["dense", "mst"], default=None,
                    help="profiling: only this stage on --points points (dense: in R^--dim)")
    ap.add_argument("--dim", type=int, default=3, help="dimension of the dense stage's points")
    args = ap.parse_args()
    N = args.n
    if args.batch_only:
        return batch_only(args.batch_only)
    if args.stage:
        return stage_only(args.stage, args.n, args.dim, args.steps, args.warmup)
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        import torch
        dist.init_process_group(pg_backend(args.impl, torch.cuda.is_available()))
    try:
        if args.impl == "reference":
            return run_reference(args, ws, rank)
        return run_gpu(args, ws, rank, local)
    finally:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
