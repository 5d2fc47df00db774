"""``persistence()`` — the drop-in for ``turbo_tops.persistence`` (python/turbo_tops/__init__.py:23-71).

Same signature and return value: a list of (m, 2) float32 arrays of
(birth, death) per dimension 0..maxdim in discovery order (death = inf for
essential classes) and an info dict. The front end runs on the GPU through
the C-ABI (``tt_persistence_h``); the column reduction runs on the host.
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np

from . import capi

_CTX = {}


def _context(device: int = 0) -> capi.Context:
    if device not in _CTX:
        _CTX[device] = capi.Context(device)
    return _CTX[device]


def persistence(x, maxdim=1, threshold=math.inf, metric="l2", graph="full", k=15, approximate=False,
                recall_samples=0, threads=0, memory_budget=0, device=0):
    """Persistence diagrams of the Vietoris–Rips filtration (see turbo_tops.persistence).

    ``approximate`` (HNSW) is not offered: the GPU computes exact kNN lists.
    ``threads`` and ``memory_budget`` are accepted and ignored (the results
    never depended on them).
    """
    if hasattr(x, "tocsr"):
        raise ValueError("graph input: use turbotops_gb300.persistence on point clouds (CSR input is not "
                         "offered by the GPU front end yet)")
    if approximate:
        raise ValueError("approximate (HNSW) kNN is not offered: the GPU front end computes exact kNN")
    if graph not in ("full", "knn"):
        raise ValueError("graph must be 'full' or 'knn'")
    x = np.ascontiguousarray(x, dtype=np.float32)
    if x.ndim != 2:
        raise ValueError("x must be a 2-d array (n, d)")
    kind, p = capi.metric_parse(str(metric))
    ctx = _context(device)
    n, dim = x.shape
    out = C.POINTER(capi.Barcode)()
    t0 = time.perf_counter()
    ctx.check(ctx.L.tt_persistence_h(ctx.h, x.ctypes.data, n, dim, kind, p, int(maxdim), float(threshold),
                                     1 if graph == "knn" else 0, int(k), C.byref(out)))
    secs = time.perf_counter() - t0
    try:
        b = out.contents
        dgms = []
        o = 0
        for d in range(b.ndims):
            m = int(b.count[d])
            arr = np.empty((m, 2), np.float32)
            if m:
                arr[:, 0] = np.ctypeslib.as_array(b.birth, shape=(b.total,))[o:o + m]
                arr[:, 1] = np.ctypeslib.as_array(b.death, shape=(b.total,))[o:o + m]
            dgms.append(arr)
            o += m
        while len(dgms) <= maxdim:
            dgms.append(np.empty((0, 2), np.float32))
        info = {"method": b.method.decode(), "threshold": float(b.threshold), "edges": int(b.edges),
                "index_bits": 64, "seconds_total": secs,
                "columns": [int(v) for v in b.columns[:max(maxdim, 0)]],
                "apparent": [int(v) for v in b.apparent[:max(maxdim, 0)]],
                "emergent": [int(v) for v in b.emergent[:max(maxdim, 0)]]}
    finally:
        ctx.L.tt_barcode_free(out)
    return dgms, info


def canonical(dgms) -> np.ndarray:
    """(dim, birth, death) rows in the CLI's canonical order (src/turbotops.cpp:208-230)."""
    rows = [np.c_[np.full(len(d), i, np.float32), d] for i, d in enumerate(dgms) if len(d)]
    if not rows:
        return np.empty((0, 3), np.float32)
    t = np.concatenate(rows).astype(np.float32)
    return t[np.lexsort((t[:, 2], t[:, 1], t[:, 0]))]


def format_diagram(dgms) -> str:
    """The CLI's text output: 'dim birth death' with %.9g, 'inf' for essential bars."""
    lines = []
    for d, b, e in canonical(dgms):
        if np.isinf(e):
            lines.append(f"{int(d)} {float(b):.9g} inf")
        else:
            lines.append(f"{int(d)} {float(b):.9g} {float(e):.9g}")
    return "\n".join(lines) + ("\n" if lines else "")
