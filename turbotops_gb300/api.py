"""``persistence()`` — the drop-in for ``turbo_tops.persistence`` (python/turbo_tops/__init__.py:23-71).

Same signature and return value: a list of (m, 2) float32 arrays of
(birth, death) per dimension 0..maxdim in discovery order (death = inf for
essential classes) and an info dict. The front end runs on the GPU through
the C-ABI (``tt_persistence_h``, ``tt_persistence_graph_h`` for graph
input); the column reduction runs on the host.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time

import numpy as np

from . import capi

_CTX = {}


def _context(device: int = 0) -> capi.Context:
    if device not in _CTX:
        _CTX[device] = capi.Context(device)
    return _CTX[device]


def _budget(memory_budget: int) -> int:
    """Options::memory_budget with the reference's default
    (memory.hpp:17-33): half of the physical memory, 8 GiB if unknown."""
    if memory_budget:
        return int(memory_budget)
    try:
        m = os.sysconf("SC_PHYS_PAGES") * os.sysconf("SC_PAGE_SIZE")
    except (ValueError, OSError):
        m = 0
    return m // 2 if m > 0 else 8 << 30


def persistence(x, maxdim=1, threshold=math.inf, metric="l2", graph="full", k=15, approximate=False,
                recall_samples=0, threads=0, memory_budget=0, device=0):
    """Persistence diagrams of the Vietoris–Rips filtration (see turbo_tops.persistence).

    ``x`` is an (n, d) point cloud or a scipy sparse matrix (the flag complex
    of the weighted graph, as the reference's ``persistence_csr``).
    ``approximate`` (HNSW) is not offered: the GPU computes exact kNN lists.
    ``threads`` is accepted and ignored (the results never depended on it).
    ``memory_budget`` (bytes, 0 = half of the host's physical memory) refuses
    a dense complex whose distance matrix would exceed it, with make_dense's
    message, as ValueError — the reference module's translation of its
    std::length_error (rips.hpp:383-416).
    """
    if hasattr(x, "tocsr"):
        rp, ci, w, n = csr_graph(x)
        return persistence_graph(rp, ci, w, n, maxdim=maxdim, threshold=threshold, device=device)
    if approximate:
        raise ValueError("approximate (HNSW) kNN is not offered: the GPU front end computes exact kNN")
    if graph not in ("full", "knn"):
        raise ValueError("graph must be 'full' or 'knn'")
    x = np.ascontiguousarray(x, dtype=np.float32)
    if x.ndim != 2:
        raise ValueError("x must be a 2-d array (n, d)")
    kind, p = capi.metric_parse(str(metric))
    n, dim = x.shape
    if graph == "full" and maxdim > 0 and math.isinf(threshold) and n * (n - 1) // 2 * 4 > _budget(memory_budget):
        if not np.isfinite(x).all():
            raise ValueError("persistence: non-finite coordinate")
        raise ValueError("rips: the dense distance matrix exceeds the memory budget; use a finite threshold "
                         "or a sparse graph")
    ctx = _context(device)
    ctx.check(ctx.L.tt_ctx_set_memory_budget(ctx.h, int(memory_budget)))
    out = C.POINTER(capi.Barcode)()
    t0 = time.perf_counter()
    ctx.check(ctx.L.tt_persistence_h(ctx.h, x.ctypes.data, n, dim, kind, p, int(maxdim), float(threshold),
                                     1 if graph == "knn" else 0, int(k), C.byref(out)))
    return _unpack(ctx, out, maxdim, time.perf_counter() - t0)


def symmetric_rows(i, j, w, n):
    """The reference's graph ingestion (python/turbotops_ext.cpp:76-99,
    src/turbotops.cpp:173-205): every entry (i, j, w) with i != j lands in
    rows i and j, and a repeated (row, column) keeps its smallest weight.
    Returns CSR arrays (row_ptr u64, col u32, weight f32) with sorted rows."""
    i = np.asarray(i, np.int64)
    j = np.asarray(j, np.int64)
    w = np.asarray(w, np.float32)
    keep = i != j
    i, j, w = i[keep], j[keep], w[keep]
    r = np.concatenate([i, j])
    c = np.concatenate([j, i])
    ww = np.concatenate([w, w])
    order = np.lexsort((ww, c, r))
    r, c, ww = r[order], c[order], ww[order]
    first = np.ones(len(r), bool)
    first[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
    r, c, ww = r[first], c[first], ww[first]
    rp = np.zeros(n + 1, np.uint64)
    np.add.at(rp, r + 1, 1)
    return np.cumsum(rp).astype(np.uint64), c.astype(np.uint32), ww.astype(np.float32)


def csr_graph(g):
    """scipy sparse input -> the reference's CsrGraph (persistence_csr,
    python/turbotops_ext.cpp:76-99, with its checks and messages)."""
    g = g.tocsr()
    g.sort_indices()
    n = int(g.shape[0])
    indptr = np.asarray(g.indptr, np.int64)
    indices = np.asarray(g.indices, np.int64)
    data = np.asarray(g.data, np.float32)
    if indptr.shape[0] != n + 1 or indices.shape[0] != data.shape[0]:
        raise ValueError("inconsistent CSR arrays")
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
    # entries are checked in order, the index before the weight (as the reference's loop)
    bad_idx = (indices < 0) | (indices >= n)
    bad_w = ~((data >= 0) & np.isfinite(data))
    bad = bad_idx | bad_w
    if bad.any():
        first = int(np.argmax(bad))
        raise ValueError("column index out of range" if bad_idx[first] else "weights must be finite and >= 0")
    rp, ci, w = symmetric_rows(rows, indices, data, n)
    return rp, ci, w, n


def persistence_graph(rp, ci, w, n, maxdim=1, threshold=math.inf, device=0):
    """tops::persistence(const CsrGraph&, maxdim, threshold) (turbotops.hpp:179-207)
    on host CSR arrays (u64 row_ptr, u32 col, f32 weight)."""
    rp = np.ascontiguousarray(rp, np.uint64)
    ci = np.ascontiguousarray(ci, np.uint32)
    w = np.ascontiguousarray(w, np.float32)
    ctx = _context(device)
    out = C.POINTER(capi.Barcode)()
    t0 = time.perf_counter()
    ctx.check(ctx.L.tt_persistence_graph_h(ctx.h, rp.ctypes.data, ci.ctypes.data if ci.size else None,
                                           w.ctypes.data if w.size else None, int(n), int(maxdim),
                                           float(threshold), C.byref(out)))
    return _unpack(ctx, out, maxdim, time.perf_counter() - t0)


def _unpack(ctx, out, maxdim, secs):
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
