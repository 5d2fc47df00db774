"""TEST INFRASTRUCTURE ONLY — ctypes front for the CPU oracle (oracle.cpp).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, as the checker. The product (turbotops_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

KIND = {"l1": 0, "manhattan": 0, "l2": 1, "euclidean": 1, "linf": 2, "chebyshev": 2}


def metric_code(metric: str) -> tuple[int, float]:
    """Metric::parse (metric.hpp:240-253) + Metric::minkowski canonicalisation."""
    if metric in KIND:
        return KIND[metric], {0: 1.0, 1: 2.0, 2: float("inf")}[KIND[metric]]
    if metric.startswith("lp:"):
        v = metric[3:]
        p = float("inf") if v == "inf" else float(np.float32(v))
        if not p >= 1:
            raise ValueError("metric: p must be in [1, inf]")
        if p == 1:
            return 0, 1.0
        if p == 2:
            return 1, 2.0
        if np.isinf(p):
            return 2, p
        return 3, p
    raise ValueError(f"metric: unknown '{metric}'")


_lib = None


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        L.or_set_lp_model.argtypes = [C.c_int]
        L.or_get_lp_model.restype = C.c_int
        L.or_powf.restype = C.c_float
        L.or_powf.argtypes = [C.c_float, C.c_float]
        L.or_rcp.restype = C.c_float
        L.or_rcp.argtypes = [C.c_float]
        L.or_dist.restype = C.c_float
        L.or_dist.argtypes = [C.c_int, C.c_float, P, P, C.c_uint32]
        L.or_dense.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, P]
        L.or_enclosing_radius.restype = C.c_float
        L.or_enclosing_radius.argtypes = [P, C.c_uint32]
        L.or_dim0.restype = C.c_uint64
        L.or_dim0.argtypes = [P, P, P, P, C.c_uint32, C.c_float, C.c_uint32, P, P, P, P, P, P, P, P]
        L.or_emergent.argtypes = [P, P, P, P, C.c_uint32, P, P, C.c_uint64, P, P, P]
        L.or_assemble.restype = C.c_uint64
        L.or_assemble.argtypes = [P, C.c_uint32, C.c_float, P, P, C.c_uint64, P, C.c_uint64, P, P,
                                  C.c_uint64, P]
        L.or_knn.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_uint32, P]
        L.or_knn_rows.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_uint32, C.c_uint32,
                                  C.c_uint32, C.c_uint32, P]
        L.or_knn_graph.restype = C.c_uint64
        L.or_knn_graph.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, P, C.c_uint32, P, P, P]
        L.or_radius_graph.restype = C.c_uint64
        L.or_radius_graph.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_float, P, P, P,
                                      C.c_uint64]
        L.or_mst_h0.restype = C.c_uint64
        L.or_mst_h0.argtypes = [P, C.c_uint32, C.c_uint32, C.c_int, C.c_float, C.c_float, P]
        L.or_redzed_edges.restype = C.c_uint64
        L.or_redzed_edges.argtypes = [P, P, P, P, C.c_uint32, C.c_float, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def _pts(x):
    return np.ascontiguousarray(x, np.float32)


def dense(x: np.ndarray, metric: str) -> np.ndarray:
    x = _pts(x)
    n, dim = x.shape
    k, p = metric_code(metric)
    m = np.empty((n, n), np.float32)
    lib().or_dense(_p(x), n, dim, k, p, _p(m))
    return m


def dist(a, b, metric: str) -> float:
    a, b = _pts(a), _pts(b)
    k, p = metric_code(metric)
    return lib().or_dist(k, p, _p(a), _p(b), a.size)


def enclosing_radius(mat: np.ndarray) -> np.float32:
    mat = np.ascontiguousarray(mat, np.float32)
    return np.float32(lib().or_enclosing_radius(_p(mat), mat.shape[0]))


def dim0(mat=None, csr=None, n=None, thr=float("inf"), maxdim=1) -> dict:
    """Reducer::dim0 on a dense full matrix or a CSR (rp, ci, w)."""
    if mat is not None:
        mat = np.ascontiguousarray(mat, np.float32)
        n = mat.shape[0]
        rp = ci = w = None
        cap = n * (n - 1) // 2
    else:
        rp, ci, w = (np.ascontiguousarray(a) for a in csr)
        cap = ci.size // 2
    eidx = np.empty(cap, np.uint64)
    ed = np.empty(cap, np.float32)
    app = np.empty(cap, np.uint8)
    cidx = np.empty(cap, np.uint64)
    cd = np.empty(cap, np.float32)
    h0 = np.empty(2 * n + 2, np.float32)
    nc = np.zeros(1, np.uint64)
    nh = np.zeros(1, np.uint64)
    m = lib().or_dim0(_p(mat), _p(rp), _p(ci), _p(w), n, thr, maxdim, _p(eidx), _p(ed), _p(app),
                      _p(cidx), _p(cd), _p(nc), _p(h0), _p(nh))
    c = int(nc[0])
    return {"eidx": eidx[:m], "ed": ed[:m], "app": app[:m], "cidx": cidx[:c], "cd": cd[:c],
            "h0": h0[: 2 * int(nh[0])]}


def emergent(mat=None, csr=None, n=None, cidx=None, cd=None) -> dict:
    if mat is not None:
        mat = np.ascontiguousarray(mat, np.float32)
        n = mat.shape[0]
        rp = ci = w = None
    else:
        rp, ci, w = (np.ascontiguousarray(a) for a in csr)
    cidx = np.ascontiguousarray(cidx, np.uint64)
    cd = np.ascontiguousarray(cd, np.float32)
    k = cidx.size
    fi = np.empty(k, np.uint64)
    fd = np.empty(k, np.float32)
    fa = np.empty(k, np.uint8)
    lib().or_emergent(_p(mat), _p(rp), _p(ci), _p(w), n, _p(cidx), _p(cd), k, _p(fi), _p(fd), _p(fa))
    return {"emi": fi, "emd": fd, "emf": fa}


def assemble(mat, thr, sidx, sd, piv) -> dict:
    mat = np.ascontiguousarray(mat, np.float32)
    n = mat.shape[0]
    sidx = np.ascontiguousarray(sidx, np.uint64)
    sd = np.ascontiguousarray(sd, np.float32)
    piv = np.ascontiguousarray(np.sort(piv), np.uint64)
    napp = np.zeros(1, np.uint64)
    cnt = lib().or_assemble(_p(mat), n, thr, _p(sidx), _p(sd), sidx.size, _p(piv), piv.size, None,
                            None, 0, _p(napp))
    ci = np.empty(cnt, np.uint64)
    cd = np.empty(cnt, np.float32)
    lib().or_assemble(_p(mat), n, thr, _p(sidx), _p(sd), sidx.size, _p(piv), piv.size, _p(ci), _p(cd),
                      cnt, _p(napp))
    return {"c2idx": ci, "c2d": cd, "app2n": int(napp[0])}


def knn(x, metric, k) -> np.ndarray:
    x = _pts(x)
    n, dim = x.shape
    kk = min(k, n - 1) if n else 0
    ids = np.empty((n, kk), np.uint32)
    c, p = metric_code(metric)
    lib().or_knn(_p(x), n, dim, c, p, k, _p(ids))
    return ids


def knn_rows(x, metric, k, q0, q1, threads) -> np.ndarray:
    """kNN lists of queries [q0, q1) against the whole cloud, on `threads` threads."""
    x = _pts(x)
    n, dim = x.shape
    kk = min(k, n - 1) if n else 0
    ids = np.empty((q1 - q0, kk), np.uint32)
    c, p = metric_code(metric)
    lib().or_knn_rows(_p(x), n, dim, c, p, k, q0, q1, threads, _p(ids))
    return ids


def knn_graph(x, metric, ids) -> tuple:
    x = _pts(x)
    n, dim = x.shape
    ids = np.ascontiguousarray(ids, np.uint32)
    k = ids.shape[1] if ids.ndim == 2 else 0
    rp = np.empty(n + 1, np.uint64)
    ci = np.empty(2 * n * max(k, 1), np.uint32)
    w = np.empty(2 * n * max(k, 1), np.float32)
    c, p = metric_code(metric)
    nnz = lib().or_knn_graph(_p(x), n, dim, c, p, _p(ids), k, _p(rp), _p(ci), _p(w))
    return rp, ci[:nnz], w[:nnz]


def radius_graph(x, metric, tau) -> tuple:
    x = _pts(x)
    n, dim = x.shape
    c, p = metric_code(metric)
    rp = np.empty(n + 1, np.uint64)
    nnz = lib().or_radius_graph(_p(x), n, dim, c, p, tau, _p(rp), None, None, 0)
    ci = np.empty(nnz, np.uint32)
    w = np.empty(nnz, np.float32)
    lib().or_radius_graph(_p(x), n, dim, c, p, tau, _p(rp), _p(ci), _p(w), nnz)
    return rp, ci, w


def mst_h0(x, metric, thr=float("inf")) -> np.ndarray:
    x = _pts(x)
    n, dim = x.shape
    c, p = metric_code(metric)
    bars = np.empty(2 * (n + 1), np.float32)
    nb = lib().or_mst_h0(_p(x), n, dim, c, p, thr, _p(bars))
    return bars[: 2 * nb]


def redzed_edges(mat=None, csr=None, n=None, thr=float("inf")) -> tuple:
    if mat is not None:
        mat = np.ascontiguousarray(mat, np.float32)
        n = mat.shape[0]
        rp = ci = w = None
        cap = n * (n - 1) // 2
    else:
        rp, ci, w = (np.ascontiguousarray(a) for a in csr)
        cap = ci.size // 2
    d = np.empty(cap, np.float32)
    v = np.empty(2 * cap, np.int32)
    m = lib().or_redzed_edges(_p(mat), _p(rp), _p(ci), _p(w), n, thr, _p(d), _p(v))
    return d[:m], v[: 2 * m]
