"""The host reduction (turbotops_gb300/csrc/tt_reduce.cpp, the reference's
Reducer::compute_pairs, rips.hpp:874-978) on the CPU, against the reference's
own outputs: whole diagrams (dim0 H0 + reduced H1/H2), and the dimension-1
pivot sets the reference dumped. The columns come from the oracle's dim0,
emergent and assemble restatements (themselves pinned to the reference by
test_oracle_golden.py); the reduction is the product's source, compiled here
with the host compiler through tests/host_reduce_shim.cpp."""
import ctypes as C
import json
import os
import subprocess

import numpy as np
import pytest

from golden_io import GOLDEN, canonical, cases, ids, thr_of
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BARS = cases("bars")
ASM = cases("asm")


@pytest.fixture(scope="module")
def shim(tmp_path_factory):
    so = str(tmp_path_factory.mktemp("hr") / "libhostreduce.so")
    src = [os.path.join(ROOT, "tests", "host_reduce_shim.cpp"),
           os.path.join(ROOT, "turbotops_gb300", "csrc", "tt_reduce.cpp")]
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread", "-o", so] + src, check=True)
    L = C.CDLL(so)
    P = C.c_void_p
    L.hr_set_threads.argtypes = [C.c_uint]
    L.hr_assemble.restype = C.c_int
    L.hr_assemble.argtypes = [P, P, P, P, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, P, P, C.c_uint64, P,
                              C.c_uint64, P, P, C.c_uint64, P, P, P, C.c_uint64, P, P]
    L.hr_compute_pairs.restype = C.c_int
    L.hr_compute_pairs.argtypes = [P, P, P, P, C.c_uint32, C.c_float, C.c_uint32, C.c_uint32, P, P, C.c_uint64,
                                   P, P, P, P, P, P, P, P]
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def reduce(L, mat, thr, dim, maxdim, cidx, cd, emi=None, emf=None):
    cidx = np.ascontiguousarray(cidx, np.uint64)
    cd = np.ascontiguousarray(cd, np.float32)
    k = cidx.size
    birth = np.empty(k + 1, np.float32)
    death = np.empty(k + 1, np.float32)
    piv = np.empty(k + 1, np.uint64)
    nb, npv, em = (np.zeros(1, np.uint64) for _ in range(3))
    mat = np.ascontiguousarray(mat, np.float32)
    rc = L.hr_compute_pairs(_p(mat), None, None, None, mat.shape[0], float(thr), dim, maxdim, _p(cidx), _p(cd), k,
                            _p(emi), _p(emf), _p(birth), _p(death), _p(nb), _p(piv), _p(npv), _p(em))
    assert rc == 0
    b = int(nb[0])
    return birth[:b], death[:b], piv[: int(npv[0])], int(em[0])


def _cx_args(cx):
    """(mat, rp, ci, w, n) pointers for a dense matrix or ((rp, ci, w), n)."""
    if isinstance(cx, tuple):
        (rp, ci, w), n = cx
        return None, _p(rp), _p(ci), _p(w), n
    return _p(cx), None, None, None, cx.shape[0]


def reduce_any(L, cx, thr, dim, maxdim, cidx, cd):
    """compute_pairs(dim) (host emergent test) on a dense or CSR complex."""
    cidx = np.ascontiguousarray(cidx, np.uint64)
    cd = np.ascontiguousarray(cd, np.float32)
    k = cidx.size
    birth, death = np.empty(k + 1, np.float32), np.empty(k + 1, np.float32)
    piv = np.empty(k + 1, np.uint64)
    nb, npv, em = (np.zeros(1, np.uint64) for _ in range(3))
    rc = L.hr_compute_pairs(*_cx_args(cx), float(thr), dim, maxdim, _p(cidx), _p(cd), k, None, None, _p(birth),
                            _p(death), _p(nb), _p(piv), _p(npv), _p(em))
    assert rc == 0
    return birth[: int(nb[0])], death[: int(nb[0])], piv[: int(npv[0])]


def host_assemble(L, cx, thr, dim, maxdim, sidx, sd, piv, want_next):
    """The product's host assemble (tt_reduce.cpp) through the shim."""
    sidx = np.ascontiguousarray(sidx, np.uint64)
    sd = np.ascontiguousarray(sd, np.float32)
    piv = np.ascontiguousarray(np.sort(piv), np.uint64)
    cap = ncap = 1 << 16
    while True:
        ci_, cd_ = np.empty(cap, np.uint64), np.empty(cap, np.float32)
        ni_, nd_ = np.empty(ncap, np.uint64), np.empty(ncap, np.float32)
        nc, nn, na = (np.zeros(1, np.uint64) for _ in range(3))
        rc = L.hr_assemble(*_cx_args(cx), float(thr), dim, maxdim, _p(sidx), _p(sd), sidx.size, _p(piv), piv.size,
                           _p(ci_), _p(cd_), cap, _p(nc), _p(ni_) if want_next else None, _p(nd_), ncap, _p(nn),
                           _p(na))
        if rc == -2:
            cap, ncap = max(cap, int(nc[0])), max(ncap, int(nn[0]))
            continue
        assert rc == 0
        c, m = int(nc[0]), int(nn[0])
        return ci_[:c], cd_[:c], ni_[:m], nd_[:m]


def higher(L, cx, thr, maxdim, eidx, ed, piv):
    """Dimensions 2..maxdim: host assemble then compute_pairs, per dimension."""
    rows, sidx, sd = [], eidx, ed
    for dim in range(1, maxdim):
        ci_, cd_, ni_, nd_ = host_assemble(L, cx, thr, dim, maxdim, sidx, sd, piv, dim + 1 < maxdim)
        b, d, piv = reduce_any(L, cx, thr, dim + 1, maxdim, ci_, cd_)
        rows.append(np.column_stack([np.full(len(b), dim + 1, np.float32), b, d]))
        sidx, sd = ni_, nd_
    return rows


def diagram(L, x, metric, maxdim, host_emergent=False):
    """tops::persistence on a dense cloud: threshold = enclosing radius,
    dim0 H0, compute_pairs(1), assemble(1) + compute_pairs(2) (the oracle's
    assemble), and above dimension 2 the product's host assemble."""
    mat = O.dense(x, metric)
    thr = O.enclosing_radius(mat)
    r = O.dim0(mat=mat, thr=thr, maxdim=maxdim)
    h0 = r["h0"].reshape(-1, 2)
    rows = [np.column_stack([np.zeros(len(h0), np.float32), h0])]
    if maxdim >= 1:
        if host_emergent:
            emi = emf = None
        else:
            e = O.emergent(mat=mat, cidx=r["cidx"], cd=r["cd"])
            emi, emf = e["emi"], e["emf"]
        b, d, piv, _ = reduce(L, mat, thr, 1, maxdim, r["cidx"], r["cd"], emi, emf)
        rows.append(np.column_stack([np.ones(len(b), np.float32), b, d]))
        if maxdim >= 3:
            rows += higher(L, mat, thr, maxdim, r["eidx"], r["ed"], piv)
        elif maxdim == 2:
            a = O.assemble(mat, thr, r["eidx"], r["ed"], piv)
            b2, d2, _, _ = reduce(L, mat, thr, 2, maxdim, a["c2idx"], a["c2d"])
            rows.append(np.column_stack([np.full(len(b2), 2, np.float32), b2, d2]))
    return canonical(np.concatenate(rows).astype(np.float32))


@pytest.mark.parametrize("c", BARS, ids=ids(BARS))
def test_diagram_vs_reference(shim, c):
    got = diagram(shim, c["x"], c["metric"], c["params"]["maxdim"])
    ref = canonical(c["bars"])
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("c", [b for b in BARS if b["params"]["maxdim"] >= 1], ids=ids([b for b in BARS if b["params"]["maxdim"] >= 1]))
def test_host_emergent_test_equals_precomputed(shim, c):
    """The emergent-pair test evaluated by the reducer itself (the path of
    dimension >= 2) gives the dimension-1 diagram the precomputed one gives."""
    a = diagram(shim, c["x"], c["metric"], 1)
    b = diagram(shim, c["x"], c["metric"], 1, host_emergent=True)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.mark.parametrize("c", ASM, ids=ids(ASM))
def test_dim1_pivots_vs_reference(shim, c):
    """The set of dimension-1 pivots (death triangles, the input of assemble)
    equals the reference's, with its threshold and columns."""
    thr = np.float32(c["thr"][0])
    b, d, piv, _ = reduce(shim, O.dense(c["x"], c["metric"]), thr, 1, 2, c["cidx"], c["cd"], c["emi"], c["emf"])
    assert np.array_equal(np.sort(piv), np.sort(c["piv"]))


def test_torus_config_pivots_vs_reference(shim):
    """Configuration 1 (torus, 1000 points, L2, enclosing radius): the
    reference's 393,249 edges reduce to its dimension-1 pivot set."""
    from turbotops_gb300 import synth
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))["torus1000_l2"]
    ref = np.load(os.path.join(GOLDEN, "cfg_torus1000_piv.npz"))["piv"]
    mat = O.dense(synth.torus(), "l2")
    thr = O.enclosing_radius(mat)
    assert float(thr) == cfg["thr"]
    r = O.dim0(mat=mat, thr=thr, maxdim=2)
    e = O.emergent(mat=mat, cidx=r["cidx"], cd=r["cd"])
    _, _, piv, _ = reduce(shim, mat, thr, 1, 2, r["cidx"], r["cd"], e["emi"], e["emf"])
    assert np.array_equal(np.sort(piv), np.sort(ref))


@pytest.mark.parametrize("metric", ["l1", "linf"])
def test_lattice_config_pivots_vs_reference(shim, metric):
    """Configuration 2 (3000 distinct points of {0..15}^4, enclosing radius):
    the reference's tie-heavy dimension-1 columns reduce to its pivot set.
    C(3000, 3) > 2^32, so the queue keeps wide entries here, and most
    cofacets share their diameter with many others."""
    from turbotops_gb300 import synth
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))[f"lattice3000_{metric}"]
    ref = np.load(os.path.join(GOLDEN, f"cfg_lattice3000_{metric}_piv.npz"))["piv"]
    mat = O.dense(synth.lattice(), metric)
    thr = O.enclosing_radius(mat)
    assert float(thr) == cfg["thr"]
    r = O.dim0(mat=mat, thr=thr, maxdim=2)
    e = O.emergent(mat=mat, cidx=r["cidx"], cd=r["cd"])
    _, _, piv, _ = reduce(shim, mat, thr, 1, 2, r["cidx"], r["cd"], e["emi"], e["emf"])
    assert np.array_equal(np.sort(piv), np.sort(ref))


GBARS = cases("gbars")


def reduce_csr(L, csr, n, thr, cidx, cd, emi, emf):
    rp, ci, w = (np.ascontiguousarray(a) for a in csr)
    cidx = np.ascontiguousarray(cidx, np.uint64)
    cd = np.ascontiguousarray(cd, np.float32)
    k = cidx.size
    birth = np.empty(k + 1, np.float32)
    death = np.empty(k + 1, np.float32)
    piv = np.empty(k + 1, np.uint64)
    nb, npv, em = (np.zeros(1, np.uint64) for _ in range(3))
    rc = L.hr_compute_pairs(None, _p(rp), _p(ci), _p(w), n, float(thr), 1, 1, _p(cidx), _p(cd), k, _p(emi),
                            _p(emf), _p(birth), _p(death), _p(nb), _p(piv), _p(npv), _p(em))
    assert rc == 0
    b = int(nb[0])
    return birth[:b], death[:b]


@pytest.mark.parametrize("c", GBARS, ids=ids(GBARS))
def test_knn_graph_diagram_vs_reference(shim, c):
    """tops::persistence on the kNN graph of a cloud (the reference CLI's
    --graph knn, maxdim 1): dim0 H0 + compute_pairs(1) over the CSR complex,
    whole diagram bit for bit (the graph-complex path of the reduction)."""
    x, metric = c["x"], c["metric"]
    n = x.shape[0]
    thr = thr_of(c["params"]["thr"])
    csr = O.knn_graph(x, metric, O.knn(x, metric, c["params"]["k"]))
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=1)
    e = O.emergent(csr=csr, n=n, cidx=r["cidx"], cd=r["cd"])
    b, d = reduce_csr(shim, csr, n, thr, r["cidx"], r["cd"], e["emi"], e["emf"])
    h0 = r["h0"].reshape(-1, 2)
    got = canonical(np.concatenate([np.column_stack([np.zeros(len(h0), np.float32), h0]),
                                    np.column_stack([np.ones(len(b), np.float32), b, d])]).astype(np.float32))
    ref = canonical(c["bars"])
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def graph_pairs(L, csr, n, thr, cidx, cd):
    rp, ci, w = (np.ascontiguousarray(a) for a in csr)
    cidx = np.ascontiguousarray(cidx, np.uint64)
    cd = np.ascontiguousarray(cd, np.float32)
    k = cidx.size
    birth = np.empty(k + 1, np.float32)
    death = np.empty(k + 1, np.float32)
    bi = np.empty(k + 1, np.uint64)
    di = np.empty(k + 1, np.uint64)
    nb, nt = np.zeros(1, np.uint64), np.zeros(1, np.uint64)
    L.hr_graph_pairs_dim1.restype = C.c_int
    L.hr_graph_pairs_dim1.argtypes = [C.c_void_p] * 3 + [C.c_uint32, C.c_float] + [C.c_void_p] * 2 + \
        [C.c_uint64] + [C.c_void_p] * 6
    assert L.hr_graph_pairs_dim1(_p(rp), _p(ci), _p(w), n, float(thr), _p(cidx), _p(cd), k, _p(birth), _p(death),
                                 _p(bi), _p(di), _p(nb), _p(nt)) == 0
    b = int(nb[0])
    return birth[:b], death[:b]


@pytest.mark.parametrize("c", GBARS, ids=ids(GBARS))
def test_knn_graph_boundary_diagram_vs_reference(shim, c):
    """The boundary reduction of a graph complex's triangles
    (graph_pairs_dim1, which the sparse front end uses for kNN graphs) gives
    the reference CLI's whole diagram bit for bit."""
    x, metric = c["x"], c["metric"]
    n = x.shape[0]
    thr = thr_of(c["params"]["thr"])
    csr = O.knn_graph(x, metric, O.knn(x, metric, c["params"]["k"]))
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=1)
    b, d = graph_pairs(shim, csr, n, thr, r["cidx"], r["cd"])
    h0 = r["h0"].reshape(-1, 2)
    got = canonical(np.concatenate([np.column_stack([np.zeros(len(h0), np.float32), h0]),
                                    np.column_stack([np.ones(len(b), np.float32), b, d])]).astype(np.float32))
    ref = canonical(c["bars"])
    assert got.shape == ref.shape
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("seed", range(12))
def test_graph_boundary_equals_coboundary_in_order(shim, seed):
    """graph_pairs_dim1 and compute_pairs(1) emit the same bars in the same
    order on kNN and radius graphs (ties from lattice points, finite
    thresholds)."""
    from turbotops_gb300 import synth
    rng = np.random.default_rng(100 + seed)
    n = int(rng.integers(30, 200))
    if seed % 3 == 0:
        x, metric = synth.uniform(n, 3, seed), "l2"
    elif seed % 3 == 1:
        x, metric = synth.grid(min(n, 216), 3, 6, seed), ["l1", "linf"][seed % 2]
    else:
        x, metric = synth.circles(1, n, 0.1, seed)[0], "l2"
    n = x.shape[0]
    if seed % 2:
        csr = O.knn_graph(x, metric, O.knn(x, metric, int(rng.integers(3, 10))))
    else:
        csr = O.radius_graph(x, metric, 2.0 if metric != "l2" else 0.35)
    thr = float("inf") if seed % 4 < 2 else float(np.quantile(csr[2], 0.7))
    thr = np.float32(thr)
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=1)
    e = O.emergent(csr=csr, n=n, cidx=r["cidx"], cd=r["cd"])
    b1, d1 = reduce_csr(shim, csr, n, thr, r["cidx"], r["cd"], e["emi"], e["emf"])
    b2, d2 = graph_pairs(shim, csr, n, thr, r["cidx"], r["cd"])
    assert np.array_equal(b1.view(np.uint32), b2.view(np.uint32))
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


def _csr(n, edges):
    """Symmetric CSR (rows ascending) of an undirected weighted edge list."""
    rows = [[] for _ in range(n)]
    for u, v, w in edges:
        rows[u].append((v, w))
        rows[v].append((u, w))
    rp = np.zeros(n + 1, np.uint64)
    ci, ww = [], []
    for u in range(n):
        for v, w in sorted(rows[u]):
            ci.append(v)
            ww.append(w)
        rp[u + 1] = len(ci)
    return rp, np.array(ci, np.uint32), np.array(ww, np.float32)


@pytest.mark.parametrize("n,edges", [
    (3, []),                                                          # no edges
    (2, [(0, 1, 1.0)]),                                               # one edge, no column
    (3, [(0, 1, 1.0), (1, 2, 1.0), (0, 2, 1.0)]),                     # a triangle of ties
    (4, [(0, 1, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 0, 1.0)]),        # an essential 4-cycle
    (4, [(0, 1, 1.0), (1, 2, 1.0), (2, 3, 1.0), (3, 0, 1.0), (0, 2, 1.5)]),   # the cycle dies at 1.5
    (5, [(0, 1, 0.5), (1, 2, 0.5), (2, 0, 2.0), (2, 3, 0.5), (3, 4, 0.5), (4, 2, 2.0), (0, 3, 3.0)]),
])
def test_graph_boundary_small_graphs(shim, n, edges):
    csr = _csr(n, edges)
    thr = np.float32(np.inf)
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=1)
    e = O.emergent(csr=csr, n=n, cidx=r["cidx"], cd=r["cd"])
    b1, d1 = reduce_csr(shim, csr, n, thr, r["cidx"], r["cd"], e["emi"], e["emf"])
    b2, d2 = graph_pairs(shim, csr, n, thr, r["cidx"], r["cd"])
    assert np.array_equal(b1.view(np.uint32), b2.view(np.uint32))
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))


@pytest.mark.parametrize("case", ["torus_dim1", "torus_dim2", "lattice_l1_dim1", "lattice_linf_dim1", "knn5k"])
def test_parallel_reduction_equals_sequential(shim, case):
    """The batch-parallel reduction (columns reduced against a snapshot of the
    pivots, committed in order, clashes reduced again) gives the sequential
    algorithm's bars in the same order, the same pivots and the same
    emergent count (the configuration-2 lattice at full size, a 500-point
    torus in dimensions 1 and 2, a 5000-point kNN complex)."""
    from turbotops_gb300 import synth
    if case.startswith("knn"):
        x = synth.gmm(5000, 32, seed=9)
        ids = O.knn(x, "l2", 15)
        csr = O.knn_graph(x, "l2", ids)
        n = x.shape[0]
        r = O.dim0(csr=csr, n=n, maxdim=1)
        e = O.emergent(csr=csr, n=n, cidx=r["cidx"], cd=r["cd"])
        out = []
        for t in (1, 8):
            shim.hr_set_threads(t)
            out.append(reduce_csr(shim, csr, n, np.float32(np.inf), r["cidx"], r["cd"], e["emi"], e["emf"]))
    else:
        x = synth.torus(500, seed=31) if case.startswith("torus") else synth.lattice()
        metric = "l2" if case.startswith("torus") else case.split("_")[1]
        mat = O.dense(x, metric)
        thr = O.enclosing_radius(mat)
        r = O.dim0(mat=mat, thr=thr, maxdim=2)
        e = O.emergent(mat=mat, cidx=r["cidx"], cd=r["cd"])
        shim.hr_set_threads(1)
        b1, d1, piv, em = reduce(shim, mat, thr, 1, 2, r["cidx"], r["cd"], e["emi"], e["emf"])
        if case.endswith("dim1"):
            out = [(b1, d1, piv, em)]
            shim.hr_set_threads(8)
            out.append(reduce(shim, mat, thr, 1, 2, r["cidx"], r["cd"], e["emi"], e["emf"]))
        else:
            a = O.assemble(mat, thr, r["eidx"], r["ed"], piv)
            out = []
            for t in (1, 8):
                shim.hr_set_threads(t)
                out.append(reduce(shim, mat, thr, 2, 2, a["c2idx"], a["c2d"]))
    shim.hr_set_threads(0)
    for a, b in zip(out[0], out[1]):
        if isinstance(a, np.ndarray):
            assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                                  b.view(np.uint32) if b.dtype == np.float32 else b)
        else:
            assert a == b


HBARS = cases("hbars")


@pytest.mark.parametrize("c", HBARS, ids=ids(HBARS))
def test_graph_higher_dims_vs_reference(shim, c):
    """Flag complexes of kNN and radius graphs up to maxdim 3 (the reference
    CLI's diagrams): the oracle's sparse dim0, then compute_pairs(1) and the
    product's host assemble + compute_pairs for every higher dimension."""
    x, metric, args, maxdim = c["x"], c["metric"], c["params"]["args"], c["params"]["maxdim"]
    n = x.shape[0]
    if args[0] == "--graph":
        csr = O.knn_graph(x, metric, O.knn(x, metric, int(args[3])))
        thr = np.float32(np.inf)
    else:
        thr = np.float32(args[1])
        csr = O.radius_graph(x, metric, thr)
    csr = tuple(np.ascontiguousarray(a) for a in csr)
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=maxdim)
    h0 = r["h0"].reshape(-1, 2)
    rows = [np.column_stack([np.zeros(len(h0), np.float32), h0])]
    b, d, piv = reduce_any(shim, (csr, n), thr, 1, maxdim, r["cidx"], r["cd"])
    rows.append(np.column_stack([np.ones(len(b), np.float32), b, d]))
    rows += higher(shim, (csr, n), thr, maxdim, r["eidx"], r["ed"], piv)
    got = canonical(np.concatenate(rows).astype(np.float32))
    got = got[got[:, 1] != got[:, 2]]
    ref = canonical(c["bars"])
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))


def test_graph_boundary_store_cap_and_triangle_limit(shim):
    """The boundary reduction gives up (for compute_pairs) once its stored
    fill-in passes the cap, and returns the same bars under a cap it stays
    within."""
    from turbotops_gb300 import synth
    x = synth.circles(1, 150, 0.1, 7)[0]
    csr = O.knn_graph(x, "l2", O.knn(x, "l2", 8))
    n = x.shape[0]
    thr = np.float32(np.inf)
    r = O.dim0(csr=csr, n=n, thr=thr, maxdim=1)
    rp, ci, w = (np.ascontiguousarray(a) for a in csr)
    cidx = np.ascontiguousarray(r["cidx"], np.uint64)
    cd = np.ascontiguousarray(r["cd"], np.float32)
    k = cidx.size
    fn = shim.hr_graph_pairs_dim1_capped
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * 3 + [C.c_uint32, C.c_float] + [C.c_void_p] * 2 + [C.c_uint64, C.c_uint64] + \
        [C.c_void_p] * 3

    def run(cap):
        birth, death = np.empty(k + 1, np.float32), np.empty(k + 1, np.float32)
        nb = np.zeros(1, np.uint64)
        st = fn(_p(rp), _p(ci), _p(w), n, float(thr), _p(cidx), _p(cd), k, cap, _p(birth), _p(death), _p(nb))
        return st, birth[: int(nb[0])], death[: int(nb[0])]
    assert run(4)[0] == 1
    st, b, d = run(1 << 40)
    assert st == 0
    b0, d0 = graph_pairs(shim, csr, n, thr, r["cidx"], r["cd"])
    assert np.array_equal(b.view(np.uint32), b0.view(np.uint32)) and np.array_equal(d.view(np.uint32), d0.view(np.uint32))
