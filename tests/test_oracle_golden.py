"""Pin the CPU oracle to the reference's own outputs (golden fixtures).

Bit-exact for every integer/index output and every distance. Non-integer p
Lp fixtures (the *_a64 ones) come from the reference built on an aarch64 host
(the GB300 machine's Grace CPU), whose reciprocal estimate and libm the oracle
models (oracle/aarch64_math.h); the other fixtures are host-independent.
"""
import numpy as np
import pytest

from golden_io import cases, ids, thr_of
from oracle import oracle as O

DENSE = cases("dense")
ASM = cases("asm")
KNN = cases("knn")
RADIUS = cases("radius")
MST = cases("mst")
RZD = cases("rzd")
RZS = cases("rzs")
SDIM0 = cases("sdim0")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("c", DENSE, ids=ids(DENSE))
def test_dense_matrix(c):
    n = c["x"].shape[0]
    m = O.dense(c["x"], c["metric"]).ravel()
    ref = c["mat"]
    assert np.array_equal(bits(m), bits(ref))
    assert bits(O.enclosing_radius(m.reshape(n, n))) == bits(c["encl"])[0]


@pytest.mark.parametrize("c", ASM, ids=ids(ASM))
def test_dim0_and_assemble(c):
    mat = O.dense(c["x"], c["metric"])
    thr = thr_of(c["params"]["thr"])
    if np.isinf(thr):
        thr = O.enclosing_radius(mat)
    assert bits(thr) == bits(c["thr"])[0]
    r = O.dim0(mat=mat, thr=thr, maxdim=2)
    for k in ["eidx", "app", "cidx", "h0"]:
        assert np.array_equal(r[k], c[k]), k
    assert np.array_equal(bits(r["ed"]), bits(c["ed"]))
    assert np.array_equal(bits(r["cd"]), bits(c["cd"]))
    e = O.emergent(mat=mat, cidx=r["cidx"], cd=r["cd"])
    assert np.array_equal(e["emi"], c["emi"])
    assert np.array_equal(e["emf"], c["emf"])
    a = O.assemble(mat, thr, r["eidx"], r["ed"], c["piv"])
    assert np.array_equal(a["c2idx"], c["c2idx"])
    assert np.array_equal(bits(a["c2d"]), bits(c["c2d"]))
    assert a["app2n"] == int(c["app2n"][0])


@pytest.mark.parametrize("c", KNN, ids=ids(KNN))
def test_knn_lists_and_graph(c):
    k = c["params"]["k"]
    ids_ = O.knn(c["x"], c["metric"], k)
    assert np.array_equal(ids_.ravel(), c["ids"])
    rp, ci, w = O.knn_graph(c["x"], c["metric"], ids_)
    assert np.array_equal(rp, c["rp"]) and np.array_equal(ci, c["ci"])
    assert np.array_equal(bits(w), bits(c["w"]))


@pytest.mark.parametrize("c", RADIUS, ids=ids(RADIUS))
def test_radius_graph(c):
    rp, ci, w = O.radius_graph(c["x"], c["metric"], thr_of(c["params"]["tau"]))
    assert np.array_equal(rp, c["rp"]) and np.array_equal(ci, c["ci"])
    assert np.array_equal(bits(w), bits(c["w"]))


@pytest.mark.parametrize("c", MST, ids=ids(MST))
def test_mst_h0(c):
    b = O.mst_h0(c["x"], c["metric"], thr_of(c["params"]["thr"]))
    assert np.array_equal(bits(b), bits(c["h0"]))


@pytest.mark.parametrize("c", RZD, ids=ids(RZD))
def test_redzed_dense_edges(c):
    mat = O.dense(c["x"], c["metric"])
    d, v = O.redzed_edges(mat=mat, thr=float(c["thr"][0]))
    assert np.array_equal(bits(d), bits(c["rd"])) and np.array_equal(v, c["rv"])


@pytest.mark.parametrize("c", RZS, ids=ids(RZS))
def test_redzed_sparse_edges(c):
    csr = (c["knn_rp"], c["knn_ci"], c["knn_w"])
    d, v = O.redzed_edges(csr=csr, n=c["x"].shape[0])
    assert np.array_equal(bits(d), bits(c["rd"])) and np.array_equal(v, c["rv"])


@pytest.mark.parametrize("c", SDIM0, ids=ids(SDIM0))
def test_sparse_dim0(c):
    csr = (c["g_rp"], c["g_ci"], c["g_w"])
    n = c["x"].shape[0]
    r = O.dim0(csr=csr, n=n, maxdim=2)
    for k in ["eidx", "app", "cidx", "h0"]:
        assert np.array_equal(r[k], c[k]), k
    e = O.emergent(csr=csr, n=n, cidx=r["cidx"], cd=r["cd"])
    assert np.array_equal(e["emi"], c["emi"]) and np.array_equal(e["emf"], c["emf"])
