"""CUDA path vs the reference goldens and the oracle: exact kNN lists, the
symmetric kNN graph, the radius graph and the complete-graph MST (H0)."""
import os

import numpy as np
import pytest

from golden_io import cases, ids, thr_of
from gpu_util import bits, ctx, dev, host
from oracle import oracle as O
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu

KNN = cases("knn")
RADIUS = cases("radius")
MST = cases("mst")


@pytest.mark.parametrize("c", KNN, ids=ids(KNN))
def test_knn_vs_reference(c):
    k = c["params"]["k"]
    x = dev(c["x"])
    i, d = ops.knn(ctx(), x, k, c["metric"])
    assert np.array_equal(host(i).view(np.uint32).ravel(), c["ids"])
    rp, ci, w = ops.knn_graph(ctx(), x, k, c["metric"])
    assert np.array_equal(host(rp).view(np.uint64), c["rp"])
    assert np.array_equal(host(ci).view(np.uint32), c["ci"])
    assert np.array_equal(bits(host(w)), bits(c["w"]))


@pytest.mark.parametrize("c", RADIUS, ids=ids(RADIUS))
def test_radius_vs_reference(c):
    rp, ci, w = ops.radius_graph(ctx(), dev(c["x"]), thr_of(c["params"]["tau"]), c["metric"])
    assert np.array_equal(host(rp).view(np.uint64), c["rp"])
    assert np.array_equal(host(ci).view(np.uint32), c["ci"])
    assert np.array_equal(bits(host(w)), bits(c["w"]))


@pytest.mark.parametrize("c", MST, ids=ids(MST))
def test_mst_vs_reference(c):
    d = ops.mst_deaths(ctx(), dev(c["x"]), c["metric"])
    bars = ops.h0_bars(d, thr_of(c["params"]["thr"]))
    assert np.array_equal(bits(bars), bits(c["h0"]))


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5", "lp:2.5"])
@pytest.mark.parametrize("n,dim,k,kind", [(1000, 32, 15, "gauss"), (700, 3, 8, "grid"), (513, 5, 31, "gauss"),
                                          (129, 16, 1, "gauss"), (6, 4, 15, "gauss")])
def test_knn_graph_vs_oracle(metric, n, dim, k, kind):
    x = synth.gauss(n, dim, n + dim) if kind == "gauss" else synth.grid(n, dim, 12, n)
    i, d = ops.knn(ctx(), dev(x), k, metric)
    ref = O.knn(x, metric, k)
    assert np.array_equal(host(i).view(np.uint32), ref)
    rp, ci, w = ops.knn_graph(ctx(), dev(x), k, metric)
    orp, oci, ow = O.knn_graph(x, metric, ref)
    assert np.array_equal(host(rp).view(np.uint64), orp)
    assert np.array_equal(host(ci).view(np.uint32), oci)
    assert np.array_equal(bits(host(w)), bits(ow))


@pytest.mark.parametrize("metric", ["lp:1.5", "lp:2.5"])
@pytest.mark.parametrize("n,dim,kind", [(5000, 8, "gauss"), (4500, 3, "grid"), (4200, 32, "gmm")])
def test_lp_knn_in_cell_order_vs_oracle(metric, n, dim, kind):
    """From 4,096 points the Lp scan takes its queries cell by cell (nearest
    of strided pivots): the lists are the oracle's, ties on the lattice
    included."""
    if kind == "gmm":
        x = synth.gmm(n, dim, 6, n)
    elif kind == "grid":
        x = synth.grid(n, dim, 25, n)
    else:
        x = synth.gauss(n, dim, n + dim)
    i, _ = ops.knn(ctx(), dev(x), 15, metric)
    assert np.array_equal(host(i).view(np.uint32), O.knn_rows(x, metric, 15, 0, n, os.cpu_count() or 1))


def test_lp_scans_refuse_dimensions_above_64():
    """The cell order of the Lp scans is skipped where the scans refuse the
    dimension: the caller gets the scans' own error, and the context keeps
    working."""
    x = synth.gauss(4100, 65, 1)
    for run in (lambda: ops.knn(ctx(), dev(x), 15, "lp:1.5"), lambda: ops.mst_deaths(ctx(), dev(x), "lp:1.5")):
        with pytest.raises(Exception, match="1 <= dim <= 64"):
            run()
    y = synth.gauss(4100, 8, 2)
    i, _ = ops.knn(ctx(), dev(y), 15, "lp:1.5")
    assert i.shape == (4100, 15)


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5"])
@pytest.mark.parametrize("n,dim", [(2000, 32), (1500, 3), (300, 7), (2, 3)])
def test_mst_vs_oracle(metric, n, dim):
    x = synth.gauss(n, dim, 3 * n + dim) if dim != 3 else synth.grid(n, 3, 20, n)
    d = ops.mst_deaths(ctx(), dev(x), metric)
    assert np.array_equal(bits(ops.h0_bars(d)), bits(O.mst_h0(x, metric)))


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5"])
@pytest.mark.parametrize("n,dim,kind", [(4200, 16, "gmm"), (5000, 3, "grid"), (4500, 2, "grid"),
                                        (4096, 8, "gauss")])
def test_mst_knn_seeded_rounds_vs_oracle(metric, n, dim, kind):
    """From 4,096 points the Borůvka rounds start from 16-nearest-neighbour
    lists and scan only the interior points that can still carry their
    component's minimum: the same deaths as the oracle's Prim tree, also on
    lattices where distances tie everywhere and on well-separated clusters
    (whose last rounds have no list entry outside the component)."""
    if kind == "gmm":
        x = synth.gmm(n, dim, 6, n)
    elif kind == "grid":
        x = synth.grid(n, dim, 90 if dim == 2 else 25, n)
    else:
        x = synth.gauss(n, dim, n + dim)
    d = ops.mst_deaths(ctx(), dev(x), metric)
    assert np.array_equal(bits(ops.h0_bars(d)), bits(O.mst_h0(x, metric)))


def test_radius_vs_oracle_ties():
    x = synth.grid(800, 4, 7, 3)
    for metric, tau in [("l1", 3.0), ("linf", 1.0), ("l2", 2.0), ("lp:1.5", 2.5), ("lp:3", 2.0)]:
        rp, ci, w = ops.radius_graph(ctx(), dev(x), tau, metric)
        orp, oci, ow = O.radius_graph(x, metric, tau)
        assert np.array_equal(host(rp).view(np.uint64), orp)
        assert np.array_equal(host(ci).view(np.uint32), oci)
        assert np.array_equal(bits(host(w)), bits(ow))


@pytest.mark.parametrize("m", [1500, 3000])
def test_knn_graph_hub_rows(m):
    """A hub: the origin is in every list of m points on a sphere, so its row
    holds m + k entries — the row-local sort below 2048 entries, the global
    sort of all entries above; both must give the oracle's CSR."""
    rng = np.random.default_rng(m)
    s = rng.normal(size=(m, 64))   # in R^64 random unit vectors are ~sqrt(2) apart
    s /= np.linalg.norm(s, axis=1, keepdims=True)
    x = np.ascontiguousarray(np.vstack([np.zeros((1, 64)), s]), dtype=np.float32)
    k = 4
    ref = O.knn(x, "l2", k)
    rp, ci, w = ops.knn_graph(ctx(), dev(x), k, "l2")
    orp, oci, ow = O.knn_graph(x, "l2", ref)
    assert np.diff(orp)[0] >= m
    assert np.array_equal(host(rp).view(np.uint64), orp)
    assert np.array_equal(host(ci).view(np.uint32), oci)
    assert np.array_equal(bits(host(w)), bits(ow))
