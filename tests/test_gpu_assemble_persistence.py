"""CUDA path vs the reference: dim-2 assemble (with the reference's own
dimension-1 pivots) and whole diagrams through tt_persistence_h (GPU front
end + host reduction), compared bar for bar in the CLI's canonical order."""
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from golden_io import GOLDEN, canonical, cases, ids, thr_of
from gpu_util import bits, ctx, decode_keys, dev, host
from oracle import oracle as O
import turbotops_gb300 as tg
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu

ASM = cases("asm")
BARS = cases("bars")


def sha(*arrs):
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


@pytest.mark.parametrize("c", ASM, ids=ids(ASM))
def test_assemble_vs_reference(c):
    mat, enc = ops.make_dense(ctx(), dev(c["x"]), c["metric"])
    thr = thr_of(c["params"]["thr"])
    thr = enc if np.isinf(thr) else thr
    r = ops.dim0(ctx(), mat=mat, threshold=thr, maxdim=2)
    piv = dev(c["piv"].view(np.int64))
    ci, cd, napp = ops.assemble(ctx(), mat, thr, r["keys"], piv)
    assert np.array_equal(host(ci).view(np.uint64), c["c2idx"])
    assert np.array_equal(bits(host(cd)), bits(c["c2d"]))
    assert napp == int(c["app2n"][0])


@pytest.mark.parametrize("c", BARS, ids=ids(BARS))
def test_persistence_vs_reference(c):
    dgms, info = tg.persistence(c["x"], maxdim=c["params"]["maxdim"], metric=c["metric"])
    got = tg.canonical(dgms)
    ref = canonical(c["bars"])
    assert got.shape == ref.shape
    assert np.array_equal(bits(got), bits(ref))


@pytest.mark.parametrize("name,metric", [("lattice3000_linf", "linf"), ("lattice3000_l1", "l1")])
def test_lattice_config_front_end_checksums(name, metric):
    """Full-size tie-heavy configuration: every front-end output of the
    reference (sorted edges, apparent flags, columns, H0, dim-2 columns built
    from the reference's pivots) reproduced bit for bit (checksums)."""
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))[name]
    x = synth.lattice()
    mat, enc = ops.make_dense(ctx(), dev(x), metric)
    assert np.float32(enc) == np.float32(cfg["thr"])
    r = ops.dim0(ctx(), mat=mat, threshold=enc, maxdim=2)
    idx, d = decode_keys(r["keys"])
    assert idx.size == cfg["edges"] and sha(idx, d) == cfg["edges_sha"]
    assert sha(host(r["app"])) == cfg["app_sha"]
    assert sha(host(r["cidx"]).view(np.uint64), host(r["cd"])) == cfg["cols_sha"]
    piv = np.load(os.path.join(GOLDEN, f"cfg_{name}_piv.npz"))["piv"]
    ci, cd, napp = ops.assemble(ctx(), mat, enc, r["keys"], dev(piv.view(np.int64)))
    assert ci.numel() == cfg["c2"] and napp == cfg["app2"]
    assert sha(host(ci).view(np.uint64), host(cd)) == cfg["c2_sha"]


def test_torus_config_front_end_checksums():
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))["torus1000_l2"]
    x = synth.torus()
    mat, enc = ops.make_dense(ctx(), dev(x), "l2")
    assert np.float32(enc) == np.float32(cfg["thr"])
    r = ops.dim0(ctx(), mat=mat, threshold=enc, maxdim=2)
    idx, d = decode_keys(r["keys"])
    assert sha(idx, d) == cfg["edges_sha"] and sha(host(r["app"])) == cfg["app_sha"]
    assert sha(host(r["cidx"]).view(np.uint64), host(r["cd"])) == cfg["cols_sha"]
    piv = np.load(os.path.join(GOLDEN, "cfg_torus1000_piv.npz"))["piv"]
    ci, cd, napp = ops.assemble(ctx(), mat, enc, r["keys"], dev(piv.view(np.int64)))
    assert sha(host(ci).view(np.uint64), host(cd)) == cfg["c2_sha"] and napp == cfg["app2"]


@pytest.mark.parametrize("metric,maxdim,graph,thr", [("l2", 1, "full", "inf"), ("l1", 2, "full", "inf"),
                                                    ("l2", 1, "full", "0.3"), ("l2", 1, "knn", "inf"),
                                                    ("linf", 0, "full", "inf"), ("l2", 0, "full", "0.2")])
def test_persistence_paths_vs_oracle_h0_and_counts(metric, maxdim, graph, thr):
    """Every dispatch path runs; H0 agrees with the oracle's dim0 / MST."""
    x = synth.uniform(400, 3, 77)
    t = thr_of(thr)
    dgms, info = tg.persistence(x, maxdim=maxdim, metric=metric, graph=graph, threshold=t, k=8)
    assert len(dgms) == maxdim + 1
    if maxdim == 0 and graph == "full":
        ref = O.mst_h0(x, metric, t)
    elif graph == "full" and np.isinf(t):
        m = O.dense(x, metric)
        ref = O.dim0(mat=m, thr=O.enclosing_radius(m), maxdim=maxdim)["h0"]
    elif graph == "full":
        ref = O.dim0(csr=O.radius_graph(x, metric, t), n=400, thr=t, maxdim=maxdim)["h0"]
    else:
        ids_ = O.knn(x, metric, 8)
        ref = O.dim0(csr=O.knn_graph(x, metric, ids_), n=400, maxdim=maxdim)["h0"]
    assert np.array_equal(bits(dgms[0].ravel()), bits(ref))


def test_persistence_validation_messages():
    x = synth.uniform(10, 2, 1)
    with pytest.raises(ValueError, match="threshold must be non-negative"):
        tg.persistence(x, threshold=-1.0)
    with pytest.raises(ValueError, match="k must be >= 1"):
        tg.persistence(x, graph="knn", k=0)
    with pytest.raises(ValueError, match="non-finite coordinate"):
        y = x.copy()
        y[3, 1] = np.nan
        tg.persistence(y)
    with pytest.raises(ValueError, match="unknown 'cosine'"):
        tg.persistence(x, metric="cosine")
    # make_dense's memory budget: 10 points need 180 bytes of lower triangle
    with pytest.raises(ValueError, match="rips: the dense distance matrix exceeds the memory budget"):
        tg.persistence(x, memory_budget=179)
    a, _ = tg.persistence(x, memory_budget=180)
    b, _ = tg.persistence(x)
    assert all(np.array_equal(u, v) for u, v in zip(a, b))
    c, _ = tg.persistence(x, maxdim=0, memory_budget=1)       # the MST path takes no matrix
    assert np.array_equal(np.sort(c[0][:, 1]), np.sort(b[0][:, 1]))


def test_graph_input_equals_point_knn_path():
    """persistence(CsrGraph) on the kNN graph of a cloud is the same flag
    complex as persistence(points, graph='knn'): identical diagrams."""
    import numpy as np
    from turbotops_gb300 import api, ops, synth
    from gpu_util import ctx, dev, host
    x = synth.gauss(700, 6, 31)
    d1, i1 = api.persistence(x, maxdim=1, graph="knn", k=8)
    rp, ci, w = ops.knn_graph(ctx(), dev(x), 8, "l2")
    d2, i2 = api.persistence_graph(host(rp).view(np.uint64), host(ci).view(np.uint32), host(w), 700, maxdim=1)
    assert np.array_equal(api.canonical(d1), api.canonical(d2))
    assert i2["method"] == "sparse" and i2["edges"] == i1["edges"]
    # a finite threshold keeps edges <= threshold
    t = float(np.median(host(w)))
    d3, _ = api.persistence_graph(host(rp).view(np.uint64), host(ci).view(np.uint32), host(w), 700, maxdim=1,
                                  threshold=t)
    assert all((b[:, 1][np.isfinite(b[:, 1])] <= t).all() for b in d3)


def test_scipy_sparse_input_and_csr_validation():
    import numpy as np
    scipy_sparse = pytest.importorskip("scipy.sparse")
    from turbotops_gb300 import api
    # a one-directional, duplicated edge list: symmetrised, smallest weight kept
    i = np.array([0, 1, 2, 3, 0, 1])
    j = np.array([1, 2, 3, 0, 2, 0])
    w = np.array([1, 1, 1, 1, 1.5, 0.5], np.float32)
    g = scipy_sparse.coo_matrix((w, (i, j)), shape=(4, 4))
    dg, info = api.persistence(g, maxdim=1)
    rp, ci, ww = api.symmetric_rows(i, j, w, 4)
    dg2, _ = api.persistence_graph(rp, ci, ww, 4, maxdim=1)
    assert np.array_equal(api.canonical(dg), api.canonical(dg2))
    assert sorted(dg[0][:, 1].tolist()) == [0.5, 1.0, 1.0, np.inf]
    with pytest.raises(ValueError, match="weights must be finite and >= 0"):
        api.persistence(scipy_sparse.coo_matrix((np.array([-1.0], np.float32), ([0], [1])), shape=(2, 2)))
    # CsrGraph::valid(): asymmetric weights, unsorted rows, self loops
    bad = [
        (np.array([0, 1, 2], np.uint64), np.array([1, 0], np.uint32), np.array([1, 2], np.float32)),
        (np.array([0, 2, 3, 4], np.uint64), np.array([2, 1, 0, 0], np.uint32), np.array([1, 1, 1, 1], np.float32)),
        (np.array([0, 1, 1], np.uint64), np.array([0], np.uint32), np.array([1], np.float32)),
    ]
    for rp, ci, ww in bad:
        with pytest.raises(ValueError, match="CsrGraph invariant violated"):
            api.persistence_graph(rp, ci, ww, len(rp) - 1, maxdim=1)
    with pytest.raises(ValueError, match="threshold must be non-negative"):
        api.persistence_graph(rp, ci, ww, 4, maxdim=1, threshold=-1.0)


HBARS = cases("hbars")


@pytest.mark.parametrize("c", HBARS, ids=ids(HBARS))
def test_graph_input_higher_dims_vs_reference(c):
    """kNN- and radius-graph flag complexes up to maxdim 3 through the public
    API (GPU graph and dim0, host reduction and assemble): the reference
    CLI's exact text."""
    args, maxdim = c["params"]["args"], c["params"]["maxdim"]
    kw = {"graph": "knn", "k": int(args[3])} if args[0] == "--graph" else {"threshold": float(np.float32(args[1]))}
    dgms, info = tg.persistence(c["x"], maxdim=maxdim, metric=c["metric"], **kw)
    from turbotops_gb300 import api
    assert api.format_diagram(dgms) == str(c["text"])
