"""The host-buffer entry points (the calls the reference's front ends bind,
and the e2e leg of the bench) against the device-resident path, and their
argument checks: a non-finite coordinate is the reference's invalid-argument
error, raised before any output is written."""
import ctypes as C
import math

import numpy as np
import pytest

from gpu_util import ctx, dev, host
from turbotops_gb300 import capi, ops, synth

pytestmark = pytest.mark.gpu

P = C.c_void_p


def _ptr(a):
    return P(a.ctypes.data) if a is not None else None


def _front_h(x, k, maxdim=1, pinned=False):
    c = ctx()
    n, dim = x.shape
    kind, p = capi.metric_parse("l2")
    cap = 2 * n * k + 16
    if pinned:
        import torch
        keep = [torch.zeros((n + 1) * 8 + cap * 8, dtype=torch.uint8).pin_memory()]
        buf = keep[0].numpy()
        rp = buf[:(n + 1) * 8].view(np.uint64)
        col = buf[(n + 1) * 8:(n + 1) * 8 + cap * 4].view(np.uint32)
        w = buf[(n + 1) * 8 + cap * 4:].view(np.float32)
    else:
        rp = np.zeros(n + 1, np.uint64)
        col = np.zeros(cap, np.uint32)
        w = np.zeros(cap, np.float32)
    h0 = np.zeros(max(n, 1), np.float32)
    cidx = np.zeros(cap, np.uint64)
    cd = np.zeros(cap, np.float32)
    cf = np.zeros(cap, np.uint64)
    ca = np.zeros(cap, np.uint8)
    nnz, nh0, ess, ncols, nedges = (C.c_uint64() for _ in range(5))
    st = c.L.tt_knn_front_h(c.h, _ptr(x), n, dim, kind, p, k, maxdim, _ptr(rp), _ptr(col), _ptr(w), cap,
                            C.byref(nnz), _ptr(h0), C.byref(nh0), C.byref(ess), _ptr(cidx), _ptr(cd), _ptr(cf),
                            _ptr(ca), cap, C.byref(ncols), C.byref(nedges))
    return st, dict(rp=rp.copy(), col=col[:nnz.value].copy(), w=w[:nnz.value].copy(), h0=h0[:nh0.value],
                    essential=ess.value, cidx=cidx[:ncols.value], cd=cd[:ncols.value], cf=cf[:ncols.value],
                    ca=ca[:ncols.value], edges=nedges.value)


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("kind,n,k", [("gmm", 3000, 15), ("gauss", 800, 7)])
def test_knn_front_h_equals_device_path(kind, n, k, pinned):
    x = synth.gmm(n, 32, seed=n) if kind == "gmm" else synth.gauss(n, 5, n)
    x = np.ascontiguousarray(x, np.float32)
    st, r = _front_h(x, k, pinned=pinned)
    assert st == capi.OK
    rp, ci, w = ops.knn_graph(ctx(), dev(x), k, "l2")
    assert np.array_equal(r["rp"], host(rp).view(np.uint64))
    assert np.array_equal(r["col"], host(ci).view(np.uint32))
    assert np.array_equal(r["w"].view(np.uint32), host(w).view(np.uint32))
    d = ops.dim0(ctx(), csr=(rp, ci, w), n=n)
    assert r["edges"] == d["keys"].numel()
    assert np.array_equal(r["h0"].view(np.uint32), host(d["h0"]).view(np.uint32))
    assert r["essential"] == d["essential"]
    assert np.array_equal(r["cidx"], host(d["cidx"]).view(np.uint64))
    assert np.array_equal(r["cd"].view(np.uint32), host(d["cd"]).view(np.uint32))
    assert np.array_equal(r["cf"], host(d["emi"]).view(np.uint64))
    assert np.array_equal(r["ca"], host(d["emf"]).view(np.uint8))


@pytest.mark.parametrize("bad", [math.nan, math.inf, -math.inf])
def test_host_entries_reject_non_finite(bad):
    x = np.ascontiguousarray(synth.gauss(500, 6, 1), np.float32)
    x[123, 4] = bad
    c = ctx()
    st, _ = _front_h(x, 5)
    assert st == capi.ERR_INVALID
    assert "non-finite coordinate" in c.L.tt_last_error(c.h).decode()
    n, dim = x.shape
    kind, p = capi.metric_parse("l2")
    rp = np.zeros(n + 1, np.uint64)
    col = np.zeros(10 * n, np.uint32)
    w = np.zeros(10 * n, np.float32)
    nnz = C.c_uint64()
    st = c.L.tt_knn_graph_h(c.h, _ptr(x), n, dim, kind, p, 5, _ptr(rp), _ptr(col), _ptr(w), 10 * n, C.byref(nnz))
    assert st == capi.ERR_INVALID
    thr = C.c_float(math.inf)
    mat = np.zeros((n, n), np.float32)
    nh0, ess, ncols, nedges = (C.c_uint64() for _ in range(4))
    st = c.L.tt_dense_front_h(c.h, _ptr(x), n, dim, kind, p, 1, C.byref(thr), _ptr(mat), None, C.byref(nh0),
                              C.byref(ess), None, None, None, None, 0, C.byref(ncols), C.byref(nedges))
    assert st == capi.ERR_INVALID
    # the context stays usable
    st, r = _front_h(np.ascontiguousarray(synth.gauss(300, 6, 2), np.float32), 5)
    assert st == capi.OK and r["rp"][-1] > 0


@pytest.mark.parametrize("bad", [math.nan, math.inf])
def test_knn_front_h_non_finite_on_the_tensor_core_path(bad):
    """The kNN front end with host buffers checks the points while the
    tensor-core kNN already runs (L2 in R^32, 3,000 points): the same error,
    raised before the graph is built, and the next call is exact again."""
    from oracle import oracle as O
    x = np.ascontiguousarray(synth.gmm(3000, 32, 8, 4), np.float32)
    bad_x = x.copy()
    bad_x[2999, 31] = bad
    c = ctx()
    st, _ = _front_h(bad_x, 15)
    assert st == capi.ERR_INVALID
    assert "non-finite coordinate" in c.L.tt_last_error(c.h).decode()
    st, r = _front_h(x, 15)
    assert st == capi.OK
    orp, oci, ow = O.knn_graph(x, "l2", O.knn(x, "l2", 15))
    assert np.array_equal(r["rp"], np.asarray(orp, np.uint64))
    assert np.array_equal(r["col"], np.asarray(oci, np.uint32))
    assert np.array_equal(r["w"].view(np.uint32), np.asarray(ow, np.float32).view(np.uint32))


def test_knn_front_h_above_packed_key_range_vs_oracle():
    """140,000 points: edge indices beyond the packed keys' 33 bits, so dim0
    runs on the wide key layout with the kept-edge count announced by the
    front end. H0, columns and emergent probes equal the oracle's dim0 on the
    same graph."""
    from oracle import oracle as O
    n, k = 140000, 8
    x = np.ascontiguousarray(synth.gauss(n, 3, 77), np.float32)
    st, r = _front_h(x, k)
    assert st == capi.OK
    csr = (r["rp"], r["col"], r["w"])
    o = O.dim0(csr=csr, n=n, maxdim=1)
    assert r["edges"] == o["eidx"].size
    assert np.array_equal(r["cidx"], o["cidx"])
    assert np.array_equal(r["cd"].view(np.uint32), o["cd"].view(np.uint32))
    od = o["h0"].reshape(-1, 2)[:, 1]
    od = np.sort(od[np.isfinite(od) & (od > 0)])
    assert np.array_equal(np.sort(r["h0"]).view(np.uint32), od.view(np.uint32))
    e = O.emergent(csr=csr, n=n, cidx=o["cidx"], cd=o["cd"])
    assert np.array_equal(r["cf"], e["emi"])
    assert np.array_equal(r["ca"], e["emf"])


@pytest.mark.parametrize("n,bad", [(3000, math.nan), (6000, math.inf)])
def test_device_entries_reject_non_finite(n, bad):
    """The device-pointer entry points that index by kNN list entries check
    the points on the device, read before the first such kernel: a
    non-finite coordinate is the reference's invalid-argument error (never a
    short list read past its end), and the context keeps working."""
    x = np.ascontiguousarray(synth.gmm(n, 32, 6, n), np.float32)
    bad_x = x.copy()
    bad_x[n // 2, 7] = bad
    c = ctx()
    kind, p = capi.metric_parse("l2")
    for run in (lambda: ops.knn_graph(c, dev(bad_x), 15, "l2"), lambda: ops.mst_deaths(c, dev(bad_x), "l2")):
        with pytest.raises(ValueError, match="non-finite coordinate"):
            run()
    xd = dev(bad_x)
    out = capi.KnnFrontOut()
    assert c.L.tt_knn_front(c.h, xd.data_ptr(), n, 32, kind, p, 15, 1, C.byref(out)) == capi.ERR_INVALID
    assert "non-finite coordinate" in c.L.tt_last_error(c.h).decode()
    d = ops.mst_deaths(c, dev(x), "l2")
    assert np.array_equal(host(d).view(np.uint32), np.sort(host(d)).view(np.uint32))
    rp, ci, w = ops.knn_graph(c, dev(x), 15, "l2")
    assert host(rp).view(np.uint64)[-1] == ci.numel()
