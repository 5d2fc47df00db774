"""CUDA path vs the reference (golden fixtures) and the oracle: dense matrices,
enclosing radius, dim0 (sorted edges, apparent pairs, H0, columns, emergent
probe) and RedZeD edge lists. Integer/index outputs and L1/L2/L-inf
distances are compared bit for bit."""
import numpy as np
import pytest
import torch

from golden_io import cases, ids, thr_of
from gpu_util import bits, ctx, decode_keys, dev, h0_pairs, host
from oracle import oracle as O
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu

DENSE = cases("dense")
ASM = cases("asm")
RZD = cases("rzd")
RZS = cases("rzs")
SDIM0 = cases("sdim0")
EXACT = {"l1", "l2", "linf"}


@pytest.mark.parametrize("c", DENSE, ids=ids(DENSE))
def test_dense_vs_reference(c):
    x = dev(c["x"])
    mat, enc = ops.make_dense(ctx(), x, c["metric"])
    m = host(mat).ravel()
    # every metric bit for bit, non-integer p included (the *_a64 fixtures:
    # the reference built on this machine's aarch64 host)
    assert np.array_equal(bits(m), bits(c["mat"]))
    assert bits(np.float32(enc)) == bits(c["encl"])[0]


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5", "lp:2.5", "lp:3"])
@pytest.mark.parametrize("shape", [(1, 3), (2, 5), (33, 16), (130, 32), (257, 48), (97, 70)])
def test_dense_vs_oracle(metric, shape):
    x = synth.gauss(*shape, seed=shape[0] * 7 + shape[1])
    mat, enc = ops.make_dense(ctx(), dev(x), metric)
    ref = O.dense(x, metric)
    assert np.array_equal(bits(host(mat)), bits(ref))
    assert bits(np.float32(enc)) == bits(O.enclosing_radius(ref))


def _check_dim0(r, ref, app=True):
    idx, d = decode_keys(r["keys"])
    assert np.array_equal(idx, ref["eidx"])
    assert np.array_equal(bits(d), bits(ref["ed"]))
    if app:
        assert np.array_equal(host(r["app"]), ref["app"])
    assert np.array_equal(host(r["cidx"]).view(np.uint64), ref["cidx"])
    assert np.array_equal(bits(host(r["cd"])), bits(ref["cd"]))
    assert np.array_equal(bits(h0_pairs(r)), bits(ref["h0"]))


def _check_emergent(r, ref):
    emi = host(r["emi"]).view(np.uint64)
    assert np.array_equal(emi, ref["emi"])
    assert np.array_equal(host(r["emf"]), ref["emf"])


@pytest.mark.parametrize("c", ASM, ids=ids(ASM))
def test_dim0_dense_vs_reference(c):
    mat, enc = ops.make_dense(ctx(), dev(c["x"]), c["metric"])
    thr = thr_of(c["params"]["thr"])
    thr = enc if np.isinf(thr) else thr
    assert bits(np.float32(thr)) == bits(c["thr"])[0]
    r = ops.dim0(ctx(), mat=mat, threshold=thr, maxdim=2)
    _check_dim0(r, c)
    _check_emergent(r, c)


@pytest.mark.parametrize("c", SDIM0, ids=ids(SDIM0))
def test_dim0_sparse_vs_reference(c):
    csr = (dev(c["g_rp"]).view(torch.int64), dev(c["g_ci"].view(np.int32)), dev(c["g_w"]))
    r = ops.dim0(ctx(), csr=csr, n=c["x"].shape[0], maxdim=2)
    _check_dim0(r, c)
    _check_emergent(r, c)


@pytest.mark.parametrize("c", RZD, ids=ids(RZD))
def test_redzed_dense_vs_reference(c):
    mat, enc = ops.make_dense(ctx(), dev(c["x"]), c["metric"])
    d, v = ops.redzed_edges(ctx(), mat=mat, threshold=float(c["thr"][0]))
    assert np.array_equal(bits(host(d)), bits(c["rd"]))
    assert np.array_equal(host(v), c["rv"])


@pytest.mark.parametrize("c", RZS, ids=ids(RZS))
def test_redzed_sparse_vs_reference(c):
    csr = (dev(c["knn_rp"]).view(torch.int64), dev(c["knn_ci"].view(np.int32)), dev(c["knn_w"]))
    d, v = ops.redzed_edges(ctx(), csr=csr, n=c["x"].shape[0])
    assert np.array_equal(bits(host(d)), bits(c["rd"]))
    assert np.array_equal(host(v), c["rv"])


@pytest.mark.parametrize("metric,n,seed,thr", [("l1", 900, 21, "inf"), ("linf", 700, 22, "inf"),
                                              ("l2", 1200, 23, "inf"), ("l2", 1000, 24, "0.4")])
def test_dim0_vs_oracle_larger(metric, n, seed, thr):
    # integer-lattice points: maximal ties in the filtration sort and in the
    # apparent-pair tests
    x = synth.grid(n, 4, 9, seed) if metric != "l2" else synth.uniform(n, 3, seed)
    mat, enc = ops.make_dense(ctx(), dev(x), metric)
    t = enc if thr == "inf" else float(np.float32(thr))
    r = ops.dim0(ctx(), mat=mat, threshold=t, maxdim=1)
    ref = O.dim0(mat=host(mat), thr=t, maxdim=1)
    _check_dim0(r, ref)
    e = O.emergent(mat=host(mat), cidx=ref["cidx"], cd=ref["cd"])
    _check_emergent(r, e)


def test_dim0_h0_only_and_empty():
    x = synth.uniform(50, 3, 5)
    mat, enc = ops.make_dense(ctx(), dev(x), "l2")
    r = ops.dim0(ctx(), mat=mat, threshold=0.0, maxdim=0)   # no kept edges
    assert r["keys"].numel() == 0 and r["essential"] == 50
    r = ops.dim0(ctx(), mat=mat, threshold=enc, maxdim=0)
    ref = O.dim0(mat=host(mat), thr=enc, maxdim=0)
    assert np.array_equal(bits(h0_pairs(r)), bits(ref["h0"]))
    one, _ = ops.make_dense(ctx(), dev(x[:1]), "l2")
    r = ops.dim0(ctx(), mat=one, threshold=0.0, maxdim=1)
    assert r["essential"] == 1 and r["keys"].numel() == 0
