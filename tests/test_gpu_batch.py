"""Batched dense front end (one captured CUDA graph for many clouds) vs the
per-cloud path: every cloud's enclosing radius and RedZeD edge list must be
bit-identical to the single-cloud entry points (themselves pinned to the
reference), on the first run and on graph replays."""
import numpy as np
import pytest
import torch

from gpu_util import bits, ctx, dev, host
from oracle import oracle as O
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu


def _clouds(count, lo, hi, seed):
    return synth.circle_batch(count, lo, hi, seed)


@pytest.mark.parametrize("use_graph", [True, False])
@pytest.mark.parametrize("metric", ["l2", "l1"])
def test_batch_matches_per_cloud(use_graph, metric):
    clouds = _clouds(14, 2, 400, 21) + [synth.uniform(1, 3, 5), synth.uniform(2, 3, 6)]
    sizes = [c.shape[0] for c in clouds]
    b = ops.DenseBatch(ctx(), sizes, 3, metric, use_graph=use_graph)
    b.load(dev(np.concatenate(clouds)))
    for rep in range(2):   # first run captures the graph, the second replays it
        b.run()
        r = b.result()
        off = host(r["edge_offset"])
        rad = host(r["radius"])
        d_all, v_all = host(r["diam"]), host(r["verts"])
        for q, x in enumerate(clouds):
            mat, enc = ops.make_dense(ctx(), dev(x), metric)
            assert bits(rad[q]) == bits(np.float32(enc)), q
            d, v = ops.redzed_edges(ctx(), mat=mat, threshold=enc)
            s, e = int(off[q]), int(off[q + 1])
            assert np.array_equal(bits(d_all[s:e]), bits(host(d))), q
            assert np.array_equal(v_all[2 * s:2 * e], host(v)), q
    b.close()


def test_batch_vs_oracle():
    clouds = _clouds(6, 50, 300, 33)
    b = ops.DenseBatch(ctx(), [c.shape[0] for c in clouds], 3, "l2")
    b.load(dev(np.concatenate(clouds)))
    b.run()
    r = b.result()
    off = host(r["edge_offset"])
    for q, x in enumerate(clouds):
        m = O.dense(x, "l2")
        d, v = O.redzed_edges(mat=m, thr=O.enclosing_radius(m))
        s, e = int(off[q]), int(off[q + 1])
        assert np.array_equal(bits(host(r["diam"])[s:e]), bits(d))
        assert np.array_equal(host(r["verts"])[2 * s:2 * e], v)
    b.close()


def test_large_batch_matches_per_cloud():
    """A batch whose sort exceeds 4M keys (the radix sort then orders every
    tile by digit in shared memory and writes runs): still the per-cloud
    edge lists, bit for bit."""
    clouds = _clouds(5, 1700, 2000, 41)
    sizes = [c.shape[0] for c in clouds]
    assert sum(s * (s - 1) // 2 for s in sizes) >= 1 << 22
    b = ops.DenseBatch(ctx(), sizes, 3, "l2", use_graph=True)
    b.load(dev(np.concatenate(clouds)))
    for _ in range(2):
        b.run()
        r = b.result()
        off = host(r["edge_offset"])
        d_all, v_all = host(r["diam"]), host(r["verts"])
        for q, x in enumerate(clouds):
            mat, enc = ops.make_dense(ctx(), dev(x), "l2")
            d, v = ops.redzed_edges(ctx(), mat=mat, threshold=enc)
            s, e = int(off[q]), int(off[q + 1])
            assert np.array_equal(bits(d_all[s:e]), bits(host(d))), q
            assert np.array_equal(v_all[2 * s:2 * e], host(v)), q
    b.close()
