"""tcgen05 Gram-filtered exact kNN (L2, R^32) vs the exhaustive scan and the
reference: the lists and distances must be identical (the filter only
decides which candidates get the exact lane-ordered distance); the filter
must also be selective (a broken Gram product would let almost every
candidate through, or drop true neighbours)."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest
import torch

from golden_io import GOLDEN, cases, ids
from gpu_util import ctx, dev, host
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu

KNN32 = [c for c in cases("knn") if c["x"].shape[1] == 32 and c["metric"] == "l2"]


def _knn(x, k, mode):
    c = ctx()
    c.check(c.L.tt_ctx_set_knn_mode(c.h, mode))
    try:
        i, d = ops.knn(c, dev(x), k, "l2")
        torch.cuda.synchronize()
        return host(i).view(np.uint32), host(d), int(c.L.tt_ctx_filter_evals(c.h))
    finally:
        c.check(c.L.tt_ctx_set_knn_mode(c.h, 0))


@pytest.mark.parametrize("n,k,kind", [(300, 15, "gmm"), (2000, 15, "gmm"), (777, 5, "gauss"), (1500, 1, "uniform"),
                                      (4096, 16, "gmm"), (20000, 15, "gmm")])
def test_tensor_filter_equals_exhaustive_scan(n, k, kind):
    x = {"gmm": lambda: synth.gmm(n, 32, seed=n),
         "gauss": lambda: synth.gauss(n, 32, n),
         "uniform": lambda: synth.uniform(n, 32, n)}[kind]()
    i1, d1, _ = _knn(x, k, 1)
    i2, d2, evals = _knn(x, k, 2)
    assert np.array_equal(i1, i2)
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
    if n >= 20000:
        assert evals < 0.02 * n * n, evals   # the Gram filter must prune


@pytest.mark.parametrize("c", KNN32, ids=ids(KNN32))
def test_tensor_filter_vs_reference(c):
    i2, _, _ = _knn(c["x"], c["params"]["k"], 2)
    assert np.array_equal(i2.ravel(), c["ids"])


def test_tensor_filter_full_config_checksum():
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))["gmm100k_l2_k15"]
    i2, _, evals = _knn(synth.gmm(), 15, 0)   # automatic selection: the tensor path
    assert hashlib.sha256(np.ascontiguousarray(i2).tobytes()).hexdigest()[:16] == cfg["ids_sha"]
    assert evals > 0


def _cases_tile_order():
    rng = np.random.default_rng(7)
    g = synth.gmm(30001, 32, seed=11)
    out = {
        # ragged last tile, shuffled rows (the regrouping must undo any input order)
        "gmm_ragged_shuffled": (g[rng.permutation(len(g))], 15),
        # every point repeated: k-th distances are 0 and ties are broken by id
        "duplicates": (np.repeat(synth.gauss(1500, 32, 3), 20, axis=0), 15),
        # integer lattice: massive distance ties across tiles
        "lattice": (rng.integers(0, 3, (6000, 32)).astype(np.float32), 12),
        # large common offset: the Gram-form margins dominate
        "offset": (synth.gmm(8000, 32, seed=5) + np.float32(1000.0), 15),
        # tiny coordinates: subnormal squares
        "tiny": (synth.gauss(5000, 32, 9) * np.float32(1e-21), 7),
        # well separated clusters, k = 1
        "far_clusters": (synth.gmm(12000, 32, centres=4, seed=2) * np.float32(50.0), 1),
        # point scales from 1e-3 to 1e3 side by side: the per-tile TF32 error
        # terms differ by six orders of magnitude
        "wide_range": (synth.gauss(9000, 32, 4) * (10.0 ** rng.uniform(-3, 3, (9000, 1))).astype(np.float32), 9),
        # clusters of near-duplicates (spread 1e-4 around points far from the
        # origin): the neighbours sit inside the filter's rounding band
        "near_duplicates": (np.repeat(synth.gauss(400, 32, 6) * np.float32(30.0), 25, axis=0)
                            + rng.normal(0, 1e-4, (10000, 32)).astype(np.float32), 15),
    }
    return out


TILE_CASES = _cases_tile_order()


@pytest.mark.parametrize("name", sorted(TILE_CASES))
def test_tile_order_equals_exhaustive_scan(name):
    x, k = TILE_CASES[name]
    x = np.ascontiguousarray(x, dtype=np.float32)
    i1, d1, _ = _knn(x, k, 1)
    i2, d2, _ = _knn(x, k, 2)
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
    assert np.array_equal(i1, i2)


def test_tile_order_prunes_and_matches_at_scale():
    """400,003 points: the pivot count reaches its cap and the last tile is
    ragged; the lists equal the exhaustive scan's and most Gram tiles are
    never computed."""
    x = synth.gmm(400003, 32, seed=21)
    i1, d1, _ = _knn(x, 10, 1)
    c = ctx()
    i2, d2, _ = _knn(x, 10, 2)
    tiles = int(c.L.tt_ctx_filter_tiles(c.h))
    nt = (len(x) + 127) // 128
    assert np.array_equal(i1, i2)
    assert np.array_equal(d1.view(np.uint32), d2.view(np.uint32))
    assert 0 < tiles < 0.5 * nt * nt, (tiles, nt * nt)


def test_tensor_core_accumulation_bound():
    """The Gram filter's margins are derived for an FP32 accumulation error of
    at most 2^-17 (|a|^2 + |b|^2) in kind::tf32 on TF32-exact operands (the
    bound that 24-bit alignment and truncation in each accumulation step
    implies). Measured on 304 seeded 128 x 128 products, issued as the kNN
    kernel issues them: mixed exponents and signs, and rows near a common
    offset where the sum cancels; asserted 4x tighter than needed."""
    c = ctx()
    r = C.c_double()
    c.check(c.L.tt_tc_gram_check(c.h, 304, 12345, C.byref(r)))
    assert 0.0 <= r.value < 2.0 ** -19, r.value
