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
