"""Front-end outputs of the full-size kNN workload (100,000 points in R^32,
16-Gaussian mixture, seed 3, k = 15) against checksums of the reference's own
outputs on the same points: the symmetric kNN graph (CSR: row pointers,
columns, recomputed weights) and the RedZeD edge list of its flag complex
under L2 (tests/golden/configs.json), and the lists and graph under lp:1.5
(tests/golden/configs_a64.json: the reference built on this machine's aarch64
host, whose reciprocal estimate and libm decide non-integer Lp bits)."""
import hashlib
import json
import os

import numpy as np
import pytest

from gpu_util import ctx, dev, host
from turbotops_gb300 import ops, synth

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def sha(*arrs):
    h = hashlib.sha256()
    for a in arrs:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


@pytest.fixture(scope="module")
def gmm():
    return dev(synth.gmm())


def test_knn_graph_and_redzed_edges_l2(gmm):
    cfg = json.load(open(os.path.join(GOLDEN, "configs.json")))["gmm100k_l2_k15"]
    rp, ci, w = ops.knn_graph(ctx(), gmm, 15, "l2")
    assert ci.numel() == cfg["nnz"]
    assert sha(host(rp).view(np.uint64), host(ci).view(np.uint32), host(w)) == cfg["csr_sha"]
    d, v = ops.redzed_edges(ctx(), csr=(rp, ci, w), n=gmm.shape[0])
    assert sha(host(d), host(v)) == cfg["rz_sha"]


def test_knn_lists_and_graph_lp15(gmm):
    cfg = json.load(open(os.path.join(GOLDEN, "configs_a64.json")))["gmm100k_lp1.5_k15"]
    i, _ = ops.knn(ctx(), gmm, 15, "lp:1.5")
    assert sha(host(i).view(np.uint32)) == cfg["ids_sha"]
    rp, ci, w = ops.knn_graph(ctx(), gmm, 15, "lp:1.5")
    assert ci.numel() == cfg["nnz"]
    assert sha(host(rp).view(np.uint64), host(ci).view(np.uint32), host(w)) == cfg["csr_sha"]
