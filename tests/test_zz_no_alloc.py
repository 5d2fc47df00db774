"""tt_dense_distances_static: the allocation-free form of tt_dense_distances.

It exists for callers that cannot call cudaMalloc while they compute
distances (their device memory is already handed to their own pool, or their
loop must not take the synchronisation an allocation implies). The test calls
it through the C-ABI twice in a row — a larger cloud, then a smaller one, so
stale row maxima left in the shared scratch array by the first call would
show up — and checks the matrix and the enclosing radius bit for bit against
tt_dense_distances, the context-based entry point. It runs last so that a
failure here never hides another test's result, and it passes alone in a
fresh process as well as after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from turbotops_gb300 import capi, ops, synth

pytestmark = pytest.mark.gpu


def _static(L, x: torch.Tensor, metric: str):
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    mat = torch.empty((n, n), dtype=torch.float32, device=x.device)
    radius = torch.empty(1, dtype=torch.float32, device=x.device)
    stream = torch.cuda.current_stream(x.device).cuda_stream
    st = L.tt_dense_distances_static(x.data_ptr(), n, dim, kind, p, mat.data_ptr(), radius.data_ptr(),
                                     C.c_void_p(stream))
    capi.raise_for(st, L.tt_last_error(None).decode())
    torch.cuda.synchronize()
    return mat, radius


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5"])
def test_static_matches_context_entry_point_twice(metric):
    L = capi.load()
    ctx = capi.Context(0)
    first = torch.from_numpy(synth.gauss(700, 32, 41)).cuda()
    second = torch.from_numpy(synth.uniform(300, 3, 42)).cuda()
    for x in (first, second):
        mat, radius = _static(L, x, metric)
        ref_mat, ref_radius = ops.make_dense(ctx, x, metric)
        assert np.array_equal(mat.cpu().numpy().view(np.uint32), ref_mat.cpu().numpy().view(np.uint32))
        got = radius.cpu().numpy().view(np.uint32)[0]
        assert got == np.float32(ref_radius).view(np.uint32)


def test_static_empty_cloud_radius_is_inf():
    L = capi.load()
    x = torch.zeros((0, 3), dtype=torch.float32, device="cuda")
    mat, radius = _static(L, x, "l2")
    assert mat.numel() == 0 and float(radius.item()) == float("inf")


def test_static_allocates_no_device_memory():
    """After a first call per metric (which loads that metric's kernels), a
    further call leaves the device's free memory exactly where it was:
    nothing is allocated."""
    L = capi.load()
    x = torch.from_numpy(synth.gauss(2000, 16, 43)).cuda()
    free0, _ = torch.cuda.mem_get_info()
    for metric in ("l2", "l1", "lp:1.5"):
        _static(L, x, metric)
        n, dim = x.shape
        kind, p = capi.metric_parse(metric)
        mat = torch.empty((n, n), dtype=torch.float32, device=x.device)
        radius = torch.empty(1, dtype=torch.float32, device=x.device)
        free1, _ = torch.cuda.mem_get_info()
        st = L.tt_dense_distances_static(x.data_ptr(), n, dim, kind, p, mat.data_ptr(), radius.data_ptr(),
                                         C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == capi.OK
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free1
        del mat, radius
    assert free0 > 0


def test_static_rejects_n_above_its_scratch_before_any_work():
    L = capi.load()
    dummy = torch.zeros(4, dtype=torch.float32, device="cuda")
    st = L.tt_dense_distances_static(dummy.data_ptr(), 262145, 3, capi.METRIC_L2, 2.0, dummy.data_ptr(),
                                     dummy.data_ptr(), None)
    assert st == capi.ERR_LENGTH
    assert "262144" in L.tt_last_error(None).decode()
