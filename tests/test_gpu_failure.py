"""Failure detection without a GPU fault: a bounded device wait that nobody
completes runs out, the kernel records it and returns, the call reports
TT_ERR_TIMEOUT and the context (and device) keep working; and a device-memory
allocation that fails (injected on the host, before cudaMalloc would run)
surfaces as the reference's length_error class with the library's message,
after which the same context recovers."""
import numpy as np
import pytest

from gpu_util import bits, dev, host
from oracle import oracle as O
from turbotops_gb300 import capi, ops, synth
from turbotops_gb300.capi import Context

pytestmark = pytest.mark.gpu


def _dense_ok(c):
    x = synth.gauss(300, 3, 1)
    mat, enc = ops.make_dense(c, dev(x), "l2")
    assert np.array_equal(bits(host(mat)), bits(O.dense(x, "l2")))
    r = ops.dim0(c, mat=mat, threshold=enc, maxdim=1)
    assert r["keys"].numel() > 0


def test_bounded_wait_runs_out_and_context_survives():
    c = Context(0)
    for polls in (1, 4096):
        st = c.L.tt_selftest_wait_timeout(c.h, polls)
        assert st == capi.ERR_TIMEOUT
        assert "timed out" in c.L.tt_last_error(c.h).decode()
    assert c.L.tt_selftest_wait_timeout(c.h, 0) == capi.ERR_INVALID
    _dense_ok(c)


def test_injected_allocation_failure_is_a_length_error():
    c = Context(0)
    assert c.L.tt_ctx_inject_alloc_failure(c.h, 1) == capi.OK
    x = synth.gauss(300, 3, 2)
    # the first arena allocation of a fresh context: the row maxima of the
    # enclosing radius (the matrix itself is the caller's torch tensor)
    with pytest.raises(MemoryError, match="device memory exhausted"):
        ops.make_dense(c, dev(x), "l2")
    _dense_ok(c)   # the next allocation is real again
