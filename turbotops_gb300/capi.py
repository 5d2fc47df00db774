"""ctypes binding of the C-ABI (include/turbotops_gb300.h).

This is the only way Python reaches the GPU code: there is no CPU fallback.
If the CUDA library is not built, or no CUDA device is present, every entry
point raises instead of computing anything on the host.

Device memory and streams come from PyTorch (plumbing only): arguments that
are device pointers are taken from ``torch.Tensor.data_ptr()`` and every call
runs on the current torch stream of the context's device.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import threading

from . import build as _build

P = C.c_void_p
u32, u64, f32, i32 = C.c_uint32, C.c_uint64, C.c_float, C.c_int

METRIC_L1, METRIC_L2, METRIC_LINF, METRIC_LP = 0, 1, 2, 3
OK, ERR_INVALID, ERR_OVERFLOW, ERR_LENGTH, ERR_CUDA, ERR_TIMEOUT, ERR_INTERNAL = range(7)


class CsrOut(C.Structure):
    _fields_ = [("n", u32), ("nnz", u64), ("row_ptr_dev", P), ("col_dev", P), ("weight_dev", P)]


class Dim0Out(C.Structure):
    _fields_ = [("edges", u64), ("edge_keys_dev", P), ("apparent_dev", P), ("tree_dev", P),
                ("columns", u64), ("col_index_dev", P), ("col_diameter_dev", P), ("col_cofacet_dev", P),
                ("col_cofacet_app_dev", P), ("h0_finite", u64), ("h0_death_dev", P), ("essential", u64)]


class Barcode(C.Structure):
    _fields_ = [("ndims", u32), ("total", u64), ("count", C.POINTER(u64)), ("birth", C.POINTER(f32)),
                ("death", C.POINTER(f32)), ("method", C.c_char * 32), ("threshold", f32), ("edges", u64),
                ("columns", u64 * 32), ("apparent", u64 * 32), ("emergent", u64 * 32)]


class KnnFrontOut(C.Structure):
    _fields_ = [("graph", CsrOut), ("dim0", Dim0Out)]


_SIGS = {
    "tt_version": (C.c_char_p, []),
    "tt_ctx_create": (i32, [i32, P, C.POINTER(P)]),
    "tt_ctx_destroy": (None, [P]),
    "tt_last_error": (C.c_char_p, [P]),
    "tt_ctx_launches": (u64, [P]),
    "tt_ctx_synchronize": (i32, [P]),
    "tt_copy_async": (i32, [P, P, P, C.c_size_t]),
    "tt_ctx_set_knn_mode": (i32, [P, i32]),
    "tt_ctx_set_memory_budget": (i32, [P, u64]),
    "tt_parse_points_h": (i32, [P, P, u64, P, u64, C.POINTER(u32), C.POINTER(u32)]),
    "tt_ctx_filter_evals": (u64, [P]),
    "tt_ctx_filter_tiles": (u64, [P]),
    "tt_tc_gram_check": (i32, [P, u32, u64, P]),
    "tt_selftest_wait_timeout": (i32, [P, u32]),
    "tt_ctx_inject_alloc_failure": (i32, [P, u32]),
    "tt_metric_parse": (i32, [C.c_char_p, C.POINTER(i32), C.POINTER(f32)]),
    "tt_dense_distances": (i32, [P, P, u32, u32, i32, f32, P, C.POINTER(f32)]),
    "tt_dense_distances_static": (i32, [P, u32, u32, i32, f32, P, P, P]),
    "tt_dim0": (i32, [P, P, P, P, P, u32, f32, u32, C.POINTER(Dim0Out)]),
    "tt_redzed_edges": (i32, [P, P, P, P, P, u32, f32, P, P, u64, C.POINTER(u64)]),
    "tt_knn": (i32, [P, P, u32, u32, i32, f32, u32, P, P, C.POINTER(u32)]),
    "tt_knn_graph": (i32, [P, P, u32, u32, i32, f32, u32, C.POINTER(CsrOut)]),
    "tt_radius_graph": (i32, [P, P, u32, u32, i32, f32, f32, C.POINTER(CsrOut)]),
    "tt_mst_deaths": (i32, [P, P, u32, u32, i32, f32, P]),
    "tt_knn_graph_h": (i32, [P, P, u32, u32, i32, f32, u32, P, P, P, u64, C.POINTER(u64)]),
    "tt_radius_graph_h": (i32, [P, P, u32, u32, i32, f32, f32, P, P, P, u64, C.POINTER(u64)]),
    "tt_assemble": (i32, [P, P, u32, f32, P, u64, P, u64, C.POINTER(u64), C.POINTER(P), C.POINTER(P),
                          C.POINTER(u64)]),
    "tt_persistence_h": (i32, [P, P, u32, u32, i32, f32, u32, f32, i32, u32, C.POINTER(C.POINTER(Barcode))]),
    "tt_persistence_graph_h": (i32, [P, P, P, P, u32, u32, f32, C.POINTER(C.POINTER(Barcode))]),
    "tt_barcode_free": (None, [C.POINTER(Barcode)]),
    "tt_knn_front": (i32, [P, P, u32, u32, i32, f32, u32, u32, C.POINTER(KnnFrontOut)]),
    "tt_knn_front_h": (i32, [P, P, u32, u32, i32, f32, u32, u32, P, P, P, u64, C.POINTER(u64), P,
                             C.POINTER(u64), C.POINTER(u64), P, P, P, P, u64, C.POINTER(u64), C.POINTER(u64)]),
    "tt_batch_tuning": (i32, [P, P, P, P, P, P]),
    "tt_dense_redzed_h": (i32, [P, P, u32, u32, i32, f32, C.POINTER(f32), P, P, P, u64, C.POINTER(u64)]),
    "tt_dense_redzed_pred_h": (i32, [P, P, u32, u32, i32, f32, C.POINTER(f32), P, P, P, u64, C.POINTER(u64), P]),
    "tt_redzed_leftover_h": (i32, [P, P, u32, f32, P]),
    "tt_graph_redzed_h": (i32, [P, P, P, P, u32, f32, P, P, u64, C.POINTER(u64)]),
    "tt_dense_front_h": (i32, [P, P, u32, u32, i32, f32, u32, C.POINTER(f32), P, P, C.POINTER(u64),
                               C.POINTER(u64), P, P, P, P, u64, C.POINTER(u64), C.POINTER(u64)]),
}

_lib = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load the CUDA library (building it in-tree if needed). Raises if absent."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_build.LIB):
                if not build_if_missing:
                    raise RuntimeError("libturbotops_gb300.so is not built (run turbotops_gb300.build); "
                                       "there is no CPU fallback")
                _build.build()
            L = C.CDLL(_build.LIB)
            for name, (res, args) in _SIGS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def raise_for(status: int, msg: str) -> None:
    if status == OK:
        return
    if status == ERR_INVALID:
        raise ValueError(msg)
    if status == ERR_OVERFLOW:
        raise OverflowError(msg)
    if status == ERR_LENGTH:
        raise MemoryError(msg)
    raise RuntimeError(msg)


def metric_parse(s: str) -> tuple[int, float]:
    L = load()
    k, p = i32(), f32()
    st = L.tt_metric_parse(s.encode(), C.byref(k), C.byref(p))
    raise_for(st, L.tt_last_error(None).decode())
    return k.value, p.value


class Context:
    """A device context bound to the current torch stream of ``device``."""

    def __init__(self, device: int = 0, stream=None):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("turbotops_gb300 needs a CUDA device (GB300); there is no CPU fallback")
        self.L = load()
        self.device = device
        if stream is None:
            stream = torch.cuda.current_stream(device)
        self.stream = stream
        h = P()
        st = self.L.tt_ctx_create(device, P(stream.cuda_stream), C.byref(h))
        raise_for(st, self.L.tt_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.tt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, st: int) -> None:
        if st != OK:
            raise_for(st, self.L.tt_last_error(self.h).decode())

    @property
    def launches(self) -> int:
        return int(self.L.tt_ctx_launches(self.h))

    def synchronize(self):
        self.check(self.L.tt_ctx_synchronize(self.h))


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def fthr(t: float) -> float:
    return math.inf if t is None else float(t)


class BatchOut(C.Structure):
    _fields_ = [("clouds", u32), ("total_points", u64), ("radius_dev", P), ("edge_offset_dev", P),
                ("diam_dev", P), ("verts_dev", P), ("mats_dev", P), ("stream", P)]


_SIGS.update({
    "tt_batch_create": (i32, [P, P, u32, u32, i32, f32, i32, C.POINTER(P)]),
    "tt_batch_points": (P, [P]),
    "tt_batch_run": (i32, [P, i32]),
    "tt_batch_result": (i32, [P, C.POINTER(BatchOut)]),
    "tt_batch_destroy": (None, [P]),
})


class TopoOut(C.Structure):
    _fields_ = [("clouds", u32), ("h0_offset", C.POINTER(u64)), ("h0_death", C.POINTER(f32)),
                ("h0_edge", C.POINTER(u32)), ("h1_offset", C.POINTER(u64)), ("h1_birth", C.POINTER(f32)),
                ("h1_death", C.POINTER(f32)), ("h1_birth_edge", C.POINTER(u32)), ("h1_death_edge", C.POINTER(u32)),
                ("opaque", P)]


_SIGS.update({
    "tt_topo_forward": (i32, [P, P, P, u32, u32, i32, f32, i32, C.POINTER(C.POINTER(TopoOut))]),
    "tt_topo_free": (None, [C.POINTER(TopoOut)]),
    "tt_topo_adjoint": (i32, [P, P, u32, i32, f32, P, P, u64, P]),
})
