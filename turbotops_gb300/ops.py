"""Device-resident front-end stages on torch tensors (all on one CUDA device).

Each function calls exactly one C-ABI entry point; results are torch tensors
on the device. Names follow the reference functions they replace.
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import capi
from .capi import Context, ptr


def _f32(x: torch.Tensor) -> torch.Tensor:
    if x.dtype != torch.float32 or not x.is_cuda:
        raise ValueError("expected a float32 CUDA tensor")
    return x.contiguous()


def make_dense(ctx: Context, x: torch.Tensor, metric: str = "l2") -> tuple[torch.Tensor, float]:
    """rips.hpp make_dense (full layout) + enclosing_radius: (n x n matrix, radius)."""
    x = _f32(x)
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    mat = torch.empty((n, n), dtype=torch.float32, device=x.device)
    enc = C.c_float()
    ctx.check(ctx.L.tt_dense_distances(ctx.h, ptr(x), n, dim, kind, p, ptr(mat), C.byref(enc)))
    return mat, enc.value


def _view(ctx: Context, addr: int, count: int, dtype: torch.dtype, device) -> torch.Tensor:
    """Copy a context-owned device array into a fresh torch tensor (stream-ordered)."""
    out = torch.empty(count, dtype=dtype, device=device)
    if count:
        ctx.check(ctx.L.tt_copy_async(ctx.h, C.c_void_p(out.data_ptr()), C.c_void_p(addr),
                                      count * out.element_size()))
    return out


def dim0(ctx: Context, mat: torch.Tensor | None = None, csr: tuple | None = None, n: int | None = None,
         threshold: float = math.inf, maxdim: int = 1) -> dict:
    """rips.hpp Reducer::dim0 on a dense matrix or a CSR graph (rp u64, ci u32, w f32)."""
    if mat is not None:
        n = mat.shape[0]
        rp = ci = w = None
        dev = mat.device
    else:
        rp, ci, w = csr
        dev = rp.device
        if n is None:
            n = rp.numel() - 1
    out = capi.Dim0Out()
    ctx.check(ctx.L.tt_dim0(ctx.h, ptr(mat), ptr(rp), ptr(ci), ptr(w), n, float(threshold), maxdim,
                            C.byref(out)))
    m, c, h = out.edges, out.columns, out.h0_finite
    r = {
        "keys": _view(ctx, out.edge_keys_dev, m, torch.int64, dev),
        "tree": _view(ctx, out.tree_dev, m, torch.uint8, dev),
        "cidx": _view(ctx, out.col_index_dev, c, torch.int64, dev),
        "cd": _view(ctx, out.col_diameter_dev, c, torch.float32, dev),
        "emi": _view(ctx, out.col_cofacet_dev, c, torch.int64, dev),
        "emf": _view(ctx, out.col_cofacet_app_dev, c, torch.uint8, dev),
        "h0": _view(ctx, out.h0_death_dev, h, torch.float32, dev),
        "essential": out.essential,
    }
    r["app"] = _view(ctx, out.apparent_dev, m, torch.uint8, dev) if out.apparent_dev else None
    torch.cuda.current_stream(dev).synchronize()
    return r


def redzed_edges(ctx: Context, mat: torch.Tensor | None = None, csr: tuple | None = None, n: int | None = None,
                 threshold: float = math.inf) -> tuple[torch.Tensor, torch.Tensor]:
    """redzed::detail::build_edges: (diameters, vertex pairs) in (d asc, comb asc) order."""
    if mat is not None:
        n = mat.shape[0]
        rp = ci = w = None
        dev = mat.device
        cap = n * (n - 1) // 2
    else:
        rp, ci, w = csr
        dev = rp.device
        n = rp.numel() - 1 if n is None else n
        cap = ci.numel() // 2
    d = torch.empty(max(cap, 1), dtype=torch.float32, device=dev)
    v = torch.empty(2 * max(cap, 1), dtype=torch.int32, device=dev)
    cnt = C.c_uint64()
    ctx.check(ctx.L.tt_redzed_edges(ctx.h, ptr(mat), ptr(rp), ptr(ci), ptr(w), n, float(threshold), ptr(d),
                                    ptr(v), cap, C.byref(cnt)))
    m = cnt.value
    return d[:m], v[: 2 * m]


def knn(ctx: Context, x: torch.Tensor, k: int, metric: str = "l2") -> tuple[torch.Tensor, torch.Tensor]:
    """graph.hpp knn_lists_exact: (ids n x k, distances n x k), ascending (d, id)."""
    x = _f32(x)
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    kk = min(k, n - 1) if n else 0
    ids = torch.empty((n, max(kk, 1)), dtype=torch.int32, device=x.device)
    d = torch.empty((n, max(kk, 1)), dtype=torch.float32, device=x.device)
    ko = C.c_uint32()
    ctx.check(ctx.L.tt_knn(ctx.h, ptr(x), n, dim, kind, p, k, ptr(ids), ptr(d), C.byref(ko)))
    return ids[:, :kk], d[:, :kk]


def _csr(ctx: Context, out, dev) -> tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
    rp = _view(ctx, out.row_ptr_dev, out.n + 1, torch.int64, dev)
    ci = _view(ctx, out.col_dev, out.nnz, torch.int32, dev)
    w = _view(ctx, out.weight_dev, out.nnz, torch.float32, dev)
    torch.cuda.current_stream(dev).synchronize()
    return rp, ci, w


def knn_graph(ctx: Context, x: torch.Tensor, k: int, metric: str = "l2") -> tuple:
    """graph.hpp knn_lists_exact + knn_graph: CSR (row_ptr i64, col i32, weight f32)."""
    x = _f32(x)
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    out = capi.CsrOut()
    ctx.check(ctx.L.tt_knn_graph(ctx.h, ptr(x), n, dim, kind, p, k, C.byref(out)))
    return _csr(ctx, out, x.device)


def radius_graph(ctx: Context, x: torch.Tensor, tau: float, metric: str = "l2") -> tuple:
    """graph.hpp radius_graph: CSR of all pairs with d <= tau."""
    x = _f32(x)
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    out = capi.CsrOut()
    ctx.check(ctx.L.tt_radius_graph(ctx.h, ptr(x), n, dim, kind, p, float(tau), C.byref(out)))
    return _csr(ctx, out, x.device)


def mst_deaths(ctx: Context, x: torch.Tensor, metric: str = "l2") -> torch.Tensor:
    """Sorted minimum-spanning-tree weights of the complete graph (mst.hpp:25-99)."""
    x = _f32(x)
    n, dim = x.shape
    kind, p = capi.metric_parse(metric)
    d = torch.empty(max(n, 1), dtype=torch.float32, device=x.device)
    ctx.check(ctx.L.tt_mst_deaths(ctx.h, ptr(x), n, dim, kind, p, ptr(d)))
    return d[: max(n - 1, 0)]


def h0_bars(deaths, threshold: float = math.inf):
    """mst::h0's bars (mst.hpp:91-97) from sorted deaths: (birth, death) pairs."""
    import numpy as np
    d = deaths.detach().cpu().numpy() if hasattr(deaths, "detach") else np.asarray(deaths)
    n = d.size + 1 if d.size or threshold is not None else 0
    fin = d[(d <= threshold) & (d > 0)]
    ess = 1 + int((d > threshold).sum())
    bars = [np.stack([np.zeros_like(fin), fin], 1).ravel(), np.tile(np.array([0, np.inf], np.float32), ess)]
    return np.concatenate(bars).astype(np.float32)


def assemble(ctx: Context, mat: torch.Tensor, threshold: float, edge_keys: torch.Tensor,
             pivots: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor, int]:
    """rips.hpp Reducer::assemble(1): dim-2 columns (index i64, diameter f32), descending; apparent count."""
    n = mat.shape[0]
    cnt, app = C.c_uint64(), C.c_uint64()
    ci, cd = C.c_void_p(), C.c_void_p()
    piv = pivots.contiguous()
    ctx.check(ctx.L.tt_assemble(ctx.h, ptr(mat), n, float(threshold), ptr(edge_keys), edge_keys.numel(),
                                ptr(piv) if piv.numel() else None, piv.numel(), C.byref(cnt), C.byref(ci),
                                C.byref(cd), C.byref(app)))
    c = cnt.value
    idx = _view(ctx, ci.value or 0, c, torch.int64, mat.device)
    d = _view(ctx, cd.value or 0, c, torch.float32, mat.device)
    torch.cuda.current_stream(mat.device).synchronize()
    return idx, d, app.value


class DenseBatch:
    """The dense front end of a batch of clouds (tt_batch_*): per-cloud
    enclosing radius and RedZeD edge list from one captured CUDA graph."""

    def __init__(self, ctx: Context, sizes, dim: int, metric: str = "l2", use_graph: bool = True):
        import numpy as np
        self.ctx = ctx
        self.sizes = np.ascontiguousarray(sizes, np.uint32)
        self.dim = dim
        kind, p = capi.metric_parse(metric)
        h = C.c_void_p()
        ctx.check(ctx.L.tt_batch_create(ctx.h, self.sizes.ctypes.data, len(self.sizes), dim, kind, p,
                                        1 if use_graph else 0, C.byref(h)))
        self.h = h
        self.total = int(self.sizes.sum())

    def load(self, points: torch.Tensor) -> None:
        """Copy the clouds (sum(sizes) x dim, back to back) into the batch's input buffer."""
        pts = _f32(points)
        dst = self.ctx.L.tt_batch_points(self.h)
        self.ctx.check(self.ctx.L.tt_copy_async(self.ctx.h, C.c_void_p(dst), C.c_void_p(pts.data_ptr()),
                                                self.total * self.dim * 4))
        self.ctx.synchronize()

    def run(self, wait: bool = True) -> None:
        self.ctx.check(self.ctx.L.tt_batch_run(self.h, 1 if wait else 0))

    def result(self) -> dict:
        out = capi.BatchOut()
        self.ctx.check(self.ctx.L.tt_batch_result(self.h, C.byref(out)))
        dev = torch.device("cuda", self.ctx.device)
        c = out.clouds
        off = _view(self.ctx, out.edge_offset_dev, c + 1, torch.int64, dev)
        torch.cuda.current_stream(dev).synchronize()
        m = int(off[-1].item())
        r = {"radius": _view(self.ctx, out.radius_dev, c, torch.float32, dev), "edge_offset": off,
             "diam": _view(self.ctx, out.diam_dev, m, torch.float32, dev),
             "verts": _view(self.ctx, out.verts_dev, 2 * m, torch.int32, dev)}
        torch.cuda.current_stream(dev).synchronize()
        return r

    def close(self):
        if getattr(self, "h", None):
            self.ctx.L.tt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
