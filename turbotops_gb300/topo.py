"""Differentiable persistence on the GB300 front end.

``diagrams(x, sizes)`` returns, for clouds stored back to back in ``x``
(requires_grad allowed), every H0 death and H1 (birth, death) as torch
tensors whose gradients flow back through a ``torch.autograd.Function``:
its backward calls the hand-written adjoint kernel (``tt_topo_adjoint``)
that scatters dL/d(birth, death) through each bar's critical edge onto the
coordinates. The pairing is recomputed by every forward, never stored.

``topo_loss(x, sizes)`` is the loss of the benchmark's differentiable
workload: sum over clouds of  -sum(top-4 finite H1 persistence) +
sum(H0 death^2).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import capi

_CTX = {}


def _context(device: int) -> capi.Context:
    if device not in _CTX:
        _CTX[device] = capi.Context(device)
    return _CTX[device]


@dataclass
class Bars:
    h0_death: torch.Tensor        # (B0,) float32, differentiable
    h1_birth: torch.Tensor        # (B1,) float32, differentiable
    h1_death: torch.Tensor        # (B1,) float32 (+inf for essential bars), differentiable
    h0_offset: np.ndarray         # clouds + 1
    h1_offset: np.ndarray         # clouds + 1
    h0_edge: torch.Tensor         # (B0, 2) int32 point ids (critical edges)
    h1_birth_edge: torch.Tensor   # (B1, 2)
    h1_death_edge: torch.Tensor   # (B1, 2), -1 for essential bars


def _arr(ptr, count, dtype):
    return np.ctypeslib.as_array(ptr, shape=(max(count, 1),))[:count].astype(dtype, copy=True)


class _Diagrams(torch.autograd.Function):
    @staticmethod
    def forward(fctx, x, sizes, device, kind, p, threads, holder):
        ctx = _context(device)
        xs = x.detach().contiguous()
        dim = xs.shape[1]
        out = C.POINTER(capi.TopoOut)()
        ctx.check(ctx.L.tt_topo_forward(ctx.h, xs.data_ptr(), sizes.ctypes.data, len(sizes), dim, kind, p, threads,
                                        C.byref(out)))
        try:
            o = out.contents
            c = o.clouds
            h0_off = _arr(o.h0_offset, c + 1, np.int64)
            h1_off = _arr(o.h1_offset, c + 1, np.int64)
            b0, b1 = int(h0_off[-1]), int(h1_off[-1])
            h0d = _arr(o.h0_death, b0, np.float32)
            h0e = _arr(o.h0_edge, 2 * b0, np.uint32)
            h1b = _arr(o.h1_birth, b1, np.float32)
            h1d = _arr(o.h1_death, b1, np.float32)
            h1be = _arr(o.h1_birth_edge, 2 * b1, np.uint32)
            h1de = _arr(o.h1_death_edge, 2 * b1, np.uint32)
        finally:
            ctx.L.tt_topo_free(out)
        dev = x.device
        edges = torch.from_numpy(np.concatenate([h0e, h1be, h1de]).view(np.int32)).to(dev)
        fctx.save_for_backward(xs, edges)
        fctx.meta = (device, kind, p, b0, b1)
        holder.update(h0_off=h0_off, h1_off=h1_off,
                      h0e=torch.from_numpy(h0e.view(np.int32).reshape(-1, 2)),
                      h1be=torch.from_numpy(h1be.view(np.int32).reshape(-1, 2)),
                      h1de=torch.from_numpy(h1de.view(np.int32).reshape(-1, 2)))
        return (torch.from_numpy(h0d).to(dev), torch.from_numpy(h1b).to(dev), torch.from_numpy(h1d).to(dev))

    @staticmethod
    def backward(fctx, g0, gb, gd):
        xs, edges = fctx.saved_tensors
        device, kind, p, b0, b1 = fctx.meta
        ctx = _context(device)
        dev = xs.device
        z0 = torch.zeros(b0, dtype=torch.float32, device=dev)
        z1 = torch.zeros(b1, dtype=torch.float32, device=dev)
        gd = torch.nan_to_num(gd, nan=0.0, posinf=0.0, neginf=0.0) if gd is not None else z1
        g = torch.cat([g0 if g0 is not None else z0, gb if gb is not None else z1, gd]).contiguous().float()
        grad = torch.zeros_like(xs)
        ctx.check(ctx.L.tt_topo_adjoint(ctx.h, xs.data_ptr(), xs.shape[1], kind, p, edges.data_ptr(), g.data_ptr(),
                                        g.numel(), grad.data_ptr()))
        return grad, None, None, None, None, None, None


def diagrams(x: torch.Tensor, sizes, metric: str = "l2", threads: int = 0) -> Bars:
    """Dense full-Rips diagrams (H0 finite deaths, all H1 bars) of every cloud, differentiable in x."""
    if not (x.is_cuda and x.dtype == torch.float32 and x.dim() == 2):
        raise ValueError("x must be a (sum(sizes), dim) float32 CUDA tensor")
    sizes = np.ascontiguousarray(sizes, np.uint32)
    if int(sizes.sum()) != x.shape[0]:
        raise ValueError("sizes must add up to x.shape[0]")
    kind, p = capi.metric_parse(metric)
    holder: dict = {}
    h0d, h1b, h1d = _Diagrams.apply(x, sizes, x.device.index or 0, kind, p, int(threads), holder)
    return Bars(h0d, h1b, h1d, holder["h0_off"], holder["h1_off"], holder["h0e"], holder["h1be"], holder["h1de"])


def topo_loss(x: torch.Tensor, sizes, metric: str = "l2", top: int = 4, threads: int = 0) -> torch.Tensor:
    """-sum(top-`top` finite H1 persistence) + sum(H0 death^2), summed over clouds."""
    b = diagrams(x, sizes, metric, threads)
    loss = x.new_zeros(())
    for q in range(len(b.h0_offset) - 1):
        s0, e0 = int(b.h0_offset[q]), int(b.h0_offset[q + 1])
        s1, e1 = int(b.h1_offset[q]), int(b.h1_offset[q + 1])
        loss = loss + (b.h0_death[s0:e0] ** 2).sum()
        d, bb = b.h1_death[s1:e1], b.h1_birth[s1:e1]
        fin = torch.isfinite(d)
        pers = (d - bb)[fin]
        if pers.numel():
            loss = loss - torch.topk(pers, min(top, pers.numel())).values.sum()
    return loss
