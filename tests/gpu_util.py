"""Helpers for the GPU parity tests."""
import numpy as np
import torch

IDX_BITS = 33
IDX_MASK = (1 << IDX_BITS) - 1

_CTX = None


def ctx():
    global _CTX
    if _CTX is None:
        from turbotops_gb300.capi import Context
        _CTX = Context(0)
    return _CTX


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def host(t):
    return t.detach().cpu().numpy()


def decode_keys(keys):
    """Ripser keys -> (index u64, diameter f32)."""
    k = host(keys).view(np.uint64)
    d = (k >> np.uint64(IDX_BITS)).astype(np.uint32).view(np.float32)
    idx = np.uint64(IDX_MASK) - (k & np.uint64(IDX_MASK))
    return idx, d


def h0_pairs(r):
    """GPU dim0 H0 output in the reference's Barcode layout (birth, death pairs)."""
    d = host(r["h0"])
    fin = np.stack([np.zeros_like(d), d], 1).ravel()
    ess = np.tile(np.array([0, np.inf], np.float32), int(r["essential"]))
    return np.concatenate([fin, ess]).astype(np.float32)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)
