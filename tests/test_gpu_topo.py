"""Differentiable persistence: forward bars equal the persistence() drop-in's,
and the hand-written adjoint's gradient of the benchmark loss matches an FP64
CPU reference gradient (relative error <= 1e-4) and FP64 central finite
differences, on tie-free clouds (continuous noise)."""
import numpy as np
import pytest
import torch

import turbotops_gb300 as tg
from turbotops_gb300 import synth, topo

pytestmark = pytest.mark.gpu

TOL = 1e-4   # relative L2 error of the gradient vs the FP64 reference


def _clouds(count=4, n=96, sigma=0.1, seed=9):
    return synth.circles(count, n, sigma, seed)


def _selected(b, top=4):
    """Per cloud: the H1 bars the loss picks (top finite persistence)."""
    sel = []
    h1b, h1d = b.h1_birth.detach().cpu().numpy(), b.h1_death.detach().cpu().numpy()
    for q in range(len(b.h1_offset) - 1):
        s, e = int(b.h1_offset[q]), int(b.h1_offset[q + 1])
        idx = np.arange(s, e)
        fin = np.isfinite(h1d[s:e])
        idx = idx[fin]
        pers = (h1d[idx] - h1b[idx]).astype(np.float32)
        order = np.argsort(-pers, kind="stable")[:top]
        sel.extend(idx[order].tolist())
    return np.array(sel, dtype=np.int64)


def _loss64(x64: torch.Tensor, b, sel, metric="l2"):
    def dist(e):
        d = x64[e[:, 0]] - x64[e[:, 1]]
        if metric == "l2":
            return torch.sqrt((d * d).sum(1))
        if metric == "l1":
            return d.abs().sum(1)
        if metric == "linf":
            return d.abs().max(1).values
        p = float(metric[3:])
        return (d.abs() ** p).sum(1) ** (1.0 / p)
    h0e = b.h0_edge.long()
    be = b.h1_birth_edge.long()[sel]
    de = b.h1_death_edge.long()[sel]
    return (dist(h0e) ** 2).sum() - (dist(de) - dist(be)).sum()


@pytest.mark.parametrize("metric", ["l2", "l1", "linf", "lp:1.5"])
def test_adjoint_vs_fp64_reference(metric):
    clouds = _clouds()
    x = torch.from_numpy(np.concatenate(clouds)).cuda().requires_grad_(True)
    sizes = [c.shape[0] for c in clouds]
    loss = topo.topo_loss(x, sizes, metric)
    loss.backward()
    g = x.grad.detach().cpu().double()
    b = topo.diagrams(x.detach(), sizes, metric)
    sel = _selected(b)
    x64 = torch.from_numpy(np.concatenate(clouds)).double().requires_grad_(True)
    l64 = _loss64(x64, b, sel, metric)
    l64.backward()
    ref = x64.grad
    err = (g - ref).norm() / ref.norm()
    assert err < TOL, float(err)
    assert abs(float(loss) - float(l64)) <= 1e-4 * max(1.0, abs(float(l64)))


def test_fp64_central_differences_and_stable_pairing():
    clouds = _clouds(count=2, n=64, seed=12)
    x0 = np.concatenate(clouds)
    sizes = [c.shape[0] for c in clouds]
    x = torch.from_numpy(x0).cuda().requires_grad_(True)
    topo.topo_loss(x, sizes).backward()
    g = x.grad.detach().cpu().double().numpy()
    b = topo.diagrams(x.detach(), sizes)
    sel = _selected(b)
    rng = np.random.default_rng(0)
    coords = rng.choice(x0.size, 24, replace=False)
    h = 1e-5
    for c in coords:
        xp = torch.from_numpy(x0).double()
        xm = xp.clone()
        xp.view(-1)[c] += h
        xm.view(-1)[c] -= h
        fd = (float(_loss64(xp, b, sel)) - float(_loss64(xm, b, sel))) / (2 * h)
        assert abs(fd - g.reshape(-1)[c]) <= 1e-4 * max(1.0, abs(fd)), (c, fd, g.reshape(-1)[c])
    # the pairing is locally constant on tie-free input: a small step keeps it
    xs = torch.from_numpy(x0 + np.float32(1e-6) * rng.standard_normal(x0.shape).astype(np.float32)).cuda()
    b2 = topo.diagrams(xs, sizes)
    assert torch.equal(b2.h0_edge, b.h0_edge)
    assert torch.equal(b2.h1_birth_edge, b.h1_birth_edge) and torch.equal(b2.h1_death_edge, b.h1_death_edge)


def test_forward_bars_equal_persistence():
    clouds = _clouds(count=3, n=80, seed=3)
    x = torch.from_numpy(np.concatenate(clouds)).cuda()
    b = topo.diagrams(x, [c.shape[0] for c in clouds])
    for q, c in enumerate(clouds):
        dg, _ = tg.persistence(c, maxdim=1)
        h0 = np.sort(dg[0][np.isfinite(dg[0][:, 1]), 1])
        s0, e0 = int(b.h0_offset[q]), int(b.h0_offset[q + 1])
        assert np.array_equal(np.sort(b.h0_death[s0:e0].cpu().numpy()), h0)
        s1, e1 = int(b.h1_offset[q]), int(b.h1_offset[q + 1])
        got = np.stack([b.h1_birth[s1:e1].cpu().numpy(), b.h1_death[s1:e1].cpu().numpy()], 1)
        ref = dg[1]
        key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]  # noqa: E731
        assert np.array_equal(key(got), key(ref))


def test_forward_independent_of_reduction_threads():
    """The host reductions run on threads that take clouds as their device
    front end finishes; bars, critical edges and offsets must not depend on
    that schedule (all host threads vs one), an empty cloud included."""
    clouds = _clouds(count=16, n=200, seed=17)
    clouds.insert(5, np.zeros((0, 3), np.float32))
    sizes = [c.shape[0] for c in clouds]
    x = torch.from_numpy(np.concatenate(clouds)).cuda()
    a = topo.diagrams(x, sizes, threads=0)
    b = topo.diagrams(x, sizes, threads=1)
    for f in ["h0_offset", "h0_death", "h0_edge", "h1_offset", "h1_birth", "h1_death", "h1_birth_edge",
              "h1_death_edge"]:
        u, v = getattr(a, f), getattr(b, f)
        assert torch.equal(torch.as_tensor(u), torch.as_tensor(v)), f
    assert int(a.h1_offset[6]) == int(a.h1_offset[5])   # the empty cloud has no bars


def test_adjoint_at_configuration_size():
    """The bench's differentiable workload itself (64 noisy circles x 512
    points, sigma 0.1, seed 5, L2): gradient against the FP64 reference of the
    same pairing, loss within 1e-4, and the forward bars of a sample of the
    clouds against persistence() cloud by cloud."""
    clouds = synth.circles()
    assert len(clouds) == 64 and all(c.shape == (512, 3) for c in clouds)
    x = torch.from_numpy(np.concatenate(clouds)).cuda().requires_grad_(True)
    sizes = [c.shape[0] for c in clouds]
    loss = topo.topo_loss(x, sizes)
    loss.backward()
    g = x.grad.detach().cpu().double()
    b = topo.diagrams(x.detach(), sizes)
    sel = _selected(b)
    x64 = torch.from_numpy(np.concatenate(clouds)).double().requires_grad_(True)
    l64 = _loss64(x64, b, sel)
    l64.backward()
    err = (g - x64.grad).norm() / x64.grad.norm()
    assert err < TOL, float(err)
    assert abs(float(loss) - float(l64)) <= 1e-4 * max(1.0, abs(float(l64)))
    for q in (0, 21, 63):
        dg, _ = tg.persistence(clouds[q], maxdim=1)
        s1, e1 = int(b.h1_offset[q]), int(b.h1_offset[q + 1])
        got = np.stack([b.h1_birth[s1:e1].cpu().numpy(), b.h1_death[s1:e1].cpu().numpy()], 1)
        key = lambda a: a[np.lexsort((a[:, 1], a[:, 0]))]  # noqa: E731
        assert np.array_equal(key(got), key(dg[1])), q
