"""Seeded synthetic point clouds for the five benchmark workloads.

No public dataset is involved: every workload is generated here with numpy's
``default_rng`` so that the bench, the tests and the CPU baseline all see the
same float32 bits on every machine.

* ``torus(n=1000)``            seed 1 — torus R=2, r=1, angles U[0, 2pi), + N(0, 0.05^2)
* ``lattice(n=3000)``          seed 2 — distinct points of {0..15}^4, exact float32
* ``gmm(n=100000, dim=32)``    seed 3 — 16 centres ~ N(0, 4I), sigma 1, equal weights
* ``circle_batch(512)``        seed 4 — 512 clouds, n ~ U[64, 2048], circle or
                               figure-eight, radius ~ U[0.5, 2], sigma 0.03, in z = 0
* ``circles(64, 512)``         seed 5 — 64 noisy unit circles, sigma 0.1
"""
from __future__ import annotations

import numpy as np


def torus(n: int = 1000, seed: int = 1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    th = rng.uniform(0, 2 * np.pi, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    x = np.c_[(2 + np.cos(th)) * np.cos(ph), (2 + np.cos(th)) * np.sin(ph), np.sin(th)]
    x = x + rng.normal(0, 0.05, (n, 3))
    return np.ascontiguousarray(x, dtype=np.float32)


def lattice(n: int = 3000, seed: int = 2, side: int = 16, dim: int = 4) -> np.ndarray:
    rng = np.random.default_rng(seed)
    idx = rng.choice(side ** dim, n, replace=False)
    x = np.stack([(idx // side ** k) % side for k in range(dim)], 1)
    return np.ascontiguousarray(x, dtype=np.float32)


def gmm(n: int = 100_000, dim: int = 32, centres: int = 16, seed: int = 3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    c = rng.normal(0, 2, (centres, dim))
    a = rng.integers(0, centres, n)
    x = c[a] + rng.normal(0, 1, (n, dim))
    return np.ascontiguousarray(x, dtype=np.float32)


def circle_batch(count: int = 512, lo: int = 64, hi: int = 2048, seed: int = 4) -> list[np.ndarray]:
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, count)
    out = []
    for m in sizes:
        r = rng.uniform(0.5, 2)
        t = rng.uniform(0, 2 * np.pi, m)
        if rng.random() < 0.5:
            y = np.c_[r * np.cos(t), r * np.sin(t), np.zeros(m)]
        else:   # figure-eight: two circles tangent at the origin
            s = rng.random(m) < 0.5
            y = np.c_[np.where(s, r * np.cos(t) - r, r * np.cos(t) + r), r * np.sin(t), np.zeros(m)]
        y = y + rng.normal(0, 0.03, y.shape)
        out.append(np.ascontiguousarray(y, dtype=np.float32))
    return out


def circles(count: int = 64, n: int = 512, sigma: float = 0.1, seed: int = 5) -> list[np.ndarray]:
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        t = rng.uniform(0, 2 * np.pi, n)
        y = np.c_[np.cos(t), np.sin(t), np.zeros(n)] + rng.normal(0, sigma, (n, 3))
        out.append(np.ascontiguousarray(y, dtype=np.float32))
    return out


def uniform(n: int, dim: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).random((n, dim), dtype=np.float32)


def gauss(n: int, dim: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal((n, dim), dtype=np.float32)


def grid(n: int, dim: int, side: int, seed: int) -> np.ndarray:
    """Distinct integer-lattice points: maximal distance ties."""
    return lattice(n, seed, side, dim)
