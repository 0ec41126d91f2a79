"""Seeded synthetic particle sets of the benchmark configurations.

The reference ships no datasets; its test programs draw particles from
distributions in code (tests/newtonfield3.c:472-583, tests/newtonpot3.c:517-575).
These generators reproduce those distributions (numpy PCG64, fixed seeds):

* uniform(n, seed)     -- uniform in [0,1]^3, charges U[-1,1] (configs 1-2)
* plummer(n, seed)     -- Plummer sphere, scale radius a=0.05, radial cut at
                          r <= 20a = 1 (rejected draws are redrawn), centred at
                          the origin, box [-1,1]^3, charges U[0,1] (config 3);
                          radius r = a / sqrt(x1^(-2/3) - 1), z = (1 - 2 x2) r,
                          (x, y) = sqrt(r^2 - z^2) (cos, sin)(2 pi x3) as in
                          tests/newtonpot3.c:541-551
* blobs(n, seed)       -- 1-8 Gaussian blobs, sigma U[0.02,0.2], centres
                          U[0.2,0.8]^3, clipped to [0,1]^3 (config 4)
* circle(n)            -- tests/newtonfield3.c:472-493
* batch2d(nsys, seed)  -- config 4, 2D part: nsys systems, N log-uniform in
                          [1e3, 1e5], uniform in [-1,1]^2, charges U[-1,1]
* batch3d(nsys, seed)  -- config 4, 3D part: nsys systems, N log-uniform in
                          [1e3, 2e5], uniform in [0,1]^3 or blobs, p in {4,8,12}
"""
from __future__ import annotations

import math

import numpy as np


def uniform(n: int, seed: int = 2, lo=0.0, hi=1.0, qlo=-1.0, qhi=1.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(lo, hi, (n, 3))
    q = rng.uniform(qlo, qhi, n)
    return x, q


def plummer(n: int, seed: int = 3, a: float = 0.05, rcut: float = 1.0):
    rng = np.random.default_rng(seed)
    out = np.empty((n, 3))
    filled = 0
    while filled < n:
        m = int((n - filled) * 1.2) + 16
        x1 = rng.uniform(0.0, 1.0, m)
        x2 = rng.uniform(0.0, 1.0, m)
        x3 = rng.uniform(0.0, 1.0, m)
        with np.errstate(divide="ignore", invalid="ignore"):
            r = a / np.sqrt(x1 ** (-2.0 / 3.0) - 1.0)
        ok = np.isfinite(r) & (r <= rcut)
        r, x2, x3 = r[ok], x2[ok], x3[ok]
        z = (1.0 - 2.0 * x2) * r
        t = np.sqrt(np.maximum(r * r - z * z, 0.0))
        pts = np.stack([t * np.cos(2 * math.pi * x3), t * np.sin(2 * math.pi * x3), z], axis=1)
        k = min(len(pts), n - filled)
        out[filled:filled + k] = pts[:k]
        filled += k
    q = rng.uniform(0.0, 1.0, n)
    return out, q


def blobs(n: int, seed: int = 4, nblobs: int | None = None):
    rng = np.random.default_rng(seed)
    k = int(nblobs) if nblobs else int(rng.integers(1, 9))
    centres = rng.uniform(0.2, 0.8, (k, 3))
    sig = rng.uniform(0.02, 0.2, k)
    which = rng.integers(0, k, n)
    x = centres[which] + rng.normal(size=(n, 3)) * sig[which, None]
    x = np.clip(x, 0.0, np.nextafter(1.0, 0.0))
    q = rng.uniform(-1.0, 1.0, n)
    return x, q


def circle(n: int):
    R = 0.999
    a = 2 * math.pi * np.arange(n) / n
    x = np.stack([R * np.cos(a), R * np.sin(a), np.zeros(n)], axis=1)
    return x, np.full(n, 1.0 / n)


def batch2d(nsys: int = 512, seed: int = 4, nlo: float = 1e3, nhi: float = 1e5):
    """xy (n, 2), q (n,), offsets (nsys + 1,), boxes (nsys, 4) of a batch of
    independent 2D systems."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(nlo), np.log(nhi), nsys)).astype(np.int64)
    n = int(sizes.sum())
    xy = rng.uniform(-1.0, 1.0, (n, 2))
    q = rng.uniform(-1.0, 1.0, n)
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    boxes = np.tile([-1.0, -1.0, 1.0, 1.0], (nsys, 1))
    return xy, q, offs, boxes


def batch3d(nsys: int = 2048, seed: int = 4, nlo: float = 1e3, nhi: float = 2e5):
    """List of (x, q, order) of independent 3D systems in [0,1]^3."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nsys):
        n = int(np.exp(rng.uniform(np.log(nlo), np.log(nhi))))
        p = (4, 8, 12)[int(rng.integers(0, 3))]
        if rng.uniform() < 0.5:
            x, q = uniform(n, 10_000 + i)
        else:
            x, q = blobs(n, 10_000 + i)
        out.append((x, q, p))
    return out
