"""Text particle files of LibAran's test programs.

Two formats, both read and written here so that inputs (and served requests)
can be shared between the GPU path, the oracle and the reference's programs:

* FMA, as ``aran_solver3d_write_fma`` writes it
  (tests/newtonfield3parallel.c:1186-1212): a header line
  ``np half_width cx cy cz`` (the bounding cube's half width and centre), then
  ``x y z density`` per point;
* the point list ``_load_fill`` reads (tests/newtonfield3parallel.c:1020-1083):
  ``index x y z density`` per line, the index placing the point.

The reference prints with ``%g`` (6 significant digits); ``write_fma`` does the
same with ``digits=None`` and writes lossless values otherwise.
"""
from __future__ import annotations

import numpy as np


def _fmt(digits):
    return "%g" if digits is None else "%.{}g".format(int(digits))


def write_fma(path, xyz, q, lb, ub, digits: int | None = 17) -> None:
    """Header ``np half_width cx cy cz`` (cube around [lb, ub]) + points."""
    xyz = np.asarray(xyz, np.float64)
    q = np.asarray(q, np.float64)
    lb = np.asarray(lb, np.float64)
    ub = np.asarray(ub, np.float64)
    c = lb + 0.5 * (ub - lb)
    half = float(np.max(ub - c))
    f = _fmt(digits)
    with open(path, "w") as fh:
        fh.write(("%d " + " ".join([f] * 4) + "\n") % (len(q), half, c[0], c[1], c[2]))
        for (x, y, z), d in zip(xyz, q):
            fh.write((" ".join([f] * 4) + "\n") % (x, y, z, d))


def read_fma(path):
    """Returns (xyz (n, 3), q (n,), lb (3,), ub (3,)) of an FMA file."""
    with open(path) as fh:
        head = fh.readline().split()
        if len(head) != 5:
            raise ValueError(f"{path}: FMA header needs 5 fields, got {len(head)}")
        n = int(head[0])
        half = float(head[1])
        c = np.array([float(v) for v in head[2:5]])
        data = np.loadtxt(fh, dtype=np.float64, ndmin=2)
    if data.shape != (n, 4):
        raise ValueError(f"{path}: expected {n} rows of 4 values, got {data.shape}")
    return data[:, :3].copy(), data[:, 3].copy(), c - half, c + half


def write_points(path, xyz, q, digits: int | None = 17) -> None:
    """``index x y z density`` per line."""
    f = _fmt(digits)
    with open(path, "w") as fh:
        for i, ((x, y, z), d) in enumerate(zip(np.asarray(xyz), np.asarray(q))):
            fh.write(("%d " + " ".join([f] * 4) + "\n") % (i, x, y, z, d))


def read_points(path):
    """Returns (xyz, q) with point i at its file index."""
    data = np.loadtxt(path, dtype=np.float64, ndmin=2)
    if data.shape[1] != 5:
        raise ValueError(f"{path}: expected 5 columns, got {data.shape[1]}")
    idx = data[:, 0].astype(np.int64)
    n = int(idx.max()) + 1 if len(idx) else 0
    if len(np.unique(idx)) != len(idx) or n != len(idx):
        raise ValueError(f"{path}: indices must be 0..n-1, each once")
    xyz = np.empty((n, 3))
    q = np.empty(n)
    xyz[idx] = data[:, 1:4]
    q[idx] = data[:, 4]
    return xyz, q
