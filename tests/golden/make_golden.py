"""Writes the golden fixtures of tests/golden/ (run from the repository root:
``python tests/golden/make_golden.py``).

* plummer2000.fma -- 2,000 Plummer points (seed 7) in the FMA format of
  aran_solver3d_write_fma, lossless digits;
* plummer2000_p10.npz -- the oracle's FP64 FMM of that file (rotate, p = 10,
  maxbox 32, box from the FMA header): potential, field and call counters;
* circle240_p20.npz -- the oracle's 2D solve of tests/dummypot.at's
  "-np 240 -pr 20 -s 10" case (circle of radius 0.9, unit densities).

The fixtures pin the oracle against regressions and give the GPU tests
inputs and outputs that do not depend on a generator.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from aran_gb300 import fma, workloads as W  # noqa: E402


def main():
    x, q = W.plummer(2000, 7)
    path = os.path.join(HERE, "plummer2000.fma")
    fma.write_fma(path, x, q, (-1, -1, -1), (1, 1, 1))
    x, q, lb, ub = fma.read_fma(path)
    pot, st = oracle.solve(x, q, order=10, maxbox=32, field=False, lb=lb, ub=ub)
    fld, _ = oracle.solve(x, q, order=10, maxbox=32, field=True, lb=lb, ub=ub)
    np.savez(os.path.join(HERE, "plummer2000_p10.npz"), pot=pot, field=fld,
             stats=np.array([st[k] for k in oracle.STAT_NAMES]))
    n = 240
    t = 2 * np.pi * np.arange(n) / n
    xy = np.stack([0.9 * np.cos(t), 0.9 * np.sin(t)], 1)
    acc, st2 = oracle.solve2d(xy, np.ones(n), [0, n], [[-1, -1, 1, 1]], 10, 20)
    np.savez(os.path.join(HERE, "circle240_p20.npz"), xy=xy, acc=acc,
             stats=np.array([st2[k] for k in oracle.STAT_NAMES]))


if __name__ == "__main__":
    main()
