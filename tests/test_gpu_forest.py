"""Forest solves: several independent systems in one solve.

* each system's results equal those of the same system solved alone in its
  box (rel-L2 1e-12 in FP64, 1e-10 mixed: only the order of FP64 atomic
  additions differs), in both flavours and at an order with FP64 root
  levels; the call counters are the sums of the systems' own counters;
* a system may be empty or hold one particle;
* the FP64 forest matches the oracle solving each system alone;
* boxes whose extents differ from the solver's, and offsets that do not
  cover the particles, are refused before any work.
"""
import numpy as np
import pytest

from aran_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def systems():
    """Boxes of extent 1 at different origins; N from 0 to 40k."""
    out = []
    spec = [(12000, "uniform", (0.0, 0.0, 0.0)), (0, "uniform", (5.0, 5.0, 5.0)),
            (1, "uniform", (-1.0, 0.0, 2.0)), (40000, "plummer", (-0.5, -0.5, -0.5)),
            (700, "uniform", (3.25, -7.5, 0.125)), (25000, "blobs", (10.0, 0.0, 0.0))]
    for i, (n, kind, lo) in enumerate(spec):
        lo = np.array(lo)
        if kind == "uniform":
            x, q = W.uniform(max(n, 1), 60 + i)
            x = x[:n] + lo
            q = q[:n]
        elif kind == "plummer":
            x, q = W.plummer(n, 60 + i)
            x = 0.5 * x + lo + 0.5     # radius 0.5 around the box centre
        else:
            rng = np.random.default_rng(60 + i)
            c = rng.uniform(0.2, 0.8, (4, 3))
            x = np.clip(c[rng.integers(0, 4, n)] + rng.normal(0, 0.05, (n, 3)), 0.0, 0.999999)
            x = x + lo
            q = rng.uniform(-1, 1, n)
        out.append((x, q, np.concatenate([lo, lo + 1.0])))
    return out


def concat(sy):
    x = np.concatenate([s[0] for s in sy]).reshape(-1, 3)
    q = np.concatenate([s[1] for s in sy])
    offs = np.concatenate([[0], np.cumsum([len(s[1]) for s in sy])]).astype(np.int64)
    boxes = np.stack([s[2] for s in sy])
    return x, q, offs, boxes


@pytest.mark.parametrize("order,precision,flavour", [(8, "fp64", "rotate"), (8, "mixed", "rotate"),
                                                     (12, "mixed", "rotate"),
                                                     (16, "mixed", "rotate"),
                                                     (6, "mixed", "kkylin")])
def test_forest_equals_alone(aran, order, precision, flavour):
    sy = systems()
    x, q, offs, boxes = concat(sy)
    kw = dict(maxbox=32, order=order, field=True, precision=precision, flavour=flavour)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), **kw) as s:
        pot, fld = s.solve_forest(x, q, offs, boxes)
        st = s.get_stats()
    tol = 1e-12 if precision == "fp64" else 1e-10
    total = dict.fromkeys(st, 0)
    for k, (xs, qs, box) in enumerate(sy):
        a, b = offs[k], offs[k + 1]
        if b == a:
            total["zero"] += 1             # its root, cleared like any node
            continue
        with aran.Solver3d(box[:3], box[3:], **kw) as s1:
            p1, f1 = s1.solve(xs, qs)
            for key, v in s1.get_stats().items():
                total[key] += v
        if b - a == 1:
            assert pot[a] == 0.0 and p1[0] == 0.0 and not fld[a].any()
            continue
        assert rel_l2(pot[a:b], p1) < tol, k
        assert rel_l2(fld[a:b], f1) < tol, k
    assert st == total


def test_forest_matches_oracle(aran, oracle):
    sy = systems()
    x, q, offs, boxes = concat(sy)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), maxbox=32, order=10, field=True,
                       precision="fp64") as s:
        pot, fld = s.solve_forest(x, q, offs, boxes)
    for k, (xs, qs, box) in enumerate(sy):
        if len(qs) < 2:
            continue
        a, b = offs[k], offs[k + 1]
        op, _ = oracle.solve(xs, qs, order=10, maxbox=32, field=False, lb=box[:3], ub=box[3:],
                             nthreads=0)
        of, _ = oracle.solve(xs, qs, order=10, maxbox=32, field=True, lb=box[:3], ub=box[3:],
                             nthreads=0)
        assert rel_l2(pot[a:b], op) < 1e-12, k
        assert rel_l2(fld[a:b], of) < 1e-12, k


def test_forest_argument_checks(aran):
    sy = systems()
    x, q, offs, boxes = concat(sy)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), maxbox=32, order=6, field=True) as s:
        bad = boxes.copy()
        bad[2, 3] += 0.5                  # extent 1.5 along x
        with pytest.raises(aran.AranError) as ei:
            s.solve_forest(x, q, offs, bad)
        assert ei.value.code == -1
        o2 = offs.copy()
        o2[3], o2[4] = o2[4], o2[3]        # decreasing
        with pytest.raises(aran.AranError):
            s.solve_forest(x, q, o2, boxes)
        with pytest.raises(ValueError):        # the C call takes n = offsets[nsys]
            s.solve_forest(x[:-1], q[:-1], offs, boxes)
        # the solver is still usable
        pot, _ = s.solve_forest(x, q, offs, boxes)
        assert np.isfinite(pot).all()
