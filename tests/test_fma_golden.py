"""FMA particle files and the golden fixtures of tests/golden/.

CPU: the FMA writer/reader round-trips (lossless digits, and the reference's
``%g`` form), the ``index x y z density`` list reorders by index, and the
oracle reproduces the committed golden outputs from the committed FMA file.
GPU: the solver fed from the same file matches the golden outputs.
"""
import os

import numpy as np
import pytest

from aran_gb300 import fma

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FMA_FILE = os.path.join(GOLDEN, "plummer2000.fma")


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_fma_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    x = rng.uniform(-2, 3, (50, 3))
    q = rng.uniform(0, 1, 50)
    p = tmp_path / "a.fma"
    fma.write_fma(p, x, q, (-2, -2, -2), (3, 3, 3))
    x2, q2, lb, ub = fma.read_fma(p)
    assert np.array_equal(x, x2) and np.array_equal(q, q2)
    np.testing.assert_allclose(lb, -2) and np.testing.assert_allclose(ub, 3)
    # the reference's own form: %g, 6 significant digits
    fma.write_fma(p, x, q, (-2, -2, -2), (3, 3, 3), digits=None)
    first = open(p).readline().split()
    assert first == ["50", "2.5", "0.5", "0.5", "0.5"]
    x3, _, _, _ = fma.read_fma(p)
    assert np.abs(x3 - x).max() < 1e-5 * 3


def test_point_list_reorders_by_index(tmp_path):
    p = tmp_path / "pts.txt"
    p.write_text("1 0.5 0.5 0.5 2\n0 0.1 0.2 0.3 1\n")
    x, q = fma.read_points(p)
    assert np.array_equal(q, [1.0, 2.0])
    assert np.array_equal(x[0], [0.1, 0.2, 0.3])
    p.write_text("0 0 0 0 1\n0 1 1 1 1\n")
    with pytest.raises(ValueError):
        fma.read_points(p)


def test_oracle_reproduces_golden(oracle):
    x, q, lb, ub = fma.read_fma(FMA_FILE)
    g = np.load(os.path.join(GOLDEN, "plummer2000_p10.npz"))
    pot, st = oracle.solve(x, q, order=10, maxbox=32, field=False, lb=lb, ub=ub)
    fld, _ = oracle.solve(x, q, order=10, maxbox=32, field=True, lb=lb, ub=ub)
    assert rel_l2(pot, g["pot"]) < 1e-14
    assert rel_l2(fld, g["field"]) < 1e-14
    assert [st[k] for k in oracle.STAT_NAMES] == g["stats"].tolist()
    c = np.load(os.path.join(GOLDEN, "circle240_p20.npz"))
    acc, st2 = oracle.solve2d(c["xy"], np.ones(240), [0, 240], [[-1, -1, 1, 1]], 10, 20)
    assert rel_l2(acc, c["acc"]) < 1e-14
    assert [st2[k] for k in oracle.STAT_NAMES] == c["stats"].tolist()


@pytest.mark.gpu
def test_gpu_from_fma_matches_golden(aran):
    x, q, lb, ub = fma.read_fma(FMA_FILE)
    g = np.load(os.path.join(GOLDEN, "plummer2000_p10.npz"))
    with aran.Solver3d(lb, ub, maxbox=32, order=10, field=True, precision="fp64") as s:
        pot, fld = s.solve(x, q)
        st = s.get_stats()
    assert rel_l2(fld, g["field"]) < 1e-12
    assert list(st.values()) == g["stats"].tolist()
    with aran.Solver3d(lb, ub, maxbox=32, order=10, field=False, precision="fp64") as s:
        pot, _ = s.solve(x, q)
    assert rel_l2(pot, g["pot"]) < 1e-12
    c = np.load(os.path.join(GOLDEN, "circle240_p20.npz"))
    with aran.Solver2d(maxbox=10, order=20) as s:
        acc = s.solve(c["xy"], np.ones(240))
        st2 = s.get_stats()
    assert rel_l2(acc, c["acc"]) < 1e-12
    assert list(st2.values()) == c["stats"].tolist()
