"""Virtual leaves through the C ABI (aran_gpu_solver3d_set_leaf_predicate, the
GPU side of aran_solver3d_set_nf_isleaf, aran/aransolver3d.c:1272-1279)
against the oracle's tree with the same predicate: the same nodes, far and
near pairs and counters, and the FP64 results within rounding.

The predicate here depends on position, depth and count (nodes left of
x = 0 below depth 2 stay leaves up to 200 points), so it is not a plain leaf
capacity; tests/c/solver_api.c checks the virtual-maxbox predicate of the
reference's tests/newtonfield3.c:585-595 through the LibAran API.
"""
import numpy as np
import pytest

from aran_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def pred(v):
    return v.depth >= 2 and v.center[0] < 0.0 and v.point_count <= 200


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 3e-6)])
def test_leaf_predicate_matches_oracle(aran, oracle, precision, tol):
    x, q = W.plummer(30000, 44)
    lb, ub = (-1, -1, -1), (1, 1, 1)
    with aran.Solver3d(lb, ub, maxbox=16, order=8, field=False, precision=precision) as s:
        s.set_leaf_predicate(pred)
        pot, _ = s.solve(x, q)
        st = s.get_stats()
        g = s.tree_lists()
        s.set_leaf_predicate(None)
        pot_plain, _ = s.solve(x, q)
        st_plain = s.get_stats()
    with oracle.leaf_predicate(pred):
        opot, ost = oracle.solve(x, q, order=8, maxbox=16, field=False, lb=lb, ub=ub)
        o = oracle.tree_lists(x, maxbox=16, lb=lb, ub=ub)
    assert rel_l2(pot, opot) < tol
    assert st == ost
    assert st["zero"] < st_plain["zero"]            # the tree is cut at the virtual leaves
    assert st["p2p"] > st_plain["p2p"]
    gi = {int(i): (int(b), int(e), int(l)) for i, b, e, l in
          zip(g["ids"], g["begin"], g["end"], g["leaf"])}
    oi = {int(i): (int(b), int(e), int(l)) for i, b, e, l in
          zip(o["ids"], o["begin"], o["end"], o["leaf"])}
    assert gi == oi
    far = set(map(tuple, np.sort(g["far"], axis=1).tolist()))
    assert far == set(map(tuple, o["far"].tolist()))
