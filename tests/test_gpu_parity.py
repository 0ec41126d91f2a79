"""GPU path against the oracle, through the C ABI (libaran_gpu.so).

* tree, far (M2L) and near (P2P) lists and the permutation: bit-exact;
* call counters of aran_solver3d_get_stats: equal;
* FP64 path: potential/field within 1e-12 (rel-L2) of the oracle FMM with
  the same tree and operators (only summation order differs);
* mixed path: within 3e-6 (rel-L2) of the oracle FMM;
* both: within the FMM truncation error of the FP64 direct sum.
"""
import numpy as np
import pytest

from aran_gb300 import workloads as W

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
MIXED_TOL = 3e-6


def unordered(pairs):
    return set(map(tuple, np.sort(np.asarray(pairs, dtype=np.uint64), axis=1).tolist()))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def check_lists(s, oracle, x, maxbox, lb, ub, max_depth=21):
    g = s.tree_lists()
    o = oracle.tree_lists(x, maxbox=maxbox, lb=lb, ub=ub, max_depth=max_depth)
    gi = {int(i): (int(b), int(e), int(l)) for i, b, e, l in zip(g["ids"], g["begin"], g["end"], g["leaf"])}
    oi = {int(i): (int(b), int(e), int(l)) for i, b, e, l in zip(o["ids"], o["begin"], o["end"], o["leaf"])}
    assert gi == oi
    far_g = g["far"]
    assert len(far_g) == 2 * len(o["far"])  # directed vs unordered
    assert unordered(far_g) == set(map(tuple, o["far"].tolist()))
    assert unordered(g["near"]) == set(map(tuple, o["near"].tolist()))
    assert np.array_equal(g["perm"], o["perm"])


def cluster_beside_sparse(n, seed=16):
    """93 % of the points in a cube of side 0.05 at the centre, the rest
    uniform: coarse leaves touch the cluster's deep subtree, so near ranges
    of more than 2,048 points (the chunked P2P pass) occur.  (Dense enough
    for that, sparse enough that no pair falls inside the field kernel's
    |r| <= 1e-5 guard, which the potential-only oracle solve does not have.)"""
    rng = np.random.default_rng(seed)
    k = int(n * 0.93)
    x = np.concatenate([0.5 + rng.uniform(-0.025, 0.025, (k, 3)), rng.uniform(0, 1, (n - k, 3))])
    q = rng.uniform(-1, 1, n)
    return x, q


CASES = [
    # name, generator, n, maxbox, p, lb, ub
    ("uniform", lambda n: W.uniform(n, 11), 6000, 20, 8, (0, 0, 0), (1, 1, 1)),
    ("uniform-p12", lambda n: W.uniform(n, 12), 20000, 64, 12, (0, 0, 0), (1, 1, 1)),
    ("plummer", lambda n: W.plummer(n, 13), 20000, 32, 10, (-1, -1, -1), (1, 1, 1)),
    ("blobs", lambda n: W.blobs(n, 14, nblobs=3), 15000, 24, 8, (0, 0, 0), (1, 1, 1)),
    ("circle-maxbox1", lambda n: W.circle(n), 240, 1, 12, (-1, -1, -1), (1, 1, 1)),
    ("box-aspect", lambda n: W.uniform(n, 15), 8000, 16, 8, (0, 0, 0), (1.0, 1.5, 3.0)),
    ("cluster-heavy-ranges", cluster_beside_sparse, 30000, 16, 8, (0, 0, 0), (1, 1, 1)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_fp64_matches_oracle(aran, oracle, case):
    name, gen, n, maxbox, p, lb, ub = case
    x, q = gen(n)
    with aran.Solver3d(lb, ub, maxbox=maxbox, order=p, field=True, precision="fp64") as s:
        pot, fld = s.solve(x, q)
        check_lists(s, oracle, x, maxbox, lb, ub)
        st = s.get_stats()
    opot, ost = oracle.solve(x, q, order=p, maxbox=maxbox, field=False, lb=lb, ub=ub)
    ofld, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=True, lb=lb, ub=ub)
    assert rel_l2(pot, opot) < FP64_TOL
    assert rel_l2(fld, ofld) < FP64_TOL
    assert st == ost


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_mixed_matches_oracle(aran, oracle, case):
    name, gen, n, maxbox, p, lb, ub = case
    x, q = gen(n)
    with aran.Solver3d(lb, ub, maxbox=maxbox, order=p, field=True, precision="mixed") as s:
        pot, fld = s.solve(x, q)
        check_lists(s, oracle, x, maxbox, lb, ub)
    opot, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=False, lb=lb, ub=ub)
    ofld, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=True, lb=lb, ub=ub)
    assert rel_l2(pot, opot) < MIXED_TOL
    assert rel_l2(fld, ofld) < MIXED_TOL


M2L_KERNEL_CASES = [
    ("plummer-p12", lambda n: W.plummer(n, 31), 40000, 32, 12, (-1, -1, -1), (1, 1, 1)),
    ("uniform-p8", lambda n: W.uniform(n, 32), 30000, 16, 8, (0, 0, 0), (1, 1, 1)),
    ("uniform-p4", lambda n: W.uniform(n, 34), 30000, 16, 4, (0, 0, 0), (1, 1, 1)),
    ("blobs-p12", lambda n: W.blobs(n, 33, nblobs=2), 9000, 8, 12, (0, 0, 0), (1, 1, 1)),
]


@pytest.mark.parametrize("case", M2L_KERNEL_CASES, ids=[c[0] for c in M2L_KERNEL_CASES])
def test_mixed_m2l_kernels_agree(aran, oracle, case, monkeypatch):
    """The FP32 lane-parallel M2L kernel (orders 4, 8 and 12) and the sibling
    kernel (every order; ARAN_M2L_KERNEL=sibling) apply the same tables in
    FP32: both within the mixed tolerance of the oracle, and within 1e-6 of
    each other."""
    name, gen, n, maxbox, p, lb, ub = case
    x, q = gen(n)
    out = {}
    for kernel in ("lanes", "sibling"):
        monkeypatch.setenv("ARAN_M2L_KERNEL", kernel)
        with aran.Solver3d(lb, ub, maxbox=maxbox, order=p, field=True, precision="mixed") as s:
            out[kernel] = s.solve(x, q)
    monkeypatch.delenv("ARAN_M2L_KERNEL")
    opot, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=False, lb=lb, ub=ub)
    ofld, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=True, lb=lb, ub=ub)
    for kernel, (pot, fld) in out.items():
        assert rel_l2(pot, opot) < MIXED_TOL, kernel
        assert rel_l2(fld, ofld) < MIXED_TOL, kernel
    assert rel_l2(out["lanes"][0], out["sibling"][0]) < 1e-6
    assert rel_l2(out["lanes"][1], out["sibling"][1]) < 1e-6


TC_CASES = [c for c in M2L_KERNEL_CASES if c[4] in (8, 12)]


@pytest.mark.parametrize("case", TC_CASES, ids=[c[0] for c in TC_CASES])
def test_tensor_core_m2l(aran, oracle, case, monkeypatch):
    """The tcgen05 M2L (ARAN_M2L_KERNEL=tc, orders 8 and 12) applies the same
    operator as dense TF32 products with a hi/lo split, its accumulator
    drained into FP32 registers after every offset.  Its results stay within
    2e-6 of the lane-parallel kernel's (measured 6-7e-7: the dropped lo*lo
    product and the tensor core's accumulation within one offset) and within
    the mixed tolerance of the oracle's FP64 solve."""
    name, gen, n, maxbox, p, lb, ub = case
    x, q = gen(n)
    out = {}
    for kernel in ("lanes", "tc"):
        monkeypatch.setenv("ARAN_M2L_KERNEL", kernel)
        with aran.Solver3d(lb, ub, maxbox=maxbox, order=p, field=True, precision="mixed") as s:
            out[kernel] = s.solve(x, q)
            out[kernel + "_stats"] = s.get_stats()
    monkeypatch.delenv("ARAN_M2L_KERNEL")
    assert rel_l2(out["tc"][0], out["lanes"][0]) < 2e-6
    assert rel_l2(out["tc"][1], out["lanes"][1]) < 2e-6
    assert out["tc_stats"] == out["lanes_stats"]
    opot, _ = oracle.solve(x, q, order=p, maxbox=maxbox, field=False, lb=lb, ub=ub)
    assert rel_l2(out["tc"][0], opot) < MIXED_TOL


@pytest.mark.parametrize("p", [4, 8, 12])
def test_potential_only_matches_field_solve(aran, oracle, p):
    """At the orders with lane-parallel FP32 kernels the potential-only solve
    runs its own variants (the windowed L2P without the gradient locals, the
    near field without the field terms): its potential equals the full
    solve's to FP32 rounding, and both stay within the mixed tolerance of
    the oracle."""
    x, q = W.plummer(30000, 40 + p)
    lb, ub = (-1, -1, -1), (1, 1, 1)
    with aran.Solver3d(lb, ub, maxbox=32, order=p, field=False, precision="mixed") as s:
        pot_only, none = s.solve(x, q)
    assert none is None
    with aran.Solver3d(lb, ub, maxbox=32, order=p, field=True, precision="mixed") as s:
        pot, _ = s.solve(x, q)
    assert rel_l2(pot_only, pot) < 1e-7
    opot, _ = oracle.solve(x, q, order=p, maxbox=32, field=False, lb=lb, ub=ub)
    assert rel_l2(pot_only, opot) < MIXED_TOL


def test_points_outside_the_box(aran, oracle):
    """A point outside the solver's box: the key clamps it into a boundary
    cell (the oracle's contract), so an FP64 solve still equals the oracle;
    a mixed solve refuses the input (the point's distance from its cell would
    overflow the scaled FP32 expansions) with ARAN_ERR_INVALID and writes no
    output, and the solver stays usable.  Points on the upper bound are
    inside."""
    x, q = W.uniform(5000, 77)
    x[0] = (1.5, 0.5, 0.5)
    x[1] = (1.0, 1.0, 1.0)
    with aran.Solver3d(maxbox=32, order=8, field=False, precision="fp64") as s:
        pot, _ = s.solve(x, q)
    opot, _ = oracle.solve(x, q, order=8, maxbox=32, field=False)
    assert rel_l2(pot, opot) < FP64_TOL
    with aran.Solver3d(maxbox=32, order=8, field=False, precision="mixed") as s:
        with pytest.raises(aran.AranError) as ei:
            s.solve(x, q)
        assert ei.value.code == -1
        x[0] = (0.5, 0.5, 0.5)
        pot, _ = s.solve(x, q)
    opot, _ = oracle.solve(x, q, order=8, maxbox=32, field=False)
    assert rel_l2(pot, opot) < MIXED_TOL


@pytest.mark.parametrize("p", [1, 2, 4, 6, 16, 20])
def test_orders_fp64(aran, oracle, p):
    x, q = W.uniform(4000, 20 + p)
    with aran.Solver3d(maxbox=24, order=p, field=True, precision="fp64") as s:
        pot, fld = s.solve(x, q)
    opot, _ = oracle.solve(x, q, order=p, maxbox=24, field=False)
    ofld, _ = oracle.solve(x, q, order=p, maxbox=24, field=True)
    assert rel_l2(pot, opot) < FP64_TOL
    assert rel_l2(fld, ofld) < FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_p12_against_direct_sum(aran, oracle, precision):
    """p=12 on a uniform cube against the FP64 direct sum.  Here the
    truncation error of the expansion itself (the oracle's FP64 solve) is
    1.43e-6 for the potential and 5.3e-7 for the field, so the potential bound
    sits just above it and mixed precision may add at most 1.5e-7; the
    Plummer workloads (test_gpu_precision) meet 1e-6 for the potential."""
    x, q = W.uniform(30000, 2)
    with aran.Solver3d(maxbox=64, order=12, field=True, precision=precision) as s:
        pot, fld = s.solve(x, q)
    rp, rf = oracle.direct(x, q)
    assert rel_l2(pot, rp) < (1.5e-6 if precision == "fp64" else 1.6e-6)
    assert rel_l2(fld, rf) < (6e-7 if precision == "fp64" else 1e-6)


def test_single_leaf_is_direct_sum(aran, oracle):
    x, q = W.uniform(50, 5)
    with aran.Solver3d(maxbox=64, order=8, field=True, precision="fp64") as s:
        pot, fld = s.solve(x, q)
        assert s.tree_info()["nodes"] == 1
    rp, rf = oracle.direct(x, q)
    assert np.allclose(pot, rp, rtol=1e-13, atol=0)
    assert np.allclose(fld, rf, rtol=1e-12, atol=1e-12)


def test_one_particle(aran):
    with aran.Solver3d(maxbox=1, order=4, field=True) as s:
        pot, fld = s.solve(np.array([[0.3, 0.4, 0.5]]), np.array([2.0]))
    assert pot[0] == 0.0 and np.all(fld == 0.0)


def test_boundary_points_and_depth_limit(aran, oracle):
    # points on the upper faces (clamped into the last cell) and a depth limit
    rng = np.random.default_rng(9)
    x = rng.uniform(0, 1, (3000, 3))
    x[:100, 0] = 1.0
    x[100:200, 2] = 0.0
    q = rng.uniform(-1, 1, 3000)
    with aran.Solver3d(maxbox=4, order=6, field=False, precision="fp64", max_depth=4) as s:
        pot, _ = s.solve(x, q)
        check_lists(s, oracle, x, 4, (0, 0, 0), (1, 1, 1), max_depth=4)
    opot, _ = oracle.solve(x, q, order=6, maxbox=4, field=False, max_depth=4)
    assert rel_l2(pot, opot) < FP64_TOL


def test_potential_only_solver(aran, oracle):
    x, q = W.uniform(5000, 6)
    with aran.Solver3d(maxbox=32, order=8, field=False, precision="fp64") as s:
        pot, fld = s.solve(x, q)
        assert fld is None
    opot, _ = oracle.solve(x, q, order=8, maxbox=32, field=False)
    assert rel_l2(pot, opot) < FP64_TOL


def test_solver_reuse_changing_sizes(aran, oracle):
    with aran.Solver3d(maxbox=16, order=6, field=True, precision="mixed") as s:
        for n, seed in ((1000, 1), (20000, 2), (300, 3), (20000, 2)):
            x, q = W.uniform(n, seed)
            pot, fld = s.solve(x, q)
            opot, _ = oracle.solve(x, q, order=6, maxbox=16, field=False)
            assert rel_l2(pot, opot) < MIXED_TOL


def test_error_codes(aran):
    with aran.Solver3d(maxbox=8, order=4, field=False) as s:
        with pytest.raises(aran.AranError) as ei:
            s.solve(np.zeros((0, 3)), np.zeros(0))
        assert ei.value.code == -1
    with pytest.raises(aran.AranError) as ei:
        aran.Solver3d(flavour=7)
    assert ei.value.code == -1


def test_normal_flavour_matches_oracle(aran, oracle):
    # the normal flavour runs the rotation kernels: same operators, so the
    # GPU result equals the oracle's O(p^4) normal flavour to FP64 rounding
    x, q = W.uniform(6000, 11)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), maxbox=20, order=8, flavour="normal",
                       field=True, precision="fp64") as s:
        pot, fld = s.solve(x, q)
        st = s.get_stats()
    ofld, ost = oracle.solve(x, q, order=8, maxbox=20, flavour="normal", field=True)
    assert rel_l2(fld, ofld) < FP64_TOL
    assert st == ost


KK_CASES = [
    ("uniform", lambda n: W.uniform(n, 41), 6000, 20, 8, (0, 0, 0), (1, 1, 1)),
    ("plummer", lambda n: W.plummer(n, 42), 15000, 32, 12, (-1, -1, -1), (1, 1, 1)),
    ("box-aspect", lambda n: W.uniform(n, 43), 6000, 16, 6, (0, 0, 0), (1.0, 1.5, 3.0)),
    # source degrees above 16 (second lane slot of the half-warp M2L) and, in
    # FP64, fewer warps per CTA for the shared memory
    ("uniform-p20", lambda n: W.uniform(n, 44), 2500, 24, 20, (0, 0, 0), (1, 1, 1)),
    ("uniform-p28", lambda n: W.uniform(n, 45), 2500, 40, 28, (0, 0, 0), (1, 1, 1)),
]


@pytest.mark.parametrize("case", KK_CASES, ids=[c[0] for c in KK_CASES])
@pytest.mark.parametrize("precision,tol", [("fp64", FP64_TOL), ("mixed", MIXED_TOL)])
def test_kkylin_matches_oracle(aran, oracle, case, precision, tol):
    """kkylin flavour (aran_development3d_*_kkylin) against the oracle's kkylin solve.
    From order 24 the flavour's recurrence in m (cot theta factors) amplifies
    the last-bit differences of its FP64 arithmetic (a reciprocal table and a
    running radial power on the GPU, divisions and a power loop in the
    oracle): 5e-11 there (the truncation error at these orders is ~1e-10)."""
    name, gen, n, maxbox, p, lb, ub = case
    if precision == "fp64" and p >= 24:
        tol = 5e-11
    x, q = gen(n)
    if precision == "mixed" and p > 16:
        # alpha ratios up to degree 2p leave the FP32 range: refused
        with pytest.raises(aran.AranError) as ei:
            aran.Solver3d(lb, ub, maxbox=maxbox, order=p, flavour="kkylin", precision="mixed")
        assert ei.value.code == -1
        return
    with aran.Solver3d(lb, ub, maxbox=maxbox, order=p, flavour="kkylin", field=True,
                       precision=precision) as s:
        pot, fld = s.solve(x, q)
    opot, _ = oracle.solve(x, q, order=p, maxbox=maxbox, flavour="kkylin", field=False, lb=lb, ub=ub)
    ofld, _ = oracle.solve(x, q, order=p, maxbox=maxbox, flavour="kkylin", field=True, lb=lb, ub=ub)
    assert rel_l2(pot, opot) < tol
    assert rel_l2(fld, ofld) < tol


def test_linearity_and_permutation(aran):
    """Size-independent properties on 1M particles: the solve is linear in the
    charges and equivariant under a permutation of the input."""
    x, q1 = W.uniform(1_000_000, 31)
    q2 = np.random.default_rng(32).uniform(-1, 1, len(q1))
    with aran.Solver3d(maxbox=64, order=12, field=True, precision="fp64") as s:
        p1, f1 = s.solve(x, q1)
        p2, f2 = s.solve(x, q2)
        p3, f3 = s.solve(x, q1 + 2.0 * q2)
        perm = np.random.default_rng(33).permutation(len(q1))
        p4, f4 = s.solve(x[perm], q1[perm])
    assert rel_l2(p3, p1 + 2.0 * p2) < 1e-12
    assert rel_l2(f3, f1 + 2.0 * f2) < 1e-12
    assert rel_l2(p4, p1[perm]) < 1e-13
    assert rel_l2(f4, f1[perm]) < 1e-13


@pytest.fixture(scope="module")
def uniform_1m(oracle):
    x, q = W.uniform(1_000_000, 2)
    tgt = np.random.default_rng(2).choice(len(q), 10_000, replace=False)
    rp, rf = oracle.direct(x, q, targets=tgt)
    return x, q, tgt, rp, rf


@pytest.mark.parametrize("precision,tol", [("fp64", 2e-6), ("mixed", 3e-6)])
def test_1m_uniform_subset_vs_direct(aran, uniform_1m, precision, tol):
    """The uniform1m workload (N=1M uniform, p=12, leaf 64); 10,000 targets
    against the FP64 direct sum."""
    x, q, tgt, rp, rf = uniform_1m
    with aran.Solver3d(maxbox=64, order=12, field=True, precision=precision) as s:
        pot, fld = s.solve(x, q)
    assert rel_l2(pot[tgt], rp) < tol
    assert rel_l2(fld[tgt], rf) < tol


# tests/newtonpot3.at and tests/newtonfield3.at: (np, order, maxbox,
# distribution) with every flavour that runs on the GPU, FP64, per-particle
# error |acc - sum| / max(|acc|, |sum|) <= 1e-3 against the direct sum
# (tests/newtonpot3.c:680-705).  The circle has radius 0.999 in z = 0 with
# densities 1/np; "random" is uniform in [-0.999, 0.999]^3 with densities
# U[0, 2/np]; the box is [-1, 1]^3.
NEWTON_AT = [
    (12, 20, 1, "circle"),
    (24, 24, 1, "circle"),
    (24, 24, 1, "random"),
    (240, 24, 10, "circle"),
    (2400, 24, 100, "circle"),
]


def newton_points(n, dist):
    if dist == "circle":
        return W.circle(n)
    rng = np.random.default_rng(n)
    return rng.uniform(-0.999, 0.999, (n, 3)), rng.uniform(0.0, 2.0 / n, n)


@pytest.mark.parametrize("flavour", ["normal", "rotate", "kkylin"])
@pytest.mark.parametrize("n,order,maxbox,dist", NEWTON_AT)
def test_newton_at_cases(aran, oracle, flavour, n, order, maxbox, dist):
    x, q = newton_points(n, dist)
    lb, ub = (-1, -1, -1), (1, 1, 1)
    with aran.Solver3d(lb, ub, maxbox=maxbox, order=order, flavour=flavour, field=True,
                       precision="fp64") as s:
        pot, fld = s.solve(x, q)
        st = s.get_stats()
    rp, rf = oracle.direct(x, q)
    ep = np.abs(pot - rp) / np.maximum(np.abs(pot), np.abs(rp))
    nf, nr = np.linalg.norm(fld, axis=1), np.linalg.norm(rf, axis=1)
    ef = np.linalg.norm(fld - rf, axis=1) / np.maximum(np.maximum(nf, nr), 1e-300)
    assert ep.max() < 1e-3
    assert ef.max() < 1e-3
    opot, ost = oracle.solve(x, q, order=order, maxbox=maxbox, flavour=flavour, field=False,
                             lb=lb, ub=ub)
    assert rel_l2(pot, opot) < FP64_TOL
    assert st == ost


def test_order_30_mixed(aran, oracle):
    x, q = W.uniform(6000, 31)
    with aran.Solver3d((0, 0, 0), (1, 1, 1), maxbox=16, order=30, field=True,
                       precision="mixed") as s:
        pot, fld = s.solve(x, q)
    opot, _ = oracle.solve(x, q, order=30, maxbox=16, field=False, lb=(0, 0, 0), ub=(1, 1, 1))
    assert rel_l2(pot, opot) < MIXED_TOL


# semifar P2L/M2P (aran/aransolver3d.c:357-396): on a Plummer tree (coarse
# leaves next to deep subtrees) the GPU lists reproduce the oracle's counts
# exactly (fewer P2P pairs, p2l = m2p points), and the results match the
# oracle's semifar solve
@pytest.mark.parametrize("threshold", [1, 8, 64])
@pytest.mark.parametrize("field", [False, True])
def test_semifar_matches_oracle(aran, oracle, threshold, field):
    x, q = W.plummer(20000, 13)
    lb, ub = (-1, -1, -1), (1, 1, 1)
    kw = dict(maxbox=32, order=10, field=field)
    with aran.Solver3d(lb, ub, precision="fp64", semifar_threshold=threshold, **kw) as s:
        pot, fld = s.solve(x, q)
        st = s.get_stats()
    ref, ost = oracle.solve(x, q, order=10, maxbox=32, field=field, lb=lb, ub=ub,
                            semifar_threshold=threshold)
    got = fld if field else pot
    assert ost["p2l"] > 0
    for k in ("p2p", "p2l", "m2p", "m2l", "m2m", "l2l", "zero"):
        assert st[k] == ost[k], k
    assert rel_l2(got, ref) < FP64_TOL
    with aran.Solver3d(lb, ub, precision="mixed", semifar_threshold=threshold, **kw) as s:
        potm, fldm = s.solve(x, q)
    assert rel_l2(fldm if field else potm, ref) < MIXED_TOL
