"""2D Cauchy-kernel FMM on the GPU against the oracle.

* the reference's own end-to-end cases (tests/dummypot.at: circle and random
  distributions, p = 20 / 40, maxbox 1 / 10) meet their error limits against
  the direct sum, match the oracle's FMM to FP64 rounding, and reproduce its
  call counters exactly (same quadtree, same near/far lists);
* a forest of systems (different sizes and boxes, empty and one-particle
  systems included) gives, bit for bit, what each system gives alone, and
  matches the oracle system by system;
* a C4-shaped batch (many systems, N log-uniform, p = 20) against the oracle
  on sampled systems and the direct sum on sampled targets;
* device pointers give the host-pointer result; bad arguments are refused.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

COUNTERS = ("zero", "p2p", "p2m", "m2m", "m2l", "l2l", "l2p")


def circle(n, r=0.9):
    t = 2 * np.pi * np.arange(n) / n
    return np.stack([r * np.cos(t), r * np.sin(t)], 1)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


DUMMYPOT_AT = [
    ("circle", 12, 20, 1, 1e-6),
    ("circle", 2400, 20, 1, 1e-6),
    ("circle", 240, 40, 1, 1e-8),
    ("random", 240, 20, 1, 1e-6),
    ("circle", 240, 20, 10, 1e-8),
    ("circle", 2400, 20, 10, 1e-6),
]


@pytest.mark.parametrize("dist,n,order,maxbox,tol", DUMMYPOT_AT)
def test_dummypot_cases(aran, oracle, dist, n, order, maxbox, tol):
    xy = circle(n) if dist == "circle" else np.random.default_rng(0).uniform(-0.9, 0.9, (n, 2))
    q = np.ones(n)
    with aran.Solver2d(maxbox=maxbox, order=order) as s:
        acc = s.solve(xy, q)
        st = s.get_stats()
    ref = oracle.direct2d(xy, q)
    err = np.abs(acc - ref) / np.maximum(np.abs(acc), np.abs(ref))
    assert err.max() < tol
    oacc, ost = oracle.solve2d(xy, q, [0, n], [[-1, -1, 1, 1]], maxbox, order)
    assert rel_l2(acc, oacc) < 1e-12
    for k in COUNTERS:
        assert st[k] == ost[k], k


def forest(seed, sizes, order=20, maxbox=16):
    rng = np.random.default_rng(seed)
    xy, q, boxes = [], [], []
    for n in sizes:
        lo = rng.uniform(-5, 5, 2)
        ext = rng.uniform(0.1, 4.0)
        xy.append(lo + ext * rng.uniform(0, 1, (n, 2)))
        q.append(rng.uniform(-1, 1, n))
        boxes.append([lo[0], lo[1], lo[0] + ext, lo[1] + ext])
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    return np.concatenate(xy), np.concatenate(q), offs, np.array(boxes)


def test_forest_equals_systems_alone_and_oracle(aran, oracle):
    sizes = [3000, 0, 1, 2, 700, 5000, 64, 0, 1500]
    xy, q, offs, boxes = forest(11, sizes)
    with aran.Solver2d(maxbox=16, order=20) as s:
        acc = s.solve(xy, q, offs, boxes)
        st = s.get_stats()
        for i in range(len(sizes)):
            a, b = offs[i], offs[i + 1]
            if b == a:
                continue
            alone = s.solve(xy[a:b], q[a:b], [0, b - a], boxes[i:i + 1])
            np.testing.assert_array_equal(acc[a:b], alone)
    oacc, ost = oracle.solve2d(xy, q, offs, boxes, 16, 20)
    assert rel_l2(acc, oacc) < 1e-12
    for k in COUNTERS:
        assert st[k] == ost[k], k


def test_c4_batch(aran, oracle):
    rng = np.random.default_rng(4)
    nsys = 96
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(3e4), nsys)).astype(int)
    xy = rng.uniform(-1, 1, (sizes.sum(), 2))
    q = rng.uniform(-1, 1, sizes.sum())
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    boxes = np.tile([-1.0, -1.0, 1.0, 1.0], (nsys, 1))
    with aran.Solver2d(maxbox=32, order=20) as s:
        acc = s.solve(xy, q, offs, boxes)
    for i in rng.choice(nsys, 4, replace=False):
        a, b = offs[i], offs[i + 1]
        oacc, _ = oracle.solve2d(xy[a:b], q[a:b], [0, b - a], boxes[i:i + 1], 32, 20)
        assert rel_l2(acc[a:b], oacc) < 1e-12
        tgt = rng.choice(b - a, min(500, b - a), replace=False).astype(np.int32)
        ref = oracle.direct2d(xy[a:b], q[a:b], tgt)
        # truncation error of p = 20 at leaf 32 (rel-L2 about 1.5e-9 here);
        # per particle the reference's own limit (tests/dummypot.c) is 1e-6
        assert rel_l2(acc[a:b][tgt], ref) < 1e-8
        got = acc[a:b][tgt]
        assert (np.abs(got - ref) / np.maximum(np.abs(got), np.abs(ref))).max() < 1e-6


def test_device_pointers(aran):
    torch = pytest.importorskip("torch")
    xy, q, offs, boxes = forest(5, [4000, 2500])
    with aran.Solver2d(maxbox=32, order=16) as s:
        host = s.solve(xy, q, offs, boxes)
        dxy = torch.from_numpy(xy).cuda()
        dq = torch.from_numpy(q).cuda()
        dacc = torch.empty(2 * len(q), dtype=torch.float64, device="cuda")
        s.solve_device(len(q), dxy.data_ptr(), dq.data_ptr(), dacc.data_ptr(), offs, boxes)
        torch.cuda.synchronize()
        dev = dacc.cpu().numpy().view(np.complex128)
    np.testing.assert_array_equal(dev, host)


def test_bad_arguments(aran):
    with aran.Solver2d(maxbox=8, order=10) as s:
        xy = np.zeros((4, 2))
        q = np.ones(4)
        for offs, boxes in (([0, 5], None), ([1, 4], None), ([0, 3, 2, 4], None),
                            ([0, 4], [[0, 0, 0, 1]])):
            with pytest.raises(aran.AranError) as ei:
                s.solve(xy, q, offs, boxes)
            assert ei.value.code == -1


def test_c4_batch_mixed(aran, oracle):
    """Mixed precision 2D (FP32 expansions scaled by the node size, FP32
    near-field arithmetic on FP64 differences, FP64 sums) on the C4 batch
    shape: same forest and counters as FP64, results within 2e-6 (rel-L2) of
    the FP64 solve and of the direct sum."""
    rng = np.random.default_rng(4)
    nsys = 96
    sizes = np.exp(rng.uniform(np.log(1e3), np.log(3e4), nsys)).astype(int)
    xy = rng.uniform(-1, 1, (sizes.sum(), 2))
    q = rng.uniform(-1, 1, sizes.sum())
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    boxes = np.tile([-1.0, -1.0, 1.0, 1.0], (nsys, 1))
    with aran.Solver2d(maxbox=32, order=20) as s:
        a64 = s.solve(xy, q, offs, boxes)
        st64 = s.get_stats()
    with aran.Solver2d(maxbox=32, order=20, precision="mixed") as s:
        a32 = s.solve(xy, q, offs, boxes)
        st32 = s.get_stats()
    assert st32 == st64
    e = rel_l2(a32, a64)
    print("mixed vs fp64 rel-L2", e)
    assert e < 2e-6
    worst = 0.0
    for i in rng.choice(nsys, 4, replace=False):
        a, b = offs[i], offs[i + 1]
        tgt = rng.choice(b - a, min(500, b - a), replace=False).astype(np.int32)
        ref = oracle.direct2d(xy[a:b], q[a:b], tgt)
        got = a32[a:b][tgt]
        assert rel_l2(got, ref) < 2e-6
        worst = max(worst, (np.abs(got - ref) / np.maximum(np.abs(got), np.abs(ref))).max())
    print("mixed per-particle worst", worst)
    assert worst < 1e-4


def test_mixed_forest_systems_and_boxes(aran):
    """Mixed precision with systems of different box sizes and origins (the
    node scale follows each system's box) and empty or one-point systems."""
    sizes = [3000, 0, 1, 2, 700, 5000, 64, 0, 1500]
    xy, q, offs, boxes = forest(11, sizes)
    with aran.Solver2d(maxbox=16, order=20) as s:
        a64 = s.solve(xy, q, offs, boxes)
    with aran.Solver2d(maxbox=16, order=20, precision="mixed") as s:
        a32 = s.solve(xy, q, offs, boxes)
    for i in range(len(sizes)):
        a, b = offs[i], offs[i + 1]
        if b - a < 2:
            continue
        assert rel_l2(a32[a:b], a64[a:b]) < 2e-6, i


def test_input_checks_2d(aran):
    """The 2D key pass refuses a NaN coordinate (both precisions) and, in
    mixed precision, a point outside its system's box, whose key is clamped
    into a boundary cell (FP64 evaluates it there); a refused solve writes
    nothing and leaves the solver usable."""
    rng = np.random.default_rng(9)
    xy = rng.uniform(-1, 1, (4000, 2))
    q = rng.uniform(-1, 1, 4000)
    offs = np.array([0, 4000], dtype=np.int64)
    boxes = np.array([[-1.0, -1.0, 1.0, 1.0]])
    for prec in ("fp64", "mixed"):
        with aran.Solver2d(maxbox=32, order=12, precision=prec) as s:
            ref = s.solve(xy, q, offs, boxes)
            bad = xy.copy()
            bad[5, 0] = np.nan
            with pytest.raises(aran.AranError) as ei:
                s.solve(bad, q, offs, boxes)
            assert ei.value.code == -1
            out = xy.copy()
            out[7] = (1.5, 0.0)
            if prec == "mixed":
                with pytest.raises(aran.AranError) as ei:
                    s.solve(out, q, offs, boxes)
                assert ei.value.code == -1
            else:
                assert np.isfinite(s.solve(out, q, offs, boxes)).all()
            assert rel_l2(s.solve(xy, q, offs, boxes), ref) < 1e-12
