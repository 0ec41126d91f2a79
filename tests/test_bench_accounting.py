"""The benchmark's roofline accounting (CPU only): the flop count of one M2L
equals the multiply-adds of the operator the GPU applies, counted term by
term as the lane kernel walks them (z-phases, forward rotation, translation
along z, backward rotation, conjugate z-phases)."""
import bench


def enumerate_macs(p):
    macs = 0
    nm, nl = p * (p + 1) // 2, (p + 1) * (p + 2) // 2
    macs += 4 * nm                      # z-phase of the source (complex product)
    for part in range(2):               # real and imaginary parts
        for l in range(p):              # forward rotation, degrees < p
            macs += (l + 1) ** 2
        for m in range(p + 1):          # translation along z, m-major slots
            for j in range(m, p + 1):
                macs += p - m
        for l in range(p + 1):          # backward rotation, degrees <= p
            macs += (l + 1) ** 2
    macs += 4 * nl                      # conjugate z-phase of the local
    return macs


def test_m2l_flops_match_enumerated_terms():
    for p in (4, 8, 12, 16, 20):
        assert bench.m2l_flops(p) == 2 * enumerate_macs(p), p
    assert bench.m2l_flops(12) == 10140


def test_rotate_operator_flops():
    """F(p) = 4 [A(p-1) + B(p) + A(p)] with A(L) = (L+1)(L+2)(4L+3)/6 (real
    Wigner-d block times complex coefficients, degrees 0..L) and
    B(p) = p(p+1)(p+2)/3 (vertical translation), enumerated term by term."""
    def a(L):
        # for each degree l <= L, (l+1) output orders m' >= 0, each a sum over
        # 2l+1 source orders m in [-l, l]
        return sum((l + 1) * (2 * l + 1) for l in range(L + 1))

    def b(p):
        # vertical M2L: local (j, m), j <= p, from multipole (n, m), n < p,
        # m <= min(j, n)
        return sum(min(j, n) + 1 for j in range(p + 1) for n in range(p))

    for p in (4, 8, 12, 16):
        assert bench.m2l_flops_rotate(p) == 4 * (a(p - 1) + b(p) + a(p)), p
    assert (bench.m2l_flops_rotate(8), bench.m2l_flops_rotate(12),
            bench.m2l_flops_rotate(16)) == (4548, 13988, 31620)


def test_m2m_l2l_p2m_l2p_flops():
    """The per-translation and per-particle counts of the other stages,
    enumerated: M2M = two real-d rotations of degrees < p (2 x 4 A(p-1)) plus
    the vertical shift of multipole (l, m) from degrees n <= l (4 per term);
    L2L the same with degrees <= p and the local shift from degrees n >= l;
    P2M 16 flops and L2P with gradient 32 flops per coefficient."""
    def a(L):
        return sum((l + 1) * (2 * l + 1) for l in range(L + 1))

    for p in (4, 8, 12, 16):
        shift_m = sum(1 for l in range(p) for m in range(l + 1))            # tri(p) outputs
        vert_m = sum(l + 1 for l in range(p))                               # (l+1)(l+2)/2 summed
        assert bench.m2m_flops_rotate(p) == 8 * a(p - 1) + 4 * sum(
            (l + 1) * (l + 2) // 2 for l in range(p)), p
        assert shift_m == p * (p + 1) // 2 and vert_m == p * (p + 1) // 2
        vert_l = sum(p - l + 1 for l in range(p + 1) for m in range(l + 1))
        assert bench.l2l_flops_rotate(p) == 8 * a(p) + 4 * vert_l, p
        assert bench.p2m_flops(p) == 16 * (p * (p + 1) // 2)
        assert bench.l2p_flops(p) == 32 * ((p + 1) * (p + 2) // 2)


def test_stage_rooflines_arithmetic():
    stage_ms = {"total": 10.0, "sort": 0.5, "tree": 0.5, "lists": 0.5, "p2p": 2.0, "m2l": 5.0,
                "m2m": 0.5, "l2l": 0.5, "p2m": 0.25, "l2p": 0.25}
    stats = {"p2p": 1_000_000, "m2m": 1000, "l2l": 1000}
    r = bench.stage_rooflines(stage_ms, stats, {"far": 100_000}, 100_000, 12, 80.0, 8000.0)
    assert r["m2l"]["ideal_ms"] == round(1e3 * 100_000 * 13988 / 80e12, 4)
    assert r["p2p"]["work"] == 40e6
    assert r["sort+tree+lists"]["measured_ms"] == 1.5
    total = sum(v["ideal_ms"] for k, v in r.items() if isinstance(v, dict))
    assert abs(r["sum_ideal_over_step"] - total / 10.0) < 1e-3


def test_m2l_kernel_name():
    """The roofline entry names the kernel the library runs for the order,
    precision and ARAN_M2L_KERNEL choice (tc serves orders 8 and 12, the
    lane kernel 4, 8 and 12 in mixed precision, the sibling kernel the
    rest)."""
    assert bench.m2l_kernel_name("mixed", 12, "").startswith("k_m2l_lanes<12>")
    assert bench.m2l_kernel_name("mixed", 12, "tc").startswith("k_m2l_tc<12>")
    assert bench.m2l_kernel_name("mixed", 4, "tc").startswith("k_m2l_lanes<4>")
    assert bench.m2l_kernel_name("mixed", 8, "sibling").startswith("k_m2l_sibling")
    assert bench.m2l_kernel_name("mixed", 16, "").startswith("k_m2l_sibling")
    assert bench.m2l_kernel_name("fp64", 12, "lanes").startswith("k_m2l_sibling")


def test_workloads_inside_their_boxes():
    """Mixed-precision solves refuse points outside the box, so every bench
    workload and batch generator stays inside the box it is solved in."""
    import numpy as np
    from aran_gb300 import workloads as W
    for name, (gen, _n, _p, _mb, lb, ub, _d) in bench.WORKLOADS.items():
        x, _q = getattr(W, gen)(20000, 3)
        assert (x >= np.array(lb)).all() and (x <= np.array(ub)).all(), name
    x, _q = W.blobs(20000, 5)
    assert (x >= 0.0).all() and (x <= 1.0).all()
    xy, _q, _offs, boxes = W.batch2d(nsys=8)
    assert (xy >= boxes[0, :2]).all() and (xy <= boxes[0, 2:]).all()
    for x, _q, _p in W.batch3d(nsys=8, nhi=5e3):
        assert (x >= 0.0).all() and (x <= 1.0).all()
