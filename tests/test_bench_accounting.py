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
