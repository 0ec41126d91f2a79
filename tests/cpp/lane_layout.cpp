// Host check of the lane-parallel M2L stream layout (fmm_math.cuh): for
// every order it prints the section offsets, and verifies that the sections
// tile the stride, start on 16-byte boundaries, and that the forward,
// vertical and backward term enumerations the kernel walks are exactly the
// index ranges the table builder decodes.
#include <cstdio>

#include "../../aran_gb300/csrc/fmm_math.cuh"

using namespace aran;

static int fails = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAIL p=%d: %s (line %d)\n", p, #c, __LINE__);  \
      ++fails;                                                     \
    }                                                              \
  } while (0)

int main() {
  for (int p = 2; p <= 16; ++p) {
    const int F = m2l_lane_f(p), V = m2l_lane_v(p), B = m2l_lane_b(p), S = m2l_lane_stride(p);
    CHECK(F >= 2 * (p + 1));
    CHECK(F % 4 == 0 && V % 4 == 0 && B % 4 == 0 && S % 4 == 0);   // 16-byte sections
    CHECK(V - F == 8 * ((m2l_lane_nf(p) + 3) / 4));
    CHECK(B - V == 4 * ((m2l_lane_nv(p) + 3) / 4));
    CHECK(S - B == 8 * ((m2l_lane_nb(p) + 3) / 4));
    // forward / backward: lower triangles (m <= m') of degrees < p / <= p
    int t = 0;
    for (int l = 0; l < p; ++l)
      for (int mp = 0; mp <= l; ++mp)
        for (int m = 0; m <= mp; ++m, ++t) CHECK(t == m2l_lane_tet(l) + mp * (mp + 1) / 2 + m);
    CHECK(t == m2l_lane_nf(p));
    t = 0;
    for (int l = 0; l <= p; ++l)
      for (int mp = 0; mp <= l; ++mp)
        for (int m = 0; m <= mp; ++m, ++t) (void)m;
    CHECK(t == m2l_lane_nb(p));
    // vertical: per order m, the lower triangle over j, n in [m, p) and the
    // row j = p
    t = 0;
    for (int m = 0; m <= p; ++m) {
      CHECK(t == m2l_lane_vpre(p, m));
      const int k = p - m;
      t += k * (k + 1) / 2 + k;
    }
    CHECK(t == m2l_lane_nv(p));
    std::printf("p=%d f=%d v=%d b=%d stride=%d floats\n", p, F, V, B, S);
  }
  // the two orders with a kernel: the offsets the kernel was sized for
  {
    const int p = 12;
    CHECK(m2l_lane_stride(12) == 2112);
    CHECK(m2l_lane_order(8) && m2l_lane_order(12) && !m2l_lane_order(10));
  }
  std::printf(fails ? "FAILED\n" : "OK\n");
  return fails ? 1 : 0;
}
