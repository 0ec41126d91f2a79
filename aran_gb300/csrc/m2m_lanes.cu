// m2m_lanes.cu -- lane-parallel M2M and L2L for the FP32 path at the orders
// m2l_lane_order accepts (4, 8, 12).  Same operators as passes.cu's
// k_m2m_rotate and k_l2l_rotate (aran_development3d_m2m_rotate,
// arandevelopment3d.c:402-409, and aran_development3d_l2l_rotate, :444-451:
// z-phase, rotation to the z axis, translation along z --
// aran/aransphericalseriesd-translate.c:445-505 for M2M, :301-364 for L2L --
// rotation back, conjugate z-phase), with the work laid out like
// m2l_lanes.cu:
//
//  * one lane pair per parent: after the z-phase the rotation blocks and the
//    vertical factors never mix real and imaginary parts, so the even lane
//    carries the real part and the odd lane the imaginary part, and the
//    series stays in registers (the order is a compile-time constant);
//  * a CTA takes 16 parents and warp w their children of octant w.  Octant
//    o = (bx, by, bz) (bit 0 x, bit 1 y, bit 2 z) is the mirror image of
//    octant 0 (x -> -x where bx = 1, likewise y, z), so the translation obeys
//    T_o = S_o T_0 S_o with S_o the mirror's action on series: (l, m) ->
//    (-1)^{l+m} on a z flip, conjugation on a y flip, (-1)^m conjugation on
//    an x flip.  One table, octant 0's, serves every octant, and every table
//    read is a broadcast from shared memory;
//  * M2M sums the eight children's contributions in octant order through
//    shared memory and writes the parent once (as k_m2m_rotate does); L2L
//    adds the parent's translated local to each non-empty child.
#include "internal.cuh"

namespace aran {

namespace {

constexpr int kOctWarps = 8;     // warps per CTA: warp w <-> child octant w
constexpr unsigned kFull = 0xffffffffu;

__host__ __device__ constexpr int oct_tri(int k) { return k * (k + 1) / 2; }
__host__ __device__ constexpr int oct_tet(int k) { return k * (k + 1) * (k + 2) / 6; }
__host__ __device__ constexpr int oct_sq(int l) { return l * (l + 1) * (2 * l + 1) / 6; }

// Stream layout of one kind's octant-0 table (floats), DOWN = L2L:
//  * FW: the z-phases (cos, sin) of m = 0..P, padded to four floats;
//  * the forward rotation terms of degrees l < LD in the direction tables'
//    order (l, m', m), in groups of four: four even-block (real part)
//    factors, then four odd-block (imaginary part) factors;
//  * VT: the vertical factors times the octant's radial powers, per order m
//    and output degree l, over the source degrees n (M2M: n in [m, l], L2L:
//    n in [l, LD));
//  * BW: the backward rotation terms, grouped like the forward ones.
template <int P, bool DOWN>
struct OctDims {
  static constexpr int LD = DOWN ? P + 1 : P;   // degrees 0..LD-1 in and out
  static constexpr int NC = oct_tri(LD);        // coefficients
  static constexpr int NR = oct_sq(LD);         // rotation terms, sum of (l+1)^2
  static constexpr int NV = oct_tet(LD);        // vertical terms
  static constexpr int FW = (2 * (P + 1) + 3) & ~3;
  static constexpr int VT = FW + 8 * ((NR + 3) / 4);
  static constexpr int BW = VT + 4 * ((NV + 3) / 4);
  static constexpr int STRIDE = BW + 8 * ((NR + 3) / 4);
};

// index of the vertical term (order m, output degree l, source degree n)
__host__ __device__ constexpr int oct_vidx(int LD, bool down, int m, int l, int n) {
  return oct_tet(LD) - oct_tet(LD - m) +
         (down ? oct_tri(LD - m) - oct_tri(LD - l) + (n - l) : oct_tri(l - m) + (n - m));
}

__device__ __forceinline__ float sel4(const float4 &v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

// the stream table of one kind from octant 0's FP32 direction table (layout
// of tables.cu, kind 1 or 2) and the vertical factors (vm or vl)
__global__ void k_oct_lane_tables(int p, int down, const float *__restrict__ dir, int ef, int of,
                                  int ei, int oi, int ph, int rp, const float *__restrict__ vert,
                                  float *__restrict__ dst) {
  const int LD = down ? p + 1 : p;
  const int NR = oct_sq(LD), NV = oct_tet(LD);
  const int FW = (2 * (p + 1) + 3) & ~3;
  const int VT = FW + 8 * ((NR + 3) / 4), BW = VT + 4 * ((NV + 3) / 4);
  const int stride = BW + 8 * ((NR + 3) / 4);
  for (int e = threadIdx.x; e < stride; e += blockDim.x) {
    float v = 0.f;
    if (e < FW) {
      if (e < 2 * (p + 1)) v = dir[ph + e];
    } else if (e < VT || e >= BW) {
      const int q = e < VT ? e - FW : e - BW;
      const int t = 4 * (q >> 3) + (q & 3), part = (q >> 2) & 1;
      // term t of the (l, m', m) order sits at sq_off(l) + m' (l+1) + m = t
      if (t < NR) v = dir[(e < VT ? (part ? of : ef) : (part ? oi : ei)) + t];
    } else if (e - VT < NV) {
      const int t = e - VT;
      for (int m = 0; m < LD; ++m)
        for (int l = m; l < LD; ++l) {
          const int n0 = down ? l : m, n1 = down ? LD - 1 : l;
          for (int n = n0; n <= n1; ++n)
            if (oct_vidx(LD, down != 0, m, l, n) == t)
              v = down ? vert[oct_tri(l) * (p + 1) + m * (p + 1) + n] * dir[rp + n - l]
                       : vert[(oct_tri(l) + m) * p + n] * dir[rp + l - n];
        }
    }
    dst[e] = v;
  }
}

// The CTA's 16 parents are list[16 b .. 16 b + 16) (the level's internal
// nodes), or without a list the nodes off + 16 b onwards; lane pair i of
// every warp takes parent i and warp w its child octant w.  DOWN = false
// (M2M): each parent gets the sum of its children's translated multipoles,
// added in octant order.  DOWN = true (L2L): each non-empty child gets its
// parent's translated local added.
template <int P, bool DOWN>
__global__ void __launch_bounds__(32 * kOctWarps, 1)
    k_oct_lanes(int cnt, int off, const int *__restrict__ list, const int *__restrict__ child,
                const int *__restrict__ begin, const int *__restrict__ end,
                const float *__restrict__ tab_g, cplx<float> *__restrict__ ser) {
  using D = OctDims<P, DOWN>;
  constexpr int LD = D::LD, NC = D::NC;
  __shared__ __align__(16) float tab[D::STRIDE];
  __shared__ int s_par[16];
  // M2M: each warp's translated multipoles, [warp][coefficient][lane]
  extern __shared__ float part_raw[];
  for (int i = threadIdx.x; i < D::STRIDE; i += blockDim.x) tab[i] = tab_g[i];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, h = lane & 1;
  if (threadIdx.x < 16) {
    const int idx = blockIdx.x * 16 + threadIdx.x;
    int par = -1;
    if (idx < cnt) {
      par = list ? list[idx] : off + idx;
      if (child[par] < 0) par = -1;
    }
    s_par[threadIdx.x] = par;
  }
  __syncthreads();
  const int par = s_par[lane >> 1];
  const int ch = par >= 0 ? child[par] + w : -1;
  const bool live = ch >= 0 && end[ch] > begin[ch];
  float *part = part_raw + (size_t)w * NC * 32 + lane;   // coefficient c at part[32 c]
  const int bx = w & 1, by = (w >> 1) & 1, bz = w >> 2;
  const float2 *ph2 = reinterpret_cast<const float2 *>(tab);
  if (__any_sync(kFull, live)) {
    const float2 *x =
        reinterpret_cast<const float2 *>(ser + (size_t)(live ? (DOWN ? par : ch) : 0) * NC);
    // mirror S_w, z-phase and rotation to the z axis: this lane's part of the
    // phased mirrored input (l, m) is sn (x.re pa[m] + x.im pb[m])
    float y[NC];
    {
      float pa[LD], pb[LD];
#pragma unroll
      for (int m = 0; m < LD; ++m) {
        const float2 e = ph2[m];
        const float g = ((bx ^ bz) & m & 1) ? -1.f : 1.f;   // (-1)^m of x and z flips
        const float cj = (bx ^ by) ? -g : g;                 // conjugation
        pa[m] = g * (h ? e.y : e.x);
        pb[m] = cj * (h ? e.x : -e.y);
      }
      const float4 *F4 = reinterpret_cast<const float4 *>(tab + D::FW) + h;
      float4 fq = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int l = 0; l < LD; ++l) {
        const float sn = (bz && (l & 1)) ? -1.f : 1.f;
        float xp[LD];
#pragma unroll
        for (int m = 0; m <= l; ++m) {
          const float2 v = live ? __ldg(x + oct_tri(l) + m) : make_float2(0.f, 0.f);
          xp[m] = sn * fmaf(v.x, pa[m], v.y * pb[m]);
        }
#pragma unroll
        for (int mp = 0; mp <= l; ++mp) {
          float acc = 0.f;
#pragma unroll
          for (int m = 0; m <= l; ++m) {
            const int t = oct_sq(l) + mp * (l + 1) + m;
            if ((t & 3) == 0) fq = F4[2 * (t >> 2)];
            acc = fmaf(sel4(fq, t & 3), xp[m], acc);
          }
          y[oct_tri(l) + mp] = acc;
        }
      }
    }
    // translation along z, order by order (real factors, both parts alike;
    // the factors are read four at a time in the order they are stored)
    float z[NC];
    {
      const float4 *V4 = reinterpret_cast<const float4 *>(tab + D::VT);
      float4 vq = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int m = 0; m < LD; ++m)
#pragma unroll
        for (int l = m; l < LD; ++l) {
          float acc = 0.f;
          const int n0 = DOWN ? l : m, n1 = DOWN ? LD - 1 : l;
#pragma unroll
          for (int n = n0; n <= n1; ++n) {
            const int t = oct_vidx(LD, DOWN, m, l, n);
            if ((t & 3) == 0) vq = V4[t >> 2];
            acc = fmaf(sel4(vq, t & 3), y[oct_tri(n) + m], acc);
          }
          z[oct_tri(l) + m] = acc;
        }
    }
    // rotation back, conjugate z-phase, mirror S_w on the way out
    const float4 *B4 = reinterpret_cast<const float4 *>(tab + D::BW) + h;
    float4 bq = make_float4(0.f, 0.f, 0.f, 0.f);
    const float hs = h ? -1.f : 1.f;
    float *dst = reinterpret_cast<float *>(ser) + (size_t)(live ? ch : 0) * NC * 2 + h;
#pragma unroll
    for (int l = 0; l < LD; ++l) {
      float ol[LD];
#pragma unroll
      for (int mp = 0; mp <= l; ++mp) {
        float acc = 0.f;
#pragma unroll
        for (int m = 0; m <= l; ++m) {
          const int t = oct_sq(l) + mp * (l + 1) + m;
          if ((t & 3) == 0) bq = B4[2 * (t >> 2)];
          acc = fmaf(sel4(bq, t & 3), z[oct_tri(l) + m], acc);
        }
        ol[mp] = acc;
      }
#pragma unroll
      for (int mp = 0; mp <= l; ++mp) {
        // conjugate z-phase of octant 0: real part a cos + b sin, imaginary
        // part a cos - b sin, a this lane's part, b the partner's
        const float a = ol[mp];
        const float b = __shfl_xor_sync(kFull, a, 1);
        const float2 e = ph2[mp];
        float v = fmaf(a, e.x, b * (hs * e.y));
        const bool neg = ((bz & (l + mp)) ^ (bx & mp) ^ (h & (bx ^ by))) & 1;
        v = neg ? -v : v;
        if (DOWN) {
          if (live) dst[2 * (oct_tri(l) + mp)] += v;
        } else {
          part[32 * (oct_tri(l) + mp)] = live ? v : 0.f;
        }
      }
    }
  } else if (!DOWN) {
#pragma unroll 4
    for (int c = 0; c < NC; ++c) part[32 * c] = 0.f;
  }
  if (!DOWN) {
    // the parents' multipoles: the eight octants' parts summed in order
    __syncthreads();
    for (int i = threadIdx.x; i < NC * 32; i += blockDim.x) {
      const int c = i >> 5, ln = i & 31;
      const int pp = s_par[ln >> 1];
      if (pp < 0) continue;
      float acc = 0.f;
#pragma unroll
      for (int k = 0; k < 8; ++k) acc += part_raw[(size_t)k * NC * 32 + i];
      reinterpret_cast<float *>(ser)[((size_t)pp * NC + c) * 2 + (ln & 1)] = acc;
    }
  }
}

template <int P, bool DOWN>
void launch_levels(AranGpuSolver3d *s, const float *tab, cplx<float> *ser, int d0, int d1,
                   cudaStream_t st) {
  DevTree &t = s->tree;
  constexpr size_t sm = DOWN ? 0 : (size_t)kOctWarps * OctDims<P, DOWN>::NC * 32 * sizeof(float);
  smem_opt_in(k_oct_lanes<P, DOWN>, sm + sizeof(float) * OctDims<P, DOWN>::STRIDE);
  // M2M: parent depths d0 down to d1; L2L: parent depths d0 up to d1.  The
  // internal nodes of depth >= 1 sit in the parents list in node order, so
  // those of depth d are a slice of it; depth 0 (the systems' roots) goes
  // by node range
  std::vector<int> first(t.nlevels + 1, 0);
  for (int d = 1; d < t.nlevels; ++d)
    first[d + 1] = first[d] + (d < (int)t.level_internal.size() ? t.level_internal[d] : 0);
  for (int d = d0; DOWN ? d <= d1 : d >= d1; DOWN ? ++d : --d) {
    if (d < 0 || d > t.nlevels - 2 || t.level_internal[d] == 0) continue;
    const int off = t.level_off[d];
    const int cnt = d == 0 ? t.level_off[1] - off
                           : std::min(t.level_internal[d], t.n_parents - first[d]);
    if (cnt <= 0) continue;
    const int *list = d == 0 ? nullptr : t.parents.ptr + first[d];
    k_oct_lanes<P, DOWN><<<ceil_div(cnt, 16), 32 * kOctWarps, sm, st>>>(
        cnt, off, list, t.child.ptr, t.begin.ptr, t.end.ptr, tab, ser);
    ACHECK(cudaGetLastError());
    s->launches++;
  }
}

}  // namespace

void build_oct_lane_tables(OpTables<float> &tb, cudaStream_t st) {
  const int p = tb.p;
  if (!m2l_lane_order(p)) return;
  for (int down = 0; down < 2; ++down) {
    const int LD = down ? p + 1 : p;
    const int NR = oct_sq(LD), NV = oct_tet(LD);
    const int FW = (2 * (p + 1) + 3) & ~3;
    const int stride = FW + 8 * ((NR + 3) / 4) + 4 * ((NV + 3) / 4) + 8 * ((NR + 3) / 4);
    const int kind = down ? 2 : 1;
    DBuf<float> &dst = tb.oct_lanes[down];
    dst.reserve(stride);
    k_oct_lane_tables<<<1, 256, 0, st>>>(
        p, down, down ? tb.dir_l2l.ptr : tb.dir_m2m.ptr, dir_offset(p, kind, 0),
        dir_offset(p, kind, 1), dir_offset(p, kind, 2), dir_offset(p, kind, 3),
        dir_offset(p, kind, 4), dir_offset(p, kind, 5), down ? tb.vl.ptr : tb.vm.ptr, dst.ptr);
    ACHECK(cudaGetLastError());
  }
}

bool launch_m2m_lanes(AranGpuSolver3d *s, OpTables<float> &tb, cplx<float> *mult, int dhi,
                      int dlo, cudaStream_t st) {
  if (!m2l_lane_order(tb.p) || tb.oct_lanes[0].ptr == nullptr) return false;
  switch (tb.p) {
    case 4: launch_levels<4, false>(s, tb.oct_lanes[0].ptr, mult, dhi, dlo, st); return true;
    case 8: launch_levels<8, false>(s, tb.oct_lanes[0].ptr, mult, dhi, dlo, st); return true;
    case 12: launch_levels<12, false>(s, tb.oct_lanes[0].ptr, mult, dhi, dlo, st); return true;
    default: return false;
  }
}

// child depths dlo (at least 3) up to dhi
bool launch_l2l_lanes(AranGpuSolver3d *s, OpTables<float> &tb, cplx<float> *loc, int dlo,
                      int dhi, cudaStream_t st) {
  if (!m2l_lane_order(tb.p) || tb.oct_lanes[1].ptr == nullptr) return false;
  const int d0 = (dlo < 3 ? 3 : dlo) - 1, d1 = dhi - 1;
  switch (tb.p) {
    case 4: launch_levels<4, true>(s, tb.oct_lanes[1].ptr, loc, d0, d1, st); return true;
    case 8: launch_levels<8, true>(s, tb.oct_lanes[1].ptr, loc, d0, d1, st); return true;
    case 12: launch_levels<12, true>(s, tb.oct_lanes[1].ptr, loc, d0, d1, st); return true;
    default: return false;
  }
}

}  // namespace aran
