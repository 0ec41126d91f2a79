// m2l_tc.cu -- the FP32 M2L of the mixed path on the tensor cores (tcgen05,
// kind::tf32).  Same operator as m2l.cu / m2l_lanes.cu (the "point and
// shoot" translation of aran_spherical_seriesd_to_local_rotate,
// aran/aransphericalseriesd-rotate.c:165-207, applied by far_func,
// aran/aransolver3d.c:333-354), written as dense products:
//
//  * per child-0 offset d (the 189 offsets of the lanes kernel) the
//    translation of a multipole (NM complex = 2 NM reals) into a local
//    (NL complex = 2 NL reals) is a real matrix T_d, made once per solver in
//    FP64 by applying the rotation operator to unit multipoles;
//  * the other children reach T_d through the mirror images of m2l_lanes.cu:
//    T_{sigma_w d} = S_w T_d S_w with S_w a diagonal of signs, applied to
//    the gathered sources and to the accumulated locals;
//  * a CTA takes child w of 128 consecutive parents (one TMEM lane and one
//    MMA row each) and accumulates D[target][out] = sum_d sum_k
//    A_d[target][k] T_d[out][k] in tensor memory, with the multipoles of
//    the sources at offset d as A (gathered by the threads, one row each)
//    and T_d as B;
//  * FP32 accuracy from TF32 inputs: x = hi + lo with hi and lo rounded to
//    the TF32 grid (to nearest, so the tensor core's truncation of its inputs
//    is exact and unbiased), and D += A_hi B_hi + A_hi B_lo + A_lo B_hi (the
//    dropped A_lo B_lo is below FP32 rounding).
//
// Per step (one offset, 32 of the K inputs) the threads split and store
// their rows of A in the 128-byte swizzle, a TMA bulk copy brings the
// offset's pre-swizzled B (hi and lo) into a three-slot ring, and one
// thread issues 12 MMAs (M = 128, N = 16 * ceil(2 NL / 16), K = 8) whose
// completion (tcgen05.commit) frees the slots.  Every mbarrier wait is
// bounded; a wait that gives up sets the error word and the CTA drains
// what it issued, frees its tensor memory and returns.
#include <cstring>
#include <vector>

#include "internal.cuh"
#include "tcgen05.cuh"

namespace aran {


namespace {

constexpr int kTcRows = 128;   // targets per CTA = MMA M
constexpr int kTcOffsets = 189;

template <int P>
struct TcDims {
  static constexpr int NM = P * (P + 1) / 2;
  static constexpr int NL = (P + 1) * (P + 2) / 2;
  static constexpr int NIN = 2 * NM;                  // K (reals)
  static constexpr int NOUT = 2 * NL;                 // outputs (reals)
  static constexpr int NCH = (NIN + 31) / 32;         // K chunks of 32
  static constexpr int N = (NOUT + 15) / 16 * 16;     // MMA N
  static constexpr uint32_t A_BYTES = kTcRows * 128;  // one term of one step
  static constexpr uint32_t B_BYTES = N * 128;        // one term of one step
  static constexpr int ASLOTS = 2, BSLOTS = 3;
};

template <int P>
constexpr size_t tc_smem() {
  using D = TcDims<P>;
  return 1024 + (size_t)D::ASLOTS * 2 * D::A_BYTES + (size_t)D::BSLOTS * 2 * D::B_BYTES +
         (size_t)kTcRows * 27 * sizeof(int) + 256 + 64;
}

// sign of real `idx` (coefficient idx/2 in (l, m) tri order, part idx&1)
// under the mirror of child w: (l, m) -> (-1)^{l+m} on a z flip, conjugation
// on a y flip, (-1)^m conjugation on an x flip
__device__ __forceinline__ uint32_t mirror_neg(int idx, int w) {
  const int c = idx >> 1, part = idx & 1;
  int l = 0;
  while ((l + 1) * (l + 2) / 2 <= c) ++l;
  const int m = c - l * (l + 1) / 2;
  const int bx = w & 1, by = (w >> 1) & 1, bz = (w >> 2) & 1;
  return (uint32_t)(((bz & (l + m)) ^ (bx & m) ^ (part & (bx ^ by))) & 1);
}

// x rounded to the TF32 grid (10 stored significand bits), to nearest (ties
// away from zero); the tensor core then uses it exactly
__device__ __forceinline__ float tf32_rn(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}

// -------------------------------------------------------------- the tables
// T_d by columns: thread k applies the FP64 rotation operator (the stages of
// k_m2l_sibling, m2l.cu) to the unit multipole e_k and writes column k of
// T_d, split into TF32 hi and lo, in the swizzled B layout of its K chunk
template <int P>
__global__ void k_tc_tables(const double *__restrict__ dirs, int stride, int ef, int ei, int ph_off,
                            int vv, const uint8_t *__restrict__ lm_g,
                            const uint16_t *__restrict__ codes, float *__restrict__ out) {
  using D = TcDims<P>;
  constexpr int NM = D::NM, NL = D::NL;
  const int di = blockIdx.x, k = threadIdx.x;
  if (k >= D::NCH * 32) return;
  const double *tb = dirs + (size_t)codes[di] * stride;
  const double *ph = tb + ph_off;
  double yr[NM], yi[NM], rr[NM], ri[NM], tr_[NL], ti[NL], orr[NL], oi[NL];
  // phased unit source
  for (int c = 0; c < NM; ++c) {
    const double xr = (k < D::NIN && c == (k >> 1) && !(k & 1)) ? 1. : 0.;
    const double xi = (k < D::NIN && c == (k >> 1) && (k & 1)) ? 1. : 0.;
    const int m = lm_g[2 * c + 1];
    const double cr = ph[2 * m], ci = ph[2 * m + 1];
    yr[c] = xr * cr - xi * ci;
    yi[c] = xr * ci + xi * cr;
  }
  // rotation to the z axis
  for (int c = 0; c < NM; ++c) {
    const int l = lm_g[2 * c];
    const double *e = tb + ef + 2 * c;
    int step = 2 * (NM - 1);
    const int so = tri(l);
    double re = 0, im = 0;
    for (int m = 0; m <= l; ++m, e += step, step -= 2 * (m + 1)) {
      re += e[0] * yr[so + m];
      im += e[1] * yi[so + m];
    }
    rr[c] = re;
    ri[c] = im;
  }
  // translation along z (m-major slots)
  for (int kk = 0; kk < NL; ++kk) {
    int l, m;
    mmajor_lm(kk, P, l, m);
    const double *vcol = tb + vv + m2l_vrow_off(P, m) + kk;
    int vstep = m2l_vrow_len(P, m);
    double re = 0, im = 0;
    for (int n = m; n < P; ++n, vcol += vstep, vstep += P + 1 - n) {
      re += vcol[0] * rr[tri(n, m)];
      im += vcol[0] * ri[tri(n, m)];
    }
    tr_[kk] = re;
    ti[kk] = im;
  }
  // rotation back and conjugate z-phase
  for (int c = 0; c < NL; ++c) {
    const int l = lm_g[2 * c], mp = lm_g[2 * c + 1];
    const double *e = tb + ei + 2 * c;
    int step = 2 * (NL - 1);
    double re = 0, im = 0;
    int slot = l;
    for (int m = 0; m <= l; ++m, e += step, step -= 2 * (m + 1)) {
      re += e[0] * tr_[slot];
      im += e[1] * ti[slot];
      slot += P - m;
    }
    const double cr = ph[2 * mp], ci = -ph[2 * mp + 1];
    orr[c] = re * cr - im * ci;
    oi[c] = re * ci + im * cr;
  }
  const int j = k >> 5, kk = k & 31;
  float *hi = out + ((size_t)di * D::NCH + j) * 2 * (D::B_BYTES / 4);
  float *lo = hi + D::B_BYTES / 4;
  for (int n = 0; n < D::N; ++n) {
    const double v = n < D::NOUT ? ((n & 1) ? oi[n >> 1] : orr[n >> 1]) : 0.;
    const float h = tf32_rn((float)v);
    const uint32_t o = swz128(n, kk) / 4;
    hi[o] = h;
    lo[o] = tf32_rn((float)(v - (double)h));
  }
}

// ------------------------------------------------------------- the kernel
// Warp roles (288 threads): warps 0-7 produce the A rows (thread tid < 256:
// row tid & 127, K half tid >> 7) and drain the accumulators (the same
// thread: TMEM lane row, column half); warp 8 allocates tensor memory and its
// lane 0 issues the B copies and the MMAs.  Two accumulators alternate by
// offset: the MMAs of offset o go to accumulator o & 1 (the first with
// accumulate off), and once they complete the drain threads add it into
// FP32 sums in registers; the tensor core keeps each accumulation chain to
// one offset (12 x NCH MMAs), so its truncated FP32 accumulation costs
// about FP32 rounding.  mbarriers: afull / aempty per A slot (producers ->
// MMA, MMA commit -> producers), bfull / bempty per B slot (copy -> MMA, MMA
// commit -> B issue), accfull / accempty per accumulator (MMA commit ->
// drains, drains -> MMA).
constexpr int kTcWork = 256;               // producer / drain threads
constexpr int kTcAll = kTcWork + 32;       // + the MMA warp

template <int P>
__global__ void __launch_bounds__(kTcAll, 1)
    k_m2l_tc(int nparents, const int *__restrict__ parents, const int *__restrict__ child,
             const int *__restrict__ begin, const int *__restrict__ end,
             const int *__restrict__ col, const int *__restrict__ ncol,
             const int *__restrict__ ijk, const uint8_t *__restrict__ depth,
             const float *__restrict__ tabs, const int8_t *__restrict__ dvec, double scale_e,
             const float *__restrict__ mult, float *__restrict__ loc, int *__restrict__ err,
             int polls) {
  using D = TcDims<P>;
  constexpr int NCH = D::NCH, NIN = D::NIN, NOUT = D::NOUT, N = D::N;
  constexpr int ASL = D::ASLOTS, BSL = D::BSLOTS;
  constexpr int HALF = N / 2;                       // columns drained per thread
  constexpr int ACC_COLS = N <= 64 ? 64 : (N <= 128 ? 128 : 256);   // per accumulator
  constexpr int TCOLS = 2 * ACC_COLS;
  static_assert(HALF % 16 == 0, "drains in 16-column loads");
  extern __shared__ unsigned char smem_raw[];
  __shared__ uint64_t afull[ASL], aempty[ASL], bfull[BSL], bempty[BSL], accfull[2], accempty[2];
  __shared__ uint32_t s_tmem;
  __shared__ unsigned s_mask[6], s_neg[8];
  __shared__ uint8_t s_active[kTcOffsets + 3];
  __shared__ int s_nact;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool worker = tid < kTcWork;
  const int row = tid & 127, hh = (tid >> 7) & 1;
  const int w = blockIdx.x & 7;                       // child octant of the CTA
  const int bx = w & 1, by = (w >> 1) & 1, bz = (w >> 2) & 1;
  const uint32_t raw = smem_u32(smem_raw);
  const uint32_t base = (raw + 1023u) & ~1023u;
  unsigned char *gbase = smem_raw + (base - raw);
  const uint32_t a_s = base, b_s = base + ASL * 2 * D::A_BYTES;
  int *colb = reinterpret_cast<int *>(gbase + ASL * 2 * D::A_BYTES + BSL * 2 * D::B_BYTES);

  // the row's target: child w of parent blockIdx/8 * 128 + row
  const int pidx = (blockIdx.x >> 3) * kTcRows + row;
  int tgt = -1, P_ = -1;
  if (worker && pidx < nparents) {
    P_ = parents[pidx];
    const int t = child[P_] + w;
    if (end[t] > begin[t]) tgt = t;
  }
  if (worker && hh == 0) {
    for (int i = 0; i < 27; ++i) colb[row * 27 + i] = -1;
    if (tgt >= 0) {
      const int pi = ijk[3 * P_], pj = ijk[3 * P_ + 1], pk = ijk[3 * P_ + 2];
      const int nc = ncol[P_];
      for (int e = 0; e < nc; ++e) {
        const int q = col[27 * P_ + e];
        const int rx = ijk[3 * q] - pi + 1, ry = ijk[3 * q + 1] - pj + 1, rz = ijk[3 * q + 2] - pk + 1;
        colb[row * 27 + rx + 3 * (ry + 3 * rz)] = child[q];
      }
    }
  }
  if (tid < 6) s_mask[tid] = 0u;
  if (tid < 8) s_neg[tid] = 0u;
  if (tid == 0) {
    for (int b = 0; b < ASL; ++b) {
      mbar_init(&afull[b], kTcWork);
      mbar_init(&aempty[b], 1);
    }
    for (int b = 0; b < BSL; ++b) {
      mbar_init(&bfull[b], 1);
      mbar_init(&bempty[b], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], kTcWork);
    }
    fence_mbar_init();
  }
  if (warp == 8) tmem_alloc(&s_tmem, TCOLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = s_tmem;
  auto source_of = [&](int di) -> int {
    if (tgt < 0) return -1;
    const int dx = dvec[3 * di], dy = dvec[3 * di + 1], dz = dvec[3 * di + 2];
    const int cx = 2 + bx - (bx ? -dx : dx), cy = 2 + by - (by ? -dy : dy),
              cz = 2 + bz - (bz ? -dz : dz);
    const int cb = colb[row * 27 + (cx >> 1) + 3 * ((cy >> 1) + 3 * (cz >> 1))];
    return cb < 0 ? -1 : cb + ((cx & 1) | ((cy & 1) << 1) | ((cz & 1) << 2));
  };
  // offsets where some row has a source; mirror signs of the K inputs and
  // of the outputs (one bit per real, the same rule on both sides)
  if (worker) {
    unsigned m[6] = {0, 0, 0, 0, 0, 0};
    if (hh == 0)
      for (int di = 0; di < kTcOffsets; ++di)
        if (source_of(di) >= 0) m[di >> 5] |= 1u << (di & 31);
    for (int i = 0; i < 6; ++i)
      if (m[i]) atomicOr(&s_mask[i], m[i]);
    if (mirror_neg(tid, w)) atomicOr(&s_neg[tid >> 5], 1u << (tid & 31));
  }
  __syncthreads();
  if (tid == 0) {
    int n = 0;
    for (int di = 0; di < kTcOffsets; ++di)
      if ((s_mask[di >> 5] >> (di & 31)) & 1u) s_active[n++] = (uint8_t)di;
    s_nact = n;
  }
  __syncthreads();
  const int nact = s_nact;
  const int nsteps = nact * NCH;
  bool fail = false;

  if (worker) {
    // ---- producers of A, drains of the accumulators ----
    // this thread's 16 K values (4 float4) of step it
    auto load = [&](int it, float4 *r) {
      const int src = source_of(s_active[it / NCH]);
      const int j = it % NCH;
      const float4 *g = reinterpret_cast<const float4 *>(mult + (size_t)(src < 0 ? 0 : src) * NIN +
                                                         32 * j + 16 * hh);
#pragma unroll
      for (int q = 0; q < 4; ++q)
        r[q] = (src >= 0 && 32 * j + 16 * hh + 4 * q < NIN) ? __ldg(g + q)
                                                             : make_float4(0.f, 0.f, 0.f, 0.f);
    };
    auto store = [&](int it, const float4 *r) {
      const int slot = it % ASL, j = it % NCH;
      const unsigned neg = s_neg[j];
      unsigned char *ah = gbase + slot * 2 * D::A_BYTES;
      unsigned char *al = ah + D::A_BYTES;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int k0 = 16 * hh + 4 * q;
        float v[4] = {r[q].x, r[q].y, r[q].z, r[q].w};
        float h[4], l[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const float x = __uint_as_float(__float_as_uint(v[e]) ^ (((neg >> (k0 + e)) & 1u) << 31));
          h[e] = tf32_rn(x);
          l[e] = tf32_rn(x - h[e]);
        }
        const uint32_t o = swz128(row, k0);
        *reinterpret_cast<float4 *>(ah + o) = make_float4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<float4 *>(al + o) = make_float4(l[0], l[1], l[2], l[3]);
      }
    };
    float sum[HALF];
#pragma unroll
    for (int c = 0; c < HALF; ++c) sum[c] = 0.f;
    const uint32_t lane_base = (uint32_t)(32 * (warp & 3)) << 16;
    auto drain = [&](int od) {
      const int b = od & 1;
      if (!fail && !mbar_wait_or_flag(&accfull[b], (od >> 1) & 1, err, polls)) {
        fail = true;
        atomicOr(err, kErrTimeout);
      }
      if (!fail) {
        tc_fence_after();
#pragma unroll
        for (int cb = 0; cb < HALF / 16; ++cb) {
          float v[16];
          tmem_ld16(tmem + lane_base + b * ACC_COLS + hh * HALF + 16 * cb, v);
#pragma unroll
          for (int i = 0; i < 16; ++i) sum[16 * cb + i] += v[i];
        }
        tc_fence_before();
      }
      mbar_arrive(&accempty[b]);
    };
    float4 cur[4], nxt[4];
    if (nsteps > 0) load(0, cur);
    for (int it = 0; it < nsteps && !fail; ++it) {
      if (it + 1 < nsteps) load(it + 1, nxt);
      const int slot = it % ASL;
      if (it >= ASL && !mbar_wait_or_flag(&aempty[slot], ((it / ASL) - 1) & 1, err, polls)) {
        fail = true;
        atomicOr(err, kErrTimeout);
        break;
      }
      store(it, cur);
      fence_proxy_async_smem();
      mbar_arrive(&afull[slot]);
#pragma unroll
      for (int q = 0; q < 4; ++q) cur[q] = nxt[q];
      // after the last step of offset o, the accumulator of offset o - 1
      if (it % NCH == NCH - 1 && it / NCH >= 1) drain(it / NCH - 1);
    }
    if (nact > 0 && !fail) drain(nact - 1);
    // the row's sums, mirrored back and scaled, into its local
    if (!fail && nact > 0 && tgt >= 0) {
      const float ih = (float)((double)(1ull << depth[tgt]) / scale_e);
      float *lo = loc + (size_t)tgt * NOUT;
#pragma unroll
      for (int i = 0; i < HALF; i += 2) {
        const int n = hh * HALF + i;
        if (n < NOUT) {
          const unsigned neg0 = (s_neg[n >> 5] >> (n & 31)) & 1u;
          const unsigned neg1 = (s_neg[(n + 1) >> 5] >> ((n + 1) & 31)) & 1u;
          *reinterpret_cast<float2 *>(lo + n) =
              make_float2(sum[i] * (neg0 ? -ih : ih), sum[i + 1] * (neg1 ? -ih : ih));
        }
      }
    }
  } else if (lane == 0) {
    // ---- B copies and MMA issue ----
    constexpr uint32_t idesc = umma_idesc_tf32(kTcRows, N);
    auto issue_b = [&](int it) {
      const int slot = it % BSL;
      const int di = s_active[it / NCH], j = it % NCH;
      mbar_expect_tx(&bfull[slot], 2 * D::B_BYTES);
      bulk_g2s(gbase + (b_s - base) + slot * 2 * D::B_BYTES,
               tabs + ((size_t)di * NCH + j) * 2 * (D::B_BYTES / 4), 2 * D::B_BYTES, &bfull[slot]);
    };
    int issued_b = 0, committed = 0;
    for (; issued_b < BSL && issued_b < nsteps; ++issued_b) issue_b(issued_b);
    for (int it = 0; it < nsteps && !fail; ++it) {
      const int o = it / NCH, j = it % NCH, b = o & 1;
      if (j == 0 && o >= 2 && !mbar_wait_or_flag(&accempty[b], ((o >> 1) - 1) & 1, err, polls)) {
        fail = true;
        break;
      }
      if (!mbar_wait_or_flag(&afull[it % ASL], (it / ASL) & 1, err, polls) ||
          !mbar_wait_or_flag(&bfull[it % BSL], (it / BSL) & 1, err, polls)) {
        fail = true;
        break;
      }
      tc_fence_after();
      const uint32_t as = a_s + (it % ASL) * 2 * D::A_BYTES;
      const uint32_t bs = b_s + (it % BSL) * 2 * D::B_BYTES;
      const uint32_t dt = tmem + b * ACC_COLS;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const uint64_t ah = umma_desc_sw128(as + 32 * k), al = umma_desc_sw128(as + D::A_BYTES + 32 * k);
        const uint64_t bh = umma_desc_sw128(bs + 32 * k), bl = umma_desc_sw128(bs + D::B_BYTES + 32 * k);
        umma_tf32(dt, ah, bh, idesc, (j | k) ? 1u : 0u);
        umma_tf32(dt, ah, bl, idesc, 1u);
        umma_tf32(dt, al, bh, idesc, 1u);
      }
      umma_commit(&aempty[it % ASL]);
      umma_commit(&bempty[it % BSL]);
      if (j == NCH - 1) umma_commit(&accfull[b]);
      committed = it + 1;
      // refill the B slot of step it - 1 once its MMAs are done
      if (issued_b < nsteps && it >= 1) {
        if (!mbar_wait_or_flag(&bempty[(it - 1) % BSL], ((it - 1) / BSL) & 1, err, polls)) {
          fail = true;
          break;
        }
        issue_b(issued_b++);
      }
    }
    if (fail) atomicOr(err, kErrTimeout);
    // drain: the last commit covers every MMA; copies issued but not consumed
    // land before the CTA leaves
    // (and every commit's arrival has landed before the CTA's shared memory
    // can be reused)
    for (int i = committed - ASL < 0 ? 0 : committed - ASL; i < committed; ++i)
      mbar_wait(&aempty[i % ASL], (i / ASL) & 1);
    for (int i = committed - BSL < 0 ? 0 : committed - BSL; i < committed; ++i)
      mbar_wait(&bempty[i % BSL], (i / BSL) & 1);
    for (int i = committed; i < issued_b; ++i) mbar_wait(&bfull[i % BSL], (i / BSL) & 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 8) {
    __syncwarp();
    tmem_dealloc(tmem, TCOLS);
  }
}

template <int P>
void build_tc_tables(AranGpuSolver3d *s, cudaStream_t st) {
  using D = TcDims<P>;
  build_tables_fp64(s);
  // the child-0 offsets in the order of the lanes kernel (dz slowest)
  std::vector<uint16_t> codes;
  std::vector<int8_t> vec;
  for (int c = 0; c < 6; ++c)
    for (int b = 0; b < 6; ++b)
      for (int a = 0; a < 6; ++a) {
        if (a >= 2 && a <= 4 && b >= 2 && b <= 4 && c >= 2 && c <= 4) continue;
        codes.push_back((uint16_t)(a + 7 * b + 49 * c));
        vec.push_back((int8_t)(a - 3));
        vec.push_back((int8_t)(b - 3));
        vec.push_back((int8_t)(c - 3));
      }
  DBuf<uint16_t> dcodes;
  dcodes.reserve(codes.size());
  ACHECK(cudaMemcpyAsync(dcodes.ptr, codes.data(), codes.size() * 2, cudaMemcpyHostToDevice, st));
  s->tc_dvec.reserve(vec.size());
  ACHECK(cudaMemcpyAsync(s->tc_dvec.ptr, vec.data(), vec.size(), cudaMemcpyHostToDevice, st));
  s->tc_tab.reserve((size_t)kTcOffsets * D::NCH * 2 * (D::B_BYTES / 4));
  const int p = P;
  k_tc_tables<P><<<kTcOffsets, D::NCH * 32, 0, st>>>(
      s->t64.dir_m2l.ptr, dir_offset(p, 0, 6), dir_offset(p, 0, 0), dir_offset(p, 0, 2),
      dir_offset(p, 0, 4), dir_offset(p, 0, 7), s->t64.lm.ptr, dcodes.ptr, s->tc_tab.ptr);
  ACHECK(cudaGetLastError());
  ACHECK(cudaStreamSynchronize(st));
  dcodes.release();
  s->tc_p = P;
}

template <int P>
bool launch_tc(AranGpuSolver3d *s, const int *parents, int count, const float *mult, float *loc,
               cudaStream_t st) {
  DevTree &t = s->tree;
  if (s->tc_p != P) build_tc_tables<P>(s, st);
  const size_t sm = tc_smem<P>();
  int dev_smem = 0;
  ACHECK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  if ((int)(sm + 2048) > dev_smem) return false;
  smem_opt_in(k_m2l_tc<P>, sm);
  const int groups = ceil_div(count, kTcRows);
  k_m2l_tc<P><<<8 * groups, kTcAll, sm, st>>>(
      count, parents, t.child.ptr, t.begin.ptr, t.end.ptr, t.col.ptr, t.ncol.ptr, t.ijk.ptr,
      t.depth.ptr, s->tc_tab.ptr, s->tc_dvec.ptr, s->scale_e, mult, loc, s->err_dev.ptr,
      consumer_wait_polls());
  ACHECK(cudaGetLastError());
  s->launches++;
  return true;
}

}  // namespace

// The FP32 M2L on the tensor cores at orders 8 and 12; false leaves it to
// the other kernels.
bool launch_m2l_tc(AranGpuSolver3d *s, const int *parents, int count, const float *mult,
                   float *loc, cudaStream_t st) {
  if (count <= 0 || s->cfg.flavour == ARAN_FLAVOUR_KKYLIN) return false;
  switch (s->cfg.order) {
    case 8: return launch_tc<8>(s, parents, count, mult, loc, st);
    case 12: return launch_tc<12>(s, parents, count, mult, loc, st);
    default: return false;
  }
}

}  // namespace aran
