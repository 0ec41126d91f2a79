// m2l_lanes.cu -- lane-parallel M2L for the FP32 path at the orders
// m2l_lane_order(p) accepts.  Same operator as m2l.cu (the "point and shoot"
// translation of aran_spherical_seriesd_to_local_rotate,
// aran/aransphericalseriesd-rotate.c:165-207, applied by far_func,
// aran/aransolver3d.c:333-354) with the work laid out the other way round:
//
//  * after the z-phase, the rotation, the translation along z and the
//    rotation back never mix real and imaginary parts (the even/odd Wigner
//    blocks act on the real/imaginary parts, the vertical factors are real),
//    so one lane carries the real part and its neighbour the imaginary part
//    of one (target, source) translation;
//  * a warp takes child w of the 16 parents of its CTA (lane pair i <->
//    parent i), so at a given offset all 16 lane pairs apply the same table:
//    every table read is a broadcast of 16 bytes (four factors) from shared
//    memory, and a lane's whole series stays in registers, the order being a
//    compile-time constant;
//  * child w = (bx, by, bz) reaches its sources through the offsets with
//    d_x in [bx-3, bx+2] (same for y, z); the mirror image sigma_w (x -> -x
//    where bx = 1, likewise y, z) maps them onto child 0's 189 offsets, and
//    the translation obeys T_d = S T_{sigma d} S, with S the action of the
//    mirror on series: (l, m) -> (-1)^{l+m} on a z flip, conjugation on a y
//    flip, (-1)^m conjugation on an x flip.  So all eight warps walk child
//    0's offsets together, each applying S to its sources on the way in and
//    once to its accumulated locals on the way out: every table in the ring
//    serves all eight warps;
//  * the two lanes of a pair exchange their rotated-back parts with one
//    shuffle to apply the conjugate z-phase, and each lane accumulates its
//    part of the target's local in shared memory (one word per lane, no
//    conflicts), in the same offset order for every run.
//
// The offset tables stream through a three-slot ring of TMA bulk copies;
// the next offset's source multipoles are brought into shared memory by one
// bulk copy each while the current one is translated.  Every mbarrier
// wait is bounded; a wait that gives up sets the error word and the CTA
// stops.
#include "internal.cuh"
#include "async.cuh"

namespace aran {

namespace {

constexpr int kLanePar = 16;     // parents per CTA: lane pair i <-> parent i
constexpr int kLaneWarps = 8;    // consumer warps: warp w <-> child w
constexpr int kLaneNst = 3;      // table ring slots
constexpr unsigned kFull = 0xffffffffu;

template <int P>
struct LaneDims {
  static constexpr int NM = P * (P + 1) / 2;        // multipole coefficients
  static constexpr int NL = (P + 1) * (P + 2) / 2;  // local coefficients
  static constexpr int NMP = (NM + 1) & ~1;         // staged multipole stride (16-byte rows)
  static constexpr int STRIDE = m2l_lane_stride(P);
};

template <int P>
constexpr size_t lanes_smem() {
  using D = LaneDims<P>;
  size_t off = (size_t)kLaneNst * D::STRIDE * sizeof(float);
  off += 2 * kLaneNst * sizeof(uint64_t) + kLaneWarps * sizeof(uint64_t);
  off += (size_t)kLaneWarps * kLanePar * D::NMP * sizeof(cplx<float>);
  off += (size_t)kLaneWarps * D::NL * 32 * sizeof(float);
  off += (size_t)kLanePar * 216 * sizeof(int);
  off += 16 * sizeof(unsigned) + 320 * sizeof(uint16_t) + 320 * sizeof(uint16_t) + 320 * 3;
  return off + 64;
}

__device__ __forceinline__ float sel4(const float4 &v, int k) {
  return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

template <int P>
__global__ void __launch_bounds__(32 * kLaneWarps, 1)
    k_m2l_lanes(int nparents, const int *__restrict__ parents, const int *__restrict__ child,
                const int *__restrict__ begin, const int *__restrict__ end,
                const int *__restrict__ col, const int *__restrict__ ncol,
                const int *__restrict__ ijk, const uint8_t *__restrict__ depth,
                const float *__restrict__ dirs, double scale_e,
                const cplx<float> *__restrict__ mult, cplx<float> *__restrict__ loc,
                int *__restrict__ err, int polls) {
  using D = LaneDims<P>;
  constexpr int NM = D::NM, NL = D::NL, NMP = D::NMP, STRIDE = D::STRIDE;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // shared layout: ring tables | full[NST] | empty[NST] | staged multipoles
  // [warp][pair][NMP] | local parts [warp][coefficient][lane] | 16 6x6x6
  // source grids | offset mask | active offsets | offset codes | offset vectors
  size_t off = 0;
  float *tab = reinterpret_cast<float *>(smem_raw);
  off += (size_t)kLaneNst * STRIDE * sizeof(float);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + off);
  uint64_t *empty = full + kLaneNst;
  uint64_t *sbar = empty + kLaneNst;    // per warp: its staged sources have landed
  off += 2 * kLaneNst * sizeof(uint64_t) + kLaneWarps * sizeof(uint64_t);
  cplx<float> *stg = reinterpret_cast<cplx<float> *>(smem_raw + off);
  off += (size_t)kLaneWarps * kLanePar * NMP * sizeof(cplx<float>);
  float *accs = reinterpret_cast<float *>(smem_raw + off);
  off += (size_t)kLaneWarps * NL * 32 * sizeof(float);
  int *grid = reinterpret_cast<int *>(smem_raw + off);
  off += (size_t)kLanePar * 216 * sizeof(int);
  unsigned *mask = reinterpret_cast<unsigned *>(smem_raw + off);
  off += 16 * sizeof(unsigned);
  uint16_t *active = reinterpret_cast<uint16_t *>(smem_raw + off);
  off += 320 * sizeof(uint16_t);
  uint16_t *dcode = reinterpret_cast<uint16_t *>(smem_raw + off);   // 189 of them
  off += 320 * sizeof(uint16_t);
  int8_t *dvec = reinterpret_cast<int8_t *>(smem_raw + off);
  __shared__ int s_nact;

  for (int i = threadIdx.x; i < kLanePar * 216; i += blockDim.x) grid[i] = -1;
  for (int i = threadIdx.x; i < kLaneWarps * NL * 32; i += blockDim.x) accs[i] = 0.f;
  if (threadIdx.x < 16) mask[threadIdx.x] = 0u;
  // child 0's offsets (dx, dy, dz) in [-3,2]^3 minus [-1,1]^3, dz slowest:
  // index = L - (near cells below L), L = (dx+3) + 6 (dy+3) + 36 (dz+3); table
  // code (dx+3) + 7 (dy+3) + 49 (dz+3)
  for (int L = threadIdx.x; L < 216; L += blockDim.x) {
    const int a = L % 6, b = (L / 6) % 6, c = L / 36;
    auto in = [](int v) { return v >= 2 && v <= 4; };
    auto below = [](int v) { return v < 2 ? 0 : (v > 4 ? 3 : v - 2); };
    if (in(a) && in(b) && in(c)) continue;
    const int nb = 9 * below(c) + (in(c) ? 3 * below(b) + (in(b) ? below(a) : 0) : 0);
    const int di = L - nb;
    dcode[di] = (uint16_t)(a + 7 * b + 49 * c);
    dvec[3 * di] = (int8_t)(a - 3);
    dvec[3 * di + 1] = (int8_t)(b - 3);
    dvec[3 * di + 2] = (int8_t)(c - 3);
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < kLaneNst; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], kLaneWarps);
    }
    for (int k = 0; k < kLaneWarps; ++k) mbar_init(&sbar[k], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // the parents of this CTA: their colleagues' children fill the grids
  for (int g = 0; g < kLanePar; ++g) {
    const int pidx = blockIdx.x * kLanePar + g;
    if (pidx >= nparents) break;
    const int Pn = parents[pidx];
    const int pi = ijk[3 * Pn], pj = ijk[3 * Pn + 1], pk = ijk[3 * Pn + 2];
    const int nc = ncol[Pn];
    for (int e = threadIdx.x; e < nc * 8; e += blockDim.x) {
      const int q = col[27 * Pn + e / 8];
      const int qc = child[q];
      if (qc < 0) continue;
      const int o = e & 7;
      const int s = qc + o;
      if (end[s] == begin[s]) continue;
      const int gx = 2 * (ijk[3 * q] - pi + 1) + (o & 1);
      const int gy = 2 * (ijk[3 * q + 1] - pj + 1) + ((o >> 1) & 1);
      const int gz = 2 * (ijk[3 * q + 2] - pk + 1) + ((o >> 2) & 1);
      grid[g * 216 + gx + 6 * (gy + 6 * gz)] = s;
    }
  }
  __syncthreads();
  // lane pair i = lane / 2 <-> parent i; h = 0 real part, 1 imaginary part
  const int pi_ = lane >> 1, h = lane & 1;
  int tgt = -1;
  {
    const int pidx = blockIdx.x * kLanePar + pi_;
    if (w < kLaneWarps && pidx < nparents) {
      const int t = child[parents[pidx]] + w;
      if (end[t] > begin[t]) tgt = t;
    }
  }
  // child w = (bx, by, bz) at cell (2+bx, 2+by, 2+bz) of the grid; its
  // offset for child 0's offset d is sigma_w d
  const int bx = w & 1, by = (w >> 1) & 1, bz = (w >> 2) & 1;
  const int tx = 2 + bx, ty = 2 + by, tz = 2 + bz;
  auto source_of = [&](int di) -> int {
    if (tgt < 0) return -1;
    const int dx = dvec[3 * di], dy = dvec[3 * di + 1], dz = dvec[3 * di + 2];
    const int cx = tx - (bx ? -dx : dx), cy = ty - (by ? -dy : dy), cz = tz - (bz ? -dz : dz);
    if (cx < 0 || cx > 5 || cy < 0 || cy > 5 || cz < 0 || cz > 5) return -1;
    return grid[pi_ * 216 + cx + 6 * (cy + 6 * cz)];
  };
  if (w < kLaneWarps)
    for (int di = 0; di < 189; ++di) {
      const unsigned any = __ballot_sync(kFull, source_of(di) >= 0);
      if (lane == 0 && any) atomicOr(&mask[di >> 5], 1u << (di & 31));
    }
  __syncthreads();
  for (int di = threadIdx.x; di < 189; di += blockDim.x) {
    const unsigned m = mask[di >> 5];
    if ((m >> (di & 31)) & 1u) {
      int pos = __popc(m & ((1u << (di & 31)) - 1u));
      for (int k = 0; k < (di >> 5); ++k) pos += __popc(mask[k]);
      active[pos] = (uint16_t)di;
    }
  }
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int k = 0; k < 6; ++k) tot += __popc(mask[k]);
    s_nact = tot;
  }
  __syncthreads();
  const int nact = s_nact;

  // the ring: thread 0 fills the first slots; afterwards warp 0 refills
  // slot b with offset it + NST once all warps have released it (no
  // separate producer warp, so two warps share each scheduler's registers)
  constexpr uint32_t kTabBytes = STRIDE * (uint32_t)sizeof(float);
  auto issue = [&](int i) {
    const int b = i % kLaneNst;
    mbar_expect_tx(&full[b], kTabBytes);
    bulk_g2s(tab + (size_t)b * STRIDE, dirs + (size_t)dcode[active[i]] * STRIDE, kTabBytes,
             &full[b]);
  };
  int issued = 0;   // table copies issued (thread 0)
  if (threadIdx.x == 0)
    for (; issued < kLaneNst && issued < nact; ++issued) issue(issued);

  cplx<float> *my_stg = stg + (size_t)(w * kLanePar + pi_) * NMP;
  float *my_acc = accs + (size_t)w * NL * 32 + lane;   // coefficient c at my_acc[32 c]
  // up to order 8 the target's local part stays in registers (at order 12
  // the series already fill them, and it lives in shared memory)
  constexpr bool RACC = P <= 8;
  float racc[RACC ? NL : 1];
#pragma unroll
  for (int c = 0; c < (RACC ? NL : 1); ++c) racc[c] = 0.f;
  int next_i = 0, next_s = -1;
  auto find_next = [&](int from) {
    for (next_i = from; next_i < nact; ++next_i) {
      next_s = source_of(active[next_i]);
      if (__any_sync(kFull, next_s >= 0)) break;
    }
  };
  // one bulk copy per source (issued by the pair's first lane) completing
  // on the warp's barrier; pairs without a source zero their slot
  static_assert(NM % 2 == 0, "bulk copies of whole 16-byte rows");
  constexpr uint32_t kSrcBytes = NM * (uint32_t)sizeof(cplx<float>);
  bool pending = false;
  uint32_t sph = 0;
  auto prefetch = [&]() {
    if (next_i >= nact) return;
    const unsigned cp = __ballot_sync(kFull, h == 0 && next_s >= 0);
    if (lane == 0) mbar_expect_tx(&sbar[w], (uint32_t)__popc(cp) * kSrcBytes);
    __syncwarp();
    if (next_s >= 0) {
      if (h == 0) bulk_g2s(my_stg, mult + (size_t)next_s * NM, kSrcBytes, &sbar[w]);
    } else {
      for (int c = h; c < NM; c += 2) my_stg[c] = cmake<float>(0.f, 0.f);
    }
    pending = true;
  };
  find_next(0);
  prefetch();

  int it = 0;
  for (; it < nact; ++it) {
    const int b = it % kLaneNst;
    const bool ok = __all_sync(kFull, mbar_wait_or_flag(&full[b], (it / kLaneNst) & 1, err, polls));
    if (!ok) {
      if (lane == 0) atomicOr(err, kErrTimeout);
      break;
    }
    if (it == next_i) {
      const float *tb = tab + (size_t)b * STRIDE;
      const float2 *ph2 = reinterpret_cast<const float2 *>(tb);    // (cos, sin) of m phi
      if (!__all_sync(kFull, mbar_wait(&sbar[w], sph))) {
        if (lane == 0) atomicOr(err, kErrTimeout);
        break;
      }
      sph ^= 1u;
      pending = false;
      __syncwarp();
      // mirror S, z-phase and rotation to the z axis (degrees < p): this
      // lane's part of the phased mirrored source (l, m) is
      // sn (x.re pa[m] + x.im pb[m]), sn = -1 for odd l under a z flip
      float y[NM];
      {
        float pa[P], pb[P];
#pragma unroll
        for (int m = 0; m < P; ++m) {
          const float2 e = ph2[m];
          const float g = ((bx ^ bz) & m & 1) ? -1.f : 1.f;       // (-1)^m of x and z flips
          const float cj = (bx ^ by) ? -g : g;                     // conjugation
          pa[m] = g * (h ? e.y : e.x);
          pb[m] = cj * (h ? e.x : -e.y);
        }
        const float4 *X4 = reinterpret_cast<const float4 *>(my_stg);
        const float4 *F4 = reinterpret_cast<const float4 *>(tb + m2l_lane_f(P)) + h;
        const float f0 = h ? 0.f : 2.f;
        float4 xq = make_float4(0.f, 0.f, 0.f, 0.f), fq = xq;
#pragma unroll
        for (int l = 0; l < P; ++l) {
          const float sn = (bz && (l & 1)) ? -1.f : 1.f;
          float xp[P], yd[P], yt[P];
#pragma unroll
          for (int m = 0; m <= l; ++m) {
            const int c = l * (l + 1) / 2 + m;
            if ((c & 1) == 0) xq = X4[c >> 1];
            const float xr = (c & 1) ? xq.z : xq.x, xi = (c & 1) ? xq.w : xq.y;
            xp[m] = sn * fmaf(xr, pa[m], xi * pb[m]);
            yd[m] = 0.f;
            yt[m] = 0.f;
          }
          // lower triangle (m <= m') direct, upper triangle by symmetry
#pragma unroll
          for (int mp = 0; mp <= l; ++mp)
#pragma unroll
            for (int m = 0; m <= mp; ++m) {
              const int t = m2l_lane_tet(l) + mp * (mp + 1) / 2 + m;
              if ((t & 3) == 0) fq = F4[2 * (t >> 2)];
              const float v = sel4(fq, t & 3);
              yd[mp] = fmaf(v, xp[m], yd[mp]);
              if (m < mp) yt[m] = fmaf(v, (mp & 1) ? -xp[mp] : xp[mp], yt[m]);
            }
          y[l * (l + 1) / 2] = fmaf(f0, yt[0], yd[0]);
#pragma unroll
          for (int m = 1; m <= l; ++m)
            y[l * (l + 1) / 2 + m] = (m & 1) ? yd[m] - yt[m] : yd[m] + yt[m];
        }
      }
      find_next(it + 1);
      __syncwarp();           // both lanes of every pair are done with the staged source
      prefetch();
      // translation along z in the scaled frame (y carries 1/beta_n from
      // the forward table, the backward table restores (-1)^{j+m} beta_j):
      // z(j, m) = sum_n S(j, n) y(n, m), S symmetric, m-major slots
      float z[NL];
      {
        const float4 *V4 = reinterpret_cast<const float4 *>(tb + m2l_lane_v(P));
        float4 vq = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int m = 0; m <= P; ++m) {
          constexpr int KM = P + 1;
          const int k = P - m;
          float zz[KM];
#pragma unroll
          for (int jj = 0; jj <= k; ++jj) zz[jj] = 0.f;
#pragma unroll
          for (int jj = 0; jj < k; ++jj)
#pragma unroll
            for (int nn = 0; nn <= jj; ++nn) {
              const int t = m2l_lane_vpre(P, m) + jj * (jj + 1) / 2 + nn;
              if ((t & 3) == 0) vq = V4[t >> 2];
              const float v = sel4(vq, t & 3);
              const int n = m + nn, j = m + jj;
              zz[jj] = fmaf(v, y[n * (n + 1) / 2 + m], zz[jj]);
              if (nn < jj) zz[nn] = fmaf(v, y[j * (j + 1) / 2 + m], zz[nn]);
            }
#pragma unroll
          for (int nn = 0; nn < k; ++nn) {
            const int t = m2l_lane_vpre(P, m) + k * (k + 1) / 2 + nn;
            if ((t & 3) == 0) vq = V4[t >> 2];
            const int n = m + nn;
            zz[k] = fmaf(sel4(vq, t & 3), y[n * (n + 1) / 2 + m], zz[k]);
          }
#pragma unroll
          for (int jj = 0; jj <= k; ++jj) z[m * (P + 1) - m * (m - 1) / 2 + jj] = zz[jj];
        }
      }
      // rotation back (degrees <= p); degree l of z dies as degree l of o
      // is made, so the two share the registers
      float o[NL];
      {
        const float4 *B4 = reinterpret_cast<const float4 *>(tb + m2l_lane_b(P)) + h;
        const float f0 = h ? 0.f : 2.f;
        float4 bq = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int l = 0; l <= P; ++l) {
          float zi[P + 1], od[P + 1], ot[P + 1];
#pragma unroll
          for (int m = 0; m <= l; ++m) {
            zi[m] = z[m * (P + 1) - m * (m - 1) / 2 + (l - m)];
            od[m] = 0.f;
            ot[m] = 0.f;
          }
#pragma unroll
          for (int mp = 0; mp <= l; ++mp)
#pragma unroll
            for (int m = 0; m <= mp; ++m) {
              const int t = m2l_lane_tet(l) + mp * (mp + 1) / 2 + m;
              if ((t & 3) == 0) bq = B4[2 * (t >> 2)];
              const float v = sel4(bq, t & 3);
              od[mp] = fmaf(v, zi[m], od[mp]);
              if (m < mp) ot[m] = fmaf(v, zi[mp], ot[m]);
            }
          o[l * (l + 1) / 2] = fmaf(f0, ot[0], od[0]);
#pragma unroll
          for (int m = 1; m <= l; ++m) o[l * (l + 1) / 2 + m] = od[m] + ot[m];
        }
      }
      // conjugate z-phase and accumulate, after the last table read: real
      // part += a cos + b sin, imaginary part += a cos - b sin, with a this
      // lane's part and b the partner's
      float cph[P + 1], sph[P + 1];
#pragma unroll
      for (int m = 0; m <= P; ++m) {
        const float2 e = ph2[m];
        cph[m] = e.x;
        sph[m] = h ? -e.y : e.y;
      }
#pragma unroll
      for (int l = 0; l <= P; ++l)
#pragma unroll
        for (int mp = 0; mp <= l; ++mp) {
          const float a = o[l * (l + 1) / 2 + mp];
          const float bp = __shfl_xor_sync(kFull, a, 1);
          if (RACC) {
            racc[RACC ? l * (l + 1) / 2 + mp : 0] += fmaf(a, cph[mp], bp * sph[mp]);
          } else {
            float *slot = my_acc + 32 * (l * (l + 1) / 2 + mp);
            *slot += fmaf(a, cph[mp], bp * sph[mp]);
          }
        }
    }
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(&empty[b]);
      if (w == 0 && it + kLaneNst < nact) {
        if (!mbar_wait_or_flag(&empty[b], (it / kLaneNst) & 1, err)) {
          atomicOr(err, kErrTimeout);
        } else {
          issue(it + kLaneNst);
          ++issued;
        }
      }
    }
    __syncwarp();
  }
  // copies still in flight after an early exit land before the CTA leaves
  if (pending) mbar_wait(&sbar[w], sph);
  if (threadIdx.x == 0)
    for (int i = it; i < issued; ++i) mbar_wait(&full[i % kLaneNst], (i / kLaneNst) & 1);
  if (nact > 0 && tgt >= 0) {
    // back from the mirror frame: S on the accumulated local
    const float ih = (float)((double)(1ull << depth[tgt]) / scale_e);   // 2^depth / scale
    float *lo = reinterpret_cast<float *>(loc) + (size_t)tgt * NL * 2 + h;
#pragma unroll
    for (int l = 0; l <= P; ++l)
#pragma unroll
      for (int m = 0; m <= l; ++m) {
        const int c = l * (l + 1) / 2 + m;
        const bool neg = ((bz & (l + m)) ^ (bx & m) ^ (h & (bx ^ by))) & 1;
        lo[2 * c] = (RACC ? racc[RACC ? c : 0] : my_acc[32 * c]) * (neg ? -ih : ih);
      }
  }
}

template <int P>
bool launch_p(AranGpuSolver3d *s, OpTables<float> &tb, const int *parents, int count,
              const cplx<float> *mult, cplx<float> *loc, cudaStream_t st) {
  DevTree &t = s->tree;
  const size_t sm = lanes_smem<P>();
  int dev_smem = 0;
  ACHECK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  if ((int)sm > dev_smem) return false;
  smem_opt_in(k_m2l_lanes<P>, sm);
  k_m2l_lanes<P><<<ceil_div(count, kLanePar), 32 * kLaneWarps, sm, st>>>(
      count, parents, t.child.ptr, t.begin.ptr, t.end.ptr, t.col.ptr, t.ncol.ptr,
      t.ijk.ptr, t.depth.ptr, tb.dir_lanes.ptr, s->scale_e, mult, loc, s->err_dev.ptr,
      consumer_wait_polls());
  ACHECK(cudaGetLastError());
  s->launches++;
  return true;
}

}  // namespace

// Runs the M2L pass with the lane-parallel kernel when the order has one;
// false leaves it to m2l.cu.
bool launch_m2l_lanes(AranGpuSolver3d *s, OpTables<float> &tb, const int *parents, int count,
                      const cplx<float> *mult, cplx<float> *loc, cudaStream_t st) {
  const int p = s->cfg.order;
  if (!m2l_lane_order(p) || tb.dir_lanes.ptr == nullptr || count <= 0) return false;
  switch (p) {
    case 4: return launch_p<4>(s, tb, parents, count, mult, loc, st);
    case 8: return launch_p<8>(s, tb, parents, count, mult, loc, st);
    case 12: return launch_p<12>(s, tb, parents, count, mult, loc, st);
    default: return false;
  }
}

}  // namespace aran
