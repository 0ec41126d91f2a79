// p2p.cu -- the near field (P2P) on the device.
//
// LibAran calls the user p2p callback for every pair of points of every near
// leaf pair (near_func, aran/aransolver3d.c:254-324) with the Newton kernels
// of tests/newtonpot3.c:61-78 (potential) and tests/newtonfield3.c:91-119
// (field, |r| > 1e-5 guard).  Here every target particle sums its near
// sources directly (both sides of a pair are evaluated by their own targets
// instead of the symmetric update).
//
// Work decomposition: one block per target leaf; threads-per-target (tpt)
// grows as the leaf shrinks (n <= 8: 16, <= 16: 8, <= 32: 4, <= 64: 2,
// else 1), and a target's tpt threads take its near *leaves* round-robin so
// the per-leaf set-up is amortised over the leaf's points.  Near ranges of
// more than kBigRange points (a coarse leaf next to a deep subtree, common in
// clustered sets) are cut into leaf-aligned chunks processed by extra blocks
// that accumulate atomically.
//
// Mixed precision: positions are FP32 relative to their leaf centre, the
// centre difference comes from FP32 hi+lo centre pairs, per-source-leaf FP32
// partial sums go into FP64 accumulators, and pairs closer than 1/8 of the
// target leaf size (where FP32 cancellation would show) are recomputed from
// the FP64 positions.
#include <cub/cub.cuh>

#include <type_traits>

#include "internal.cuh"

namespace aran {

namespace {

constexpr unsigned kFull = 0xffffffffu;

// 1/sqrt(x) on the MUFU unit with denormals flushed: without the flush the
// FP32 rsqrt carries a denormal rescaling path; the near-field distances
// here are at least 1e-10 squared box units, far from denormal
__device__ __forceinline__ float rsqrt_ftz(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__global__ void k_leaf_info(int nleaves, const int *__restrict__ leaf_node,
                            const int *__restrict__ begin, const int *__restrict__ end,
                            const uint8_t *__restrict__ depth, const double *__restrict__ center,
                            double ex, double ey, double ez, int2 *__restrict__ be,
                            float4 *__restrict__ chi, float4 *__restrict__ clo) {
  int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nleaves) return;
  int node = leaf_node[L];
  be[L] = make_int2(begin[node], end[node]);
  double cx = center[3 * node], cy = center[3 * node + 1], cz = center[3 * node + 2];
  float hx = (float)cx, hy = (float)cy, hz = (float)cz;
  double h = fmin(ex, fmin(ey, ez)) / ldexp(1.0, depth[node]);
  float thr = (float)(h * 0.125);
  chi[L] = make_float4(hx, hy, hz, thr * thr);
  clo[L] = make_float4((float)(cx - (double)hx), (float)(cy - (double)hy), (float)(cz - (double)hz), 0.f);
}

__device__ __forceinline__ int rng_count(const int2 *be, int la, int lb) {
  return be[lb - 1].y - be[la].x;
}

// heavy ranges -> leaf-aligned chunks of about kBigRange points: one block
// per heavy range (listed by k_near with the offset of its first chunk), one
// thread per chunk, whose ends are the first leaves whose points start at or
// beyond p0 + i kBigRange (binary searches, independent per chunk)
__global__ void k_big_items(const int *__restrict__ heavy, int nleaves,
                            const int *__restrict__ near_off, const int *__restrict__ near_rng,
                            const int2 *__restrict__ be, int4 *__restrict__ items) {
  const int r = heavy[2 * blockIdx.x], coff = heavy[2 * blockIdx.x + 1];
  const int la = near_rng[2 * r], lb = near_rng[2 * r + 1];
  const int c = rng_count(be, la, lb);
  const int nch = (c + kBigRange - 1) / kBigRange;
  int lo = 0, hi = nleaves;                   // target leaf: last L with near_off[L] <= r
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (near_off[mid] <= r) lo = mid; else hi = mid;
  }
  const int L = lo;
  const int p0 = be[la].x;
  auto boundary = [&](int i) -> int {          // first leaf of chunk i
    if (i <= 0) return la;
    if (i >= nch) return lb;
    int l2 = la, h2 = lb;
    const int target = p0 + i * kBigRange;
    while (l2 < h2) {
      const int mid = (l2 + h2) >> 1;
      if (be[mid].x < target) l2 = mid + 1; else h2 = mid;
    }
    return l2;
  };
  for (int i = threadIdx.x; i < nch; i += blockDim.x)
    items[coff + i] = make_int4(L, boundary(i), boundary(i + 1), 0);
}

template <typename T, bool FIELD, bool MIXED, bool BIG>
__global__ void __launch_bounds__(128, 10) k_p2p(
    const int4 *__restrict__ items, const int *__restrict__ near_off,
    const int *__restrict__ near_rng, const int2 *__restrict__ be, const float4 *__restrict__ chi,
    const float4 *__restrict__ clo, const double *__restrict__ sx, const double *__restrict__ sy,
    const double *__restrict__ sz, const double *__restrict__ sq,
    const real4<float> *__restrict__ rel32, double *__restrict__ acc_pot,
    double *__restrict__ acc_fld) {
  int L, ia = 0, ib = 0;
  if (BIG) {
    int4 it = items[blockIdx.x];
    L = it.x;
    ia = it.y;
    ib = it.z;
  } else {
    L = blockIdx.x;
  }
  const int2 tbe = be[L];
  const int b = tbe.x, nt = tbe.y - tbe.x;
  const int tpt = nt <= 8 ? 16 : (nt <= 16 ? 8 : (nt <= 32 ? 4 : (nt <= 64 ? 2 : 1)));
  const int gsz = blockDim.x / tpt;
  const int sub = threadIdx.x % tpt;
  const bool leaf_strided = nt <= 8;
  const int r0 = near_off[L], r1 = near_off[L + 1];
  float4 tch = make_float4(0.f, 0.f, 0.f, 0.f), tcl = tch;
  if (MIXED) {
    tch = chi[L];
    tcl = clo[L];
  }
  for (int tb = 0; tb < nt; tb += gsz) {
    const int ti = tb + threadIdx.x / tpt;
    const bool active = ti < nt;
    if (!__any_sync(kFull, active)) continue;   // a warp with no target of this pass
    const int t = b + (active ? ti : 0);
    double pot = 0, fx = 0, fy = 0, fz = 0;
    // mixed: per-source-leaf FP32 sums are added with Kahan compensation in
    // FP32 (FP64 adds per leaf would occupy the FP64 pipe, 1/64 of FP32)
    float ks0 = 0.f, ks1 = 0.f, ks2 = 0.f, ks3 = 0.f;
    float kc0 = 0.f, kc1 = 0.f, kc2 = 0.f, kc3 = 0.f;
    auto kahan = [](float &sum, float &comp, float v) {
      const float y = v - comp;
      const float t2 = sum + y;
      comp = (t2 - sum) - y;
      sum = t2;
    };
    const double tx64 = sx[t], ty64 = sy[t], tz64 = sz[t];
    float tx = 0.f, ty = 0.f, tz = 0.f;
    if (MIXED) {
      real4<float> r = rel32[t];
      tx = r.x; ty = r.y; tz = r.z;
    }
    int kleaf = 0;
    // tiny target leaves: a target's threads take whole source leaves in turn;
    // otherwise they split every source leaf's points (keeps the warp converged)
    auto do_leaf = [&](int lf, int j0, int js) {
      const int2 sbe = be[lf];
      if (MIXED) {
        const float4 sh = chi[lf], sl = clo[lf];
        // target position relative to the source leaf centre
        const float ox = tx - ((sh.x - tch.x) + (sl.x - tcl.x));
        const float oy = ty - ((sh.y - tch.y) + (sl.y - tcl.y));
        const float oz = tz - ((sh.z - tch.z) + (sl.z - tcl.z));
        const float thr2 = tch.w;
        float p0 = 0.f, f0 = 0.f, f1 = 0.f, f2 = 0.f;
#pragma unroll 4
        for (int j = sbe.x + j0; j < sbe.y; j += js) {
          const real4<float> sj = rel32[j];
          float dx = ox - sj.x, dy = oy - sj.y, dz = oz - sj.z;
          float r2 = dx * dx + dy * dy + dz * dz;
          if (__builtin_expect(r2 < thr2, 0)) {
            if (j == t) {
              r2 = 0.f;
            } else {
              // close pair: difference from the FP64 positions
              dx = (float)(tx64 - sx[j]);
              dy = (float)(ty64 - sy[j]);
              dz = (float)(tz64 - sz[j]);
              r2 = dx * dx + dy * dy + dz * dz;
            }
          }
          const bool ok = FIELD ? (r2 > 1e-10f) : (r2 > 0.f);
          const float inv = ok ? rsqrt_ftz(r2) : 0.f;
          const float qi = sj.q * inv;
          p0 += qi;
          if (FIELD) {
            const float q3 = qi * inv * inv;
            f0 -= q3 * dx;
            f1 -= q3 * dy;
            f2 -= q3 * dz;
          }
        }
        kahan(ks0, kc0, p0);
        if (FIELD) {
          kahan(ks1, kc1, f0);
          kahan(ks2, kc2, f1);
          kahan(ks3, kc3, f2);
        }
      } else {
        for (int j = sbe.x + j0; j < sbe.y; j += js) {
          const double dx = tx64 - sx[j], dy = ty64 - sy[j], dz = tz64 - sz[j];
          const double r2 = dx * dx + dy * dy + dz * dz;
          // the point itself and coincident points: r2 == 0, skipped
          const bool ok = FIELD ? (r2 > 1e-10) : (r2 > 0.);
          const double inv = ok ? rsqrt(r2) : 0.;
          const double qi = sq[j] * inv;
          pot += qi;
          if (FIELD) {
            const double q3 = qi * inv * inv;
            fx -= q3 * dx;
            fy -= q3 * dy;
            fz -= q3 * dz;
          }
        }
      }
    };
    if (BIG) {
      if (leaf_strided)
        for (int lf = ia + sub; lf < ib; lf += tpt) do_leaf(lf, 0, 1);
      else
        for (int lf = ia; lf < ib; ++lf) do_leaf(lf, sub, tpt);
    } else {
      for (int rr = r0; rr < r1; ++rr) {
        const int la = near_rng[2 * rr], lb = near_rng[2 * rr + 1];
        if (lb <= la) continue;
        if (rng_count(be, la, lb) > kBigRange) continue;  // chunked by the BIG pass
        if (leaf_strided) {
          for (int lf = la; lf < lb; ++lf, ++kleaf)
            if (kleaf % tpt == sub) do_leaf(lf, 0, 1);
        } else {
          for (int lf = la; lf < lb; ++lf) do_leaf(lf, sub, tpt);
        }
      }
    }
    if (MIXED) {
      pot = (double)ks0 - (double)kc0;
      fx = (double)ks1 - (double)kc1;
      fy = (double)ks2 - (double)kc2;
      fz = (double)ks3 - (double)kc3;
    }
    for (int o = 1; o < tpt; o <<= 1) {
      pot += __shfl_xor_sync(kFull, pot, o);
      if (FIELD) {
        fx += __shfl_xor_sync(kFull, fx, o);
        fy += __shfl_xor_sync(kFull, fy, o);
        fz += __shfl_xor_sync(kFull, fz, o);
      }
    }
    if (active && sub == 0) {
      if (BIG) {
        atomicAdd(&acc_pot[t], pot);
        if (FIELD) {
          atomicAdd(&acc_fld[3 * (size_t)t], fx);
          atomicAdd(&acc_fld[3 * (size_t)t + 1], fy);
          atomicAdd(&acc_fld[3 * (size_t)t + 2], fz);
        }
      } else {
        acc_pot[t] = pot;
        if (FIELD) {
          acc_fld[3 * (size_t)t] = fx;
          acc_fld[3 * (size_t)t + 1] = fy;
          acc_fld[3 * (size_t)t + 2] = fz;
        }
      }
    }
  }
}

// Mixed near field, one warp per target leaf (four per block).  The warp
// walks the leaf's near source leaves; for each it stages up to 32 source
// points in shared memory, shifted to the target leaf's frame by the lane
// that loads them, and every lane sums them against its own targets from
// broadcast reads: lanes per target S = 32 / (n rounded up to a power of
// two) for n <= 16, else 1 (32 targets per pass), so the per-leaf set-up (centres, Kahan adds of the
// leaf partials) is paid once per lane per source leaf.  The pair loop has no
// branch: the distance is clamped below at h/8, and a lane whose chunk held a
// closer pair (or the point itself) takes the stand-ins back and adds those
// pairs from the FP64 positions afterwards.
// Ranges of more than kBigRange points are left to the chunked pass.
template <bool FIELD>
__global__ void __launch_bounds__(128, 8) k_p2p_warp(
    int nleaves, const int *__restrict__ near_off, const int *__restrict__ near_rng,
    const int2 *__restrict__ be, const float4 *__restrict__ chi, const float4 *__restrict__ clo,
    const double *__restrict__ sx, const double *__restrict__ sy, const double *__restrict__ sz,
    const real4<float> *__restrict__ rel32, double *__restrict__ acc_pot,
    double *__restrict__ acc_fld) {
  __shared__ float4 sbuf[4][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = blockIdx.x * 4 + w;
  if (L >= nleaves) return;
  const int2 tbe = be[L];
  const int b = tbe.x, nt = tbe.y - tbe.x;
  // lanes per target as a compile-time constant: one body per S
  const int Sd = nt <= 1 ? 32 : (nt <= 2 ? 16 : (nt <= 4 ? 8 : (nt <= 8 ? 4 : (nt <= 16 ? 2 : 1))));
  auto body = [&](auto sc) {
  constexpr int S = decltype(sc)::value;
  const int sub = lane & (S - 1);
  const float4 tch = chi[L], tcl = clo[L];
  const float thr2 = FIELD ? fmaxf(tch.w, 1e-10f) : tch.w;
  const int r0 = near_off[L], r1 = near_off[L + 1];
  float4 *buf = sbuf[w];
  const int step = 32 / S;
  for (int tb = 0; tb < nt; tb += step) {
    const int ti0 = tb + lane / S;
    const bool act0 = ti0 < nt;
    const int t0 = b + (act0 ? ti0 : 0);
    const real4<float> q0 = rel32[t0];
    float ks[4] = {}, kc[4] = {};
    auto kahan = [](float &sum, float &comp, float v) {
      const float y = v - comp;
      const float t2 = sum + y;
      comp = (t2 - sum) - y;
      sum = t2;
    };
    // one target against a staged source, r2 clamped below at thr2 (h/8
    // squared, at least the field guard 1e-10): close pairs and the point
    // itself add a bounded stand-in that close_fix takes back
    auto pair = [&](const real4<float> &q, const float4 &sv, float *p, float &rmin) {
      const float dx = q.x - sv.x, dy = q.y - sv.y, dz = q.z - sv.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      rmin = fminf(rmin, r2);
      const float inv = rsqrt_ftz(fmaxf(r2, thr2));
      const float qi = sv.w * inv;
      p[0] += qi;
      if (FIELD) {
        const float q3 = qi * inv * inv;
        p[1] -= q3 * dx;
        p[2] -= q3 * dy;
        p[3] -= q3 * dz;
      }
    };
    // for a close pair: remove the stand-in (the same FP32 expressions) and
    // add the pair from the FP64 positions (nothing for the point itself or
    // inside the field guard)
    auto close_fix = [&](const real4<float> &q, int t, const float4 &sv, int j, float *p) {
      const float dx = q.x - sv.x, dy = q.y - sv.y, dz = q.z - sv.z;
      const float r2 = dx * dx + dy * dy + dz * dz;
      if (!(r2 < thr2)) return;
      {
        const float inv = rsqrt_ftz(fmaxf(r2, thr2));
        const float qi = sv.w * inv;
        p[0] -= qi;
        if (FIELD) {
          const float q3 = qi * inv * inv;
          p[1] += q3 * dx;
          p[2] += q3 * dy;
          p[3] += q3 * dz;
        }
      }
      if (j == t) return;
      const float ex = (float)(sx[t] - sx[j]), ey = (float)(sy[t] - sy[j]),
                  ez = (float)(sz[t] - sz[j]);
      const float e2 = ex * ex + ey * ey + ez * ez;
      if (!(FIELD ? (e2 > 1e-10f) : (e2 > 0.f))) return;
      const float inv = rsqrt_ftz(e2);
      const float qi = sv.w * inv;
      p[0] += qi;
      if (FIELD) {
        const float q3 = qi * inv * inv;
        p[1] -= q3 * ex;
        p[2] -= q3 * ey;
        p[3] -= q3 * ez;
      }
    };
    for (int rr = r0; rr < r1; ++rr) {
      const int la = near_rng[2 * rr], lb = near_rng[2 * rr + 1];
      if (lb <= la) continue;
      if (rng_count(be, la, lb) > kBigRange) continue;  // chunked by the BIG pass
      for (int lf = la; lf < lb; ++lf) {
        const int2 sbe = be[lf];
        const float4 sh = chi[lf], sl = clo[lf];
        // source leaf centre relative to the target leaf centre
        const float cx = (sh.x - tch.x) + (sl.x - tcl.x);
        const float cy = (sh.y - tch.y) + (sl.y - tcl.y);
        const float cz = (sh.z - tch.z) + (sl.z - tcl.z);
        for (int j0 = sbe.x; j0 < sbe.y; j0 += 32) {
          const int cnt = min(32, sbe.y - j0);
          __syncwarp();
          if (lane < cnt) {
            const real4<float> r = rel32[j0 + lane];
            buf[lane] = make_float4(cx + r.x, cy + r.y, cz + r.z, r.q);
          }
          __syncwarp();
          float p0[4] = {0.f, 0.f, 0.f, 0.f};
          float rmin = 3.0e38f;
#pragma unroll 4
          for (int k = sub; k < cnt; k += S) pair(q0, buf[k], p0, rmin);
          const bool flag = rmin < thr2;
          if (__any_sync(kFull, flag) && flag)
            for (int k = sub; k < cnt; k += S) close_fix(q0, t0, buf[k], j0 + k, p0);
#pragma unroll
          for (int c = 0; c < (FIELD ? 4 : 1); ++c) kahan(ks[c], kc[c], p0[c]);
        }
      }
    }
    double v[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) v[c] = (double)ks[c] - (double)kc[c];
    for (int o = 1; o < S; o <<= 1)
#pragma unroll
      for (int c = 0; c < (FIELD ? 4 : 1); ++c) v[c] += __shfl_xor_sync(kFull, v[c], o);
    if (act0 && sub == 0) {
      acc_pot[t0] = v[0];
      if (FIELD) {
        acc_fld[3 * (size_t)t0] = v[1];
        acc_fld[3 * (size_t)t0 + 1] = v[2];
        acc_fld[3 * (size_t)t0 + 2] = v[3];
      }
    }
  }
  };
  if (Sd == 32) body(std::integral_constant<int, 32>{});
  else if (Sd == 16) body(std::integral_constant<int, 16>{});
  else if (Sd == 8) body(std::integral_constant<int, 8>{});
  else if (Sd == 4) body(std::integral_constant<int, 4>{});
  else if (Sd == 2) body(std::integral_constant<int, 2>{});
  else body(std::integral_constant<int, 1>{});
}

template <bool FIELD, bool MIXED, bool BIG>
void launch_one(AranGpuSolver3d *s, int grid, cudaStream_t st) {
  DevTree &t = s->tree;
  using T = typename std::conditional<MIXED, float, double>::type;
  k_p2p<T, FIELD, MIXED, BIG><<<grid, 128, 0, st>>>(
      t.big_items.ptr, t.near_off.ptr, t.near_rng.ptr, t.leaf_be.ptr, t.leaf_chi.ptr,
      t.leaf_clo.ptr, s->sx.ptr, s->sy.ptr, s->sz.ptr, s->sq.ptr, s->rel32.ptr, s->acc_pot.ptr,
      s->acc_fld.ptr);
  ACHECK(cudaGetLastError());
  s->launches++;
}

template <bool FIELD, bool MIXED>
void launch_pair(AranGpuSolver3d *s, cudaStream_t st) {
  DevTree &t = s->tree;
  if constexpr (MIXED) {
    k_p2p_warp<FIELD><<<ceil_div(t.nleaves, 4), 128, 0, st>>>(
        t.nleaves, t.near_off.ptr, t.near_rng.ptr, t.leaf_be.ptr, t.leaf_chi.ptr, t.leaf_clo.ptr,
        s->sx.ptr, s->sy.ptr, s->sz.ptr, s->rel32.ptr, s->acc_pot.ptr, s->acc_fld.ptr);
    ACHECK(cudaGetLastError());
    s->launches++;
  } else {
    launch_one<FIELD, MIXED, false>(s, s->tree.nleaves, st);
  }
  if (s->tree.n_big) launch_one<FIELD, MIXED, true>(s, s->tree.n_big, st);
}

}  // namespace

void build_p2p_work(AranGpuSolver3d *s) {
  cudaStream_t st = s->s0;
  DevTree &t = s->tree;
  const int TB = 256;
  int nl = t.nleaves;
  t.leaf_be.reserve(nl);
  t.leaf_chi.reserve(nl);
  t.leaf_clo.reserve(nl);
  double ex = s->cfg.ub[0] - s->cfg.lb[0], ey = s->cfg.ub[1] - s->cfg.lb[1],
         ez = s->cfg.ub[2] - s->cfg.lb[2];
  k_leaf_info<<<ceil_div(nl, TB), TB, 0, st>>>(nl, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                               t.depth.ptr, t.center.ptr, ex, ey, ez,
                                               t.leaf_be.ptr, t.leaf_chi.ptr, t.leaf_clo.ptr);
  ACHECK(cudaGetLastError());
  s->launches++;
  // chunk total and heavy-range count, as k_near listed them
  int *hb = s->h_small + 8;   // pinned
  hb[0] = hb[1] = 0;
  if (t.n_near_rng > 0) {
    ACHECK(cudaMemcpyAsync(hb, t.big_rng.ptr, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    ACHECK(cudaStreamSynchronize(st));
  }
  const int nbig = hb[0], nheavy = hb[1];
  t.n_big = nbig;
  if (nbig) {
    t.big_items.reserve(nbig);
    k_big_items<<<nheavy, 64, 0, st>>>(t.big_rng.ptr + 2, nl, t.near_off.ptr, t.near_rng.ptr,
                                       t.leaf_be.ptr, t.big_items.ptr);
    ACHECK(cudaGetLastError());
    s->launches++;
  }
}

void launch_p2p(AranGpuSolver3d *s, cudaStream_t st) {
  const bool mixed = s->cfg.precision == ARAN_PRECISION_MIXED;
  const bool field = s->cfg.field != 0;
  if (mixed) {
    if (field) launch_pair<true, true>(s, st);
    else launch_pair<false, true>(s, st);
  } else {
    if (field) launch_pair<true, false>(s, st);
    else launch_pair<false, false>(s, st);
  }
}

}  // namespace aran
