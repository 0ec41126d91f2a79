// passes.cu -- the FMM passes on the device.
//
// LibAran runs them as callbacks from tree traversals (aran/aransolver3d.c):
//   clear_func :399-410   -> one memset of all expansions
//   up_func :412-450      -> k_p2m (leaves) + k_m2m_rotate (level by level)
//   far_func :333-354     -> k_m2l_sibling (m2l.cu)
//   near_func :254-324    -> k_p2p (p2p.cu)
//   down_func :452-490    -> k_l2l_rotate (level by level) + k_l2p
// The operators are the "point and shoot" rotation flavour of
// aran/aransphericalseriesd-rotate.c (rotate to the z axis, translate along
// z, rotate back), with even/odd real rotation blocks and the z-phases
// applied separately; expansions are stored scaled per level (see
// fmm_math.cuh).  Every kernel is templated on the arithmetic type: double
// for the plain FP64 path, float for the mixed path (whose P2P/L2P results
// are accumulated in FP64).
#include "internal.cuh"

namespace aran {


namespace {

constexpr unsigned kFull = 0xffffffffu;

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

template <typename T>
__device__ __forceinline__ T inv_scale(int depth, double scale_e) {
  // 1/h_d = 2^d / 2^E (exact power of two)
  return (T)(ldexp(1.0, depth) / scale_e);
}

// ---------------------------------------------------------------------------
// P2M: aran/arandevelopment3d.c:169-216, one warp per non-empty leaf.
// Mhat_l^m = sum_i q_i 4pi/(2l+1) conj(S_l^m(xhat_i)), S = r^l Y_l^m by the
// trig-free recurrence of fmm_math.cuh.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_p2m(int nleaves, const int *__restrict__ leaf_node, const int *__restrict__ begin,
                      const int *__restrict__ end, const uint8_t *__restrict__ depth,
                      const real4<T> *__restrict__ rel, int p, const T *__restrict__ rec_g,
                      const T *__restrict__ p2mf_g, double scale_e, cplx<T> *__restrict__ mult) {
  extern __shared__ unsigned char smem_raw[];
  const int nm = tri(p);
  T *rec = reinterpret_cast<T *>(smem_raw);
  T *p2mf = rec + 2 * tri(p + 1);
  cplx<T> *outs = reinterpret_cast<cplx<T> *>(p2mf + p + 1 + ((p + 1) & 1));
  for (int i = threadIdx.x; i < 2 * tri(p + 1); i += blockDim.x) rec[i] = rec_g[i];
  for (int i = threadIdx.x; i <= p; i += blockDim.x) p2mf[i] = p2mf_g[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = blockIdx.x * (blockDim.x >> 5) + w;
  if (L >= nleaves) return;
  cplx<T> *out = outs + w * nm;
  for (int c = lane; c < nm; c += 32) out[c] = cmake<T>(0, 0);
  __syncwarp();
  const int node = leaf_node[L];
  const int b = begin[node], e = end[node];
  const T ih = inv_scale<T>(depth[node], scale_e);
  for (int base = b; base < e; base += 32) {
    int i = base + lane;
    T x = 0, y = 0, z = 0, q = 0;
    if (i < e) {
      real4<T> r = rel[i];
      x = r.x * ih;
      y = r.y * ih;
      z = r.z * ih;
      q = r.q;
    }
    T r2 = x * x + y * y + z * z;
    cplx<T> diag = cmake<T>(rec[0], 0);
    for (int m = 0; m < p; ++m) {
      if (m > 0) {
        T a = rec[2 * tri(m, m)];
        diag = cmake<T>(a * (x * diag.re - y * diag.im), a * (x * diag.im + y * diag.re));
      }
      cplx<T> s1 = diag, s2 = cmake<T>(0, 0);
      for (int l = m; l < p; ++l) {
        cplx<T> S;
        if (l == m) S = diag;
        else {
          T c0 = rec[2 * tri(l, m)], c1 = rec[2 * tri(l, m) + 1];
          S = cmake<T>(c0 * z * s1.re - c1 * r2 * s2.re, c0 * z * s1.im - c1 * r2 * s2.im);
          s2 = s1;
          s1 = S;
        }
        T f = q * p2mf[l];
        T re = warp_sum<T>(f * S.re);
        T im = warp_sum<T>(-f * S.im);
        if (lane == 0) {
          out[tri(l, m)].re += re;
          out[tri(l, m)].im += im;
        }
      }
    }
  }
  __syncwarp();
  for (int c = lane; c < nm; c += 32) mult[(size_t)node * nm + c] = out[c];
}

// The same P2M at a compile-time order (FP32) with the sum over a leaf's
// particles done by butterflies: the terms of each particle (lane) are made
// in m-major order (the recurrence's natural order) into a 32-value buffer;
// each full buffer is summed over the warp by one butterfly of 31 shuffles
// (afterwards lane k holds value k of the batch) instead of a 5-shuffle tree
// per value, and the lanes' batch sums add up over the leaf's chunks.
template <int P>
__global__ void __launch_bounds__(128) k_p2m_bfly(int nleaves, const int *__restrict__ leaf_node,
                                               const int *__restrict__ begin,
                                               const int *__restrict__ end,
                                               const uint8_t *__restrict__ depth,
                                               const real4<float> *__restrict__ rel,
                                               const float *__restrict__ rec_g,
                                               const float *__restrict__ p2mf_g, double scale_e,
                                               float *__restrict__ mult) {
  constexpr int NM = P * (P + 1) / 2, NV = 2 * NM, NB = (NV + 31) / 32;
  __shared__ float rec[(P + 1) * (P + 2)];
  __shared__ float p2mf[P + 1];
  for (int i = threadIdx.x; i < (P + 1) * (P + 2); i += blockDim.x) rec[i] = rec_g[i];
  for (int i = threadIdx.x; i <= P; i += blockDim.x) p2mf[i] = p2mf_g[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int L = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (L >= nleaves) return;
  const int node = leaf_node[L];
  const int b = begin[node], e = end[node];
  const float ih = inv_scale<float>(depth[node], scale_e);
  float acc[NB];
#pragma unroll
  for (int k = 0; k < NB; ++k) acc[k] = 0.f;
  for (int base = b; base < e; base += 32) {
    const int i = base + lane;
    float x = 0.f, y = 0.f, z = 0.f, q = 0.f;
    if (i < e) {
      const real4<float> r = rel[i];
      x = r.x * ih;
      y = r.y * ih;
      z = r.z * ih;
      q = r.q;
    }
    const float r2 = x * x + y * y + z * z;
    float u[32];
    float dre = rec[0], dim = 0.f;
#pragma unroll
    for (int m = 0; m < P; ++m) {
      if (m > 0) {
        const float a = rec[2 * tri(m, m)];
        const float nre = a * (x * dre - y * dim), nim = a * (x * dim + y * dre);
        dre = nre;
        dim = nim;
      }
      float s1re = dre, s1im = dim, s2re = 0.f, s2im = 0.f;
#pragma unroll
      for (int l = m; l < P; ++l) {
        float sre = dre, sim = dim;
        if (l > m) {
          const float c0 = rec[2 * tri(l, m)], c1 = rec[2 * tri(l, m) + 1];
          sre = c0 * z * s1re - c1 * r2 * s2re;
          sim = c0 * z * s1im - c1 * r2 * s2im;
          s2re = s1re;
          s2im = s1im;
          s1re = sre;
          s1im = sim;
        }
        const float f = q * p2mf[l];
        // value index 2 slot + part, slot the m-major place of (l, m)
        const int kr = 2 * (m * P - m * (m - 1) / 2 + (l - m));
#pragma unroll
        for (int part = 0; part < 2; ++part) {
          const int k = kr + part;
          u[k & 31] = part ? -f * sim : f * sre;
          if ((k & 31) == 31 || k == NV - 1) {
            if (k == NV - 1)            // last, partial batch: zero its tail
#pragma unroll
              for (int t = 0; t < 32; ++t)
                if (t > (k & 31)) u[t] = 0.f;
            // butterfly: the lane keeps the half whose index bit o matches
            // its lane bit and adds the partner's half; lane j ends with
            // value j of the batch summed over the warp
#pragma unroll
            for (int st = 0; st < 5; ++st) {
              const int o = 16 >> st, n = 32 >> st;
              const bool upper = (lane & o) != 0;
#pragma unroll
              for (int t = 0; t < n / 2; ++t) {
                const float send = upper ? u[t] : u[t + n / 2];
                const float keep = upper ? u[t + n / 2] : u[t];
                u[t] = keep + __shfl_xor_sync(kFull, send, o);
              }
            }
            acc[k >> 5] += u[0];
          }
        }
      }
    }
  }
  // lane k of batch bt holds m-major value 32 bt + k: slot (l, m), part
#pragma unroll
  for (int bt = 0; bt < NB; ++bt) {
    const int kv = 32 * bt + lane;
    if (kv >= NV) continue;
    int slot = kv >> 1, m = 0;
    while (slot > P - 1 - m) {
      slot -= P - m;
      ++m;
    }
    const int l = m + slot;
    mult[(size_t)node * NV + 2 * tri(l, m) + (kv & 1)] = acc[bt];
  }
}

// ---------------------------------------------------------------------------
// warp-cooperative pieces of the rotation operators
// ---------------------------------------------------------------------------

// src[c] = in[c] * e^{i m phi} for degrees < L (layout tri)
template <typename T>
__device__ __forceinline__ void load_phased(const cplx<T> *__restrict__ in, int ncoef,
                                            const uint8_t *lm, const T *ph, cplx<T> *src, int lane) {
  for (int c = lane; c < ncoef; c += 32) {
    cplx<T> v = in[c];
    int m = lm[2 * c + 1];
    T cr = ph[2 * m], ci = ph[2 * m + 1];
    src[c] = cmake<T>(v.re * cr - v.im * ci, v.re * ci + v.im * cr);
  }
}

// out(l,m') = (sum_m E[l][m'][m] Re in(l,m), sum_m O[l][m'][m] Im in(l,m))
template <typename T>
__device__ __forceinline__ cplx<T> rot_one(const T *__restrict__ E, const T *__restrict__ O,
                                           const cplx<T> *in, int l, int mp) {
  const T *er = E + sq_off(l) + mp * (l + 1);
  const T *orow = O + sq_off(l) + mp * (l + 1);
  const cplx<T> *src = in + tri(l);
  T re = 0, im = 0;
  for (int m = 0; m <= l; ++m) {
    cplx<T> s = src[m];
    re += er[m] * s.re;
    im += orow[m] * s.im;
  }
  return cmake<T>(re, im);
}

struct DirOffsets {
  int ef, of, ei, oi, ph, rp, stride;
};

// ---------------------------------------------------------------------------
// M2M rotate: aran/aransphericalseriesd-rotate.c:219-263 applied to the
// multipole (aran_development3d_m2m_rotate, arandevelopment3d.c:402-409).
// One block per internal node of the level: warp o translates child o, and
// the eight contributions are summed in child order.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) k_m2m_rotate(int cnt, int off, const int *__restrict__ child,
                             const int *__restrict__ begin, const int *__restrict__ end, int p,
                             const T *__restrict__ dirs, DirOffsets D, const T *__restrict__ vm,
                             const uint8_t *__restrict__ lm_g, cplx<T> *__restrict__ mult) {
  // one block of eight warps per node of the level, warp o translating
  // child o; the eight contributions are summed in child order
  extern __shared__ unsigned char smem_raw[];
  const int nm = tri(p);
  const int lane = threadIdx.x & 31, o = threadIdx.x >> 5;
  const int P = off + blockIdx.x;
  if (blockIdx.x >= cnt) return;
  const int c0 = child[P];
  if (c0 < 0) return;
  uint8_t *lm = smem_raw;
  cplx<T> *bufs = reinterpret_cast<cplx<T> *>(smem_raw + ((2 * tri(p + 1) + 15) & ~15));
  cplx<T> *part = bufs + (size_t)8 * 2 * nm;   // [child][coefficient]
  for (int i = threadIdx.x; i < 2 * tri(p + 1); i += blockDim.x) lm[i] = lm_g[i];
  __syncthreads();
  cplx<T> *src = bufs + (size_t)o * 2 * nm;
  cplx<T> *rot = src + nm;
  cplx<T> *out = part + (size_t)o * nm;
  const int ch = c0 + o;
  if (end[ch] == begin[ch]) {
    for (int c = lane; c < nm; c += 32) out[c] = cmake<T>(0, 0);
  } else {
    const T *tab = dirs + (size_t)o * D.stride;
    load_phased(mult + (size_t)ch * nm, nm, lm, tab + D.ph, src, lane);
    __syncwarp();
    for (int c = lane; c < nm; c += 32) rot[c] = rot_one(tab + D.ef, tab + D.of, src, lm[2 * c], lm[2 * c + 1]);
    __syncwarp();
    // vertical M2M (aran/aransphericalseriesd-translate.c:445-505)
    const T *rp = tab + D.rp;
    for (int c = lane; c < nm; c += 32) {
      int l = lm[2 * c], m = lm[2 * c + 1];
      const T *vrow = vm + (size_t)c * p;
      T re = 0, im = 0;
      for (int n = m; n <= l; ++n) {
        T f = vrow[n] * rp[l - n];
        cplx<T> r = rot[tri(n, m)];
        re += f * r.re;
        im += f * r.im;
      }
      src[c] = cmake<T>(re, im);
    }
    __syncwarp();
    for (int c = lane; c < nm; c += 32) {
      int l = lm[2 * c], mp = lm[2 * c + 1];
      cplx<T> v = rot_one(tab + D.ei, tab + D.oi, src, l, mp);
      T cr = tab[D.ph + 2 * mp], ci = -tab[D.ph + 2 * mp + 1];
      out[c] = cmake<T>(v.re * cr - v.im * ci, v.re * ci + v.im * cr);
    }
  }
  __syncthreads();
  for (int c = threadIdx.x; c < nm; c += blockDim.x) {
    cplx<T> a = cmake<T>(0, 0);
    for (int k = 0; k < 8; ++k) {
      a.re += part[(size_t)k * nm + c].re;
      a.im += part[(size_t)k * nm + c].im;
    }
    mult[(size_t)P * nm + c] = a;
  }
}

// ---------------------------------------------------------------------------
// L2L rotate: aran_development3d_l2l_rotate (arandevelopment3d.c:444-451),
// vertical part aran/aransphericalseriesd-translate.c:301-364.  One warp per
// non-empty node of the level, adding its parent's translated local.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_l2l_rotate(int cnt, int off, const int *__restrict__ parent,
                             const int *__restrict__ child, const int *__restrict__ begin,
                             const int *__restrict__ end, int p, const T *__restrict__ dirs,
                             DirOffsets D, const T *__restrict__ vl, const uint8_t *__restrict__ lm_g,
                             cplx<T> *__restrict__ loc) {
  extern __shared__ unsigned char smem_raw[];
  const int nl = tri(p + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  uint8_t *lm = smem_raw;
  cplx<T> *bufs = reinterpret_cast<cplx<T> *>(smem_raw + ((2 * nl + 15) & ~15));
  for (int i = threadIdx.x; i < 2 * nl; i += blockDim.x) lm[i] = lm_g[i];
  __syncthreads();
  const int C = off + blockIdx.x * wpb + w;
  if (C >= off + cnt) return;
  if (end[C] == begin[C]) return;
  const int P = parent[C];
  const int o = C - child[P];
  const T *tab = dirs + (size_t)o * D.stride;
  cplx<T> *src = bufs + (size_t)w * 2 * nl;
  cplx<T> *rot = src + nl;
  load_phased(loc + (size_t)P * nl, nl, lm, tab + D.ph, src, lane);
  __syncwarp();
  for (int c = lane; c < nl; c += 32) rot[c] = rot_one(tab + D.ef, tab + D.of, src, lm[2 * c], lm[2 * c + 1]);
  __syncwarp();
  const T *rp = tab + D.rp;
  for (int c = lane; c < nl; c += 32) {
    int l = lm[2 * c], m = lm[2 * c + 1];
    const T *vrow = vl + (size_t)c * (p + 1);
    T re = 0, im = 0;
    for (int n = l; n <= p; ++n) {
      T f = vrow[n] * rp[n - l];
      cplx<T> r = rot[tri(n, m)];
      re += f * r.re;
      im += f * r.im;
    }
    src[c] = cmake<T>(re, im);
  }
  __syncwarp();
  for (int c = lane; c < nl; c += 32) {
    int l = lm[2 * c], mp = lm[2 * c + 1];
    cplx<T> v = rot_one(tab + D.ei, tab + D.oi, src, l, mp);
    T cr = tab[D.ph + 2 * mp], ci = -tab[D.ph + 2 * mp + 1];
    cplx<T> cur = loc[(size_t)C * nl + c];
    cur.re += v.re * cr - v.im * ci;
    cur.im += v.re * ci + v.im * cr;
    loc[(size_t)C * nl + c] = cur;
  }
}

// ---------------------------------------------------------------------------
// L2P with gradient: aran_development3d_local_gradient_evaluate
// (arandevelopment3d.c:542-552, aransphericalseriesd.c:419-546) and the
// local evaluation of arandevelopment3d.c:485-494.  One warp per leaf (four
// leaves per block), one lane per particle.  The gradient uses the derivative identities of the
// regular solid harmonics (fmm_math.cuh gen_grad_coefs): d/dz and
// d/dx - i d/dy of a degree-p local are degree-(p-1) locals built once per
// leaf, so a particle only evaluates S_l^m(xhat) once.
// ---------------------------------------------------------------------------
// PC > 0: the order as a compile-time constant (loops unrolled, indices
// folded); PC = 0: the order p at run time
template <typename T, bool FIELD, int PC = 0>
__global__ void k_l2p(int nleaves, const int *__restrict__ leaf_node, const int *__restrict__ begin,
                      const int *__restrict__ end, const uint8_t *__restrict__ depth,
                      const real4<T> *__restrict__ rel, int p_rt, const T *__restrict__ rec_g,
                      const T *__restrict__ gz_g, const T *__restrict__ gm_g, double scale_e,
                      const cplx<T> *__restrict__ loc, double *__restrict__ acc_pot,
                      double *__restrict__ acc_fld) {
  extern __shared__ unsigned char smem_raw[];
  const int p = PC > 0 ? PC : p_rt;
  const int nl = tri(p + 1), nm = tri(p);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T *rec = reinterpret_cast<T *>(smem_raw);
  // per warp: the leaf's local, and the d/dz and d/dx - i d/dy locals
  cplx<T> *Lc = reinterpret_cast<cplx<T> *>(rec + ((2 * nl + 1) & ~1)) +
                (size_t)w * (nl + nm + p * p);
  cplx<T> *A = Lc + nl;
  cplx<T> *B = A + nm;
  for (int i = threadIdx.x; i < 2 * nl; i += blockDim.x) rec[i] = rec_g[i];
  __syncthreads();
  const int L = blockIdx.x * (blockDim.x >> 5) + w;
  if (L >= nleaves) return;
  const int node = leaf_node[L];
  for (int c = lane; c < nl; c += 32) Lc[c] = loc[(size_t)node * nl + c];
  __syncwarp();
  if (FIELD) {
    for (int c = lane; c < nm; c += 32) {
      // c = tri(l', m): A = L(l'+1, m) * gz
      // degree of the triangular index c: floor((sqrt(8c+1)-1)/2), corrected
      int lp = (int)((sqrtf(8.f * c + 1.f) - 1.f) * 0.5f);
      while (tri(lp + 1) <= c) ++lp;
      while (tri(lp) > c) --lp;
      int m = c - tri(lp);
      cplx<T> v = Lc[tri(lp + 1, m)];
      T g = gz_g[c];
      A[c] = cmake<T>(v.re * g, v.im * g);
    }
    for (int c = lane; c < p * p; c += 32) {
      int lp = (int)sqrtf((float)c);   // floor(sqrt(c)), corrected
      while ((lp + 1) * (lp + 1) <= c) ++lp;
      while (lp * lp > c) --lp;
      int mp = c - lp * lp - lp;
      int m = mp + 1;
      cplx<T> v;
      if (m >= 0) v = Lc[tri(lp + 1, m)];
      else {
        cplx<T> u = Lc[tri(lp + 1, -m)];
        v = ((-m) & 1) ? cmake<T>(-u.re, u.im) : cmake<T>(u.re, -u.im);
      }
      T g = gm_g[c];
      B[c] = cmake<T>(v.re * g, v.im * g);
    }
  }
  __syncwarp();
  const int b = begin[node], e = end[node];
  const T ih = inv_scale<T>(depth[node], scale_e);
  for (int i = b + lane; i < e; i += 32) {
    real4<T> r = rel[i];
    T x = r.x * ih, y = r.y * ih, z = r.z * ih;
    T r2 = x * x + y * y + z * z;
    T phi = 0, dz = 0, gre = 0, gim = 0;
    cplx<T> diag = cmake<T>(rec[0], 0);
#pragma unroll 1
    for (int m = 0; m <= p; ++m) {
      if (m > 0) {
        T a = rec[2 * tri(m, m)];
        diag = cmake<T>(a * (x * diag.re - y * diag.im), a * (x * diag.im + y * diag.re));
      }
      cplx<T> s1 = diag, s2 = cmake<T>(0, 0);
      const T wm = m == 0 ? (T)1 : (T)2;
      const T sg = (m & 1) ? (T)-1 : (T)1;
#pragma unroll 4
      for (int l = m; l <= p; ++l) {
        cplx<T> S;
        if (l == m) S = diag;
        else {
          T c0 = rec[2 * tri(l, m)], c1 = rec[2 * tri(l, m) + 1];
          S = cmake<T>(c0 * z * s1.re - c1 * r2 * s2.re, c0 * z * s1.im - c1 * r2 * s2.im);
          s2 = s1;
          s1 = S;
        }
        cplx<T> Lv = Lc[tri(l, m)];
        phi += wm * (Lv.re * S.re - Lv.im * S.im);
        if (FIELD && l < p) {
          cplx<T> a = A[tri(l, m)];
          dz += wm * (a.re * S.re - a.im * S.im);
          cplx<T> bp = B[l * l + l + m];
          gre += bp.re * S.re - bp.im * S.im;
          gim += bp.re * S.im + bp.im * S.re;
          if (m > 0) {
            // S^{-m} = (-1)^m conj(S^m)
            cplx<T> bn = B[l * l + l - m];
            T sre = sg * S.re, sim = -sg * S.im;
            gre += bn.re * sre - bn.im * sim;
            gim += bn.re * sim + bn.im * sre;
          }
        }
      }
    }
    acc_pot[i] += (double)phi;
    if (FIELD) {
      acc_fld[3 * (size_t)i] += (double)(gre * ih);
      acc_fld[3 * (size_t)i + 1] += (double)(-gim * ih);
      acc_fld[3 * (size_t)i + 2] += (double)(dz * ih);
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 L2P (+ gradient) over windows of 32 consecutive particles (leaf
// order), the order P a compile-time constant: the same evaluation as k_l2p,
// with every lane busy whatever the leaves' sizes.  Warp w takes particles
// 32 w .. 32 w + 31, which belong to leaves win_leaf[w] onwards (at most
// 32 of them); each lane evaluates with its own leaf's coefficients, staged
// four leaves at a time in shared memory: the local with the m-weight
// (2 for m > 0) folded in and, for the gradient, the d/dz local and the
// (d/dx - i d/dy) local's m' = m and m' = -m parts combined per (l, m) into
// the two real vectors that multiply (Re S, Im S) for its real and
// imaginary parts (S^{-m} = (-1)^m conj(S^m)).  Each term is formed, then
// added to its sum once.  The solid harmonics run by degree (outer,
// unrolled) and order (inner), so every table offset is a constant.
// ---------------------------------------------------------------------------
constexpr int kWinSlots = 4;     // leaves staged at a time per warp
constexpr int kWinWarps = 4;     // warps per block

template <int P, bool FIELD>
__host__ __device__ constexpr int win_slot() {   // float2 per staged leaf
  return (P + 1) * (P + 2) / 2 + (FIELD ? 3 * (P * (P + 1) / 2) : 0);
}

template <int P, bool FIELD>
__global__ void __launch_bounds__(32 * kWinWarps)
    k_l2p_win(int64_t n, int nleaves, const int *__restrict__ win_leaf,
              const int *__restrict__ leaf_node, const int *__restrict__ begin,
              const uint8_t *__restrict__ depth, const real4<float> *__restrict__ rel,
              const float *__restrict__ rec_g, const float *__restrict__ gz_g,
              const float *__restrict__ gm_g, double scale_e, const cplx<float> *__restrict__ loc,
              double *__restrict__ acc_pot, double *__restrict__ acc_fld) {
  constexpr int NL = (P + 1) * (P + 2) / 2, NM = P * (P + 1) / 2;
  constexpr int SLOT = win_slot<P, FIELD>();
  __shared__ __align__(8) float rec[2 * NL];
  __shared__ uint8_t lmt[2 * NL];
  __shared__ float2 coef[kWinWarps][kWinSlots][SLOT];
  for (int i = threadIdx.x; i < 2 * NL; i += blockDim.x) rec[i] = rec_g[i];
  for (int c = threadIdx.x; c < NL; c += blockDim.x) {
    int l = 0;
    while ((l + 1) * (l + 2) / 2 <= c) ++l;
    lmt[2 * c] = (uint8_t)l;
    lmt[2 * c + 1] = (uint8_t)(c - l * (l + 1) / 2);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t wid = (int64_t)blockIdx.x * kWinWarps + w;
  const int64_t j0 = wid * 32;
  if (j0 >= n) return;
  // the window's leaves: lane k holds leaf win_leaf + k (node, first particle)
  const int L0 = win_leaf[wid];
  int nd_k = -1;
  int64_t b_k = INT64_MAX;
  if (L0 + lane < nleaves) {
    nd_k = leaf_node[L0 + lane];
    b_k = begin[nd_k];
  }
  // bit i: particle j0 + i starts a leaf after the window's first
  const unsigned bit = (lane >= 1 && b_k > j0 && b_k < j0 + 32) ? 1u << (int)(b_k - j0) : 0u;
  const unsigned M = __reduce_or_sync(kFull, bit);
  const int nslots = __popc(M) + 1;
  const int64_t j = j0 + lane;
  const bool act = j < n;
  const int slot = __popc(M & ((2u << lane) - 1u));
  const int nd = __shfl_sync(kFull, nd_k, slot);
  const float ih = inv_scale<float>(act ? depth[nd] : 0, scale_e);
  const real4<float> r = act ? rel[j] : real4<float>{0.f, 0.f, 0.f, 0.f};
  const float x = r.x * ih, y = r.y * ih, z = r.z * ih;
  const float r2 = x * x + y * y + z * z;
  float phi = 0.f, dz = 0.f, gre = 0.f, gim = 0.f;
  for (int g0 = 0; g0 < nslots; g0 += kWinSlots) {
    // stage leaves g0 .. g0 + 3 of the window
    __syncwarp();
    for (int sidx = 0; sidx < kWinSlots && g0 + sidx < nslots; ++sidx) {
      const int node = __shfl_sync(kFull, nd_k, g0 + sidx);
      const cplx<float> *Lg = loc + (size_t)node * NL;
      float2 *cf = coef[w][sidx];
      for (int c = lane; c < NL; c += 32) {
        const cplx<float> v = Lg[c];
        const float wm = lmt[2 * c + 1] ? 2.f : 1.f;
        cf[c] = make_float2(wm * v.re, wm * v.im);
      }
      if (FIELD)
        for (int c = lane; c < NM; c += 32) {
          const int l = lmt[2 * c], m = lmt[2 * c + 1];
          const float wm = m ? 2.f : 1.f;
          // d/dz: L(l+1, m) gz
          const cplx<float> a = Lg[(l + 1) * (l + 2) / 2 + m];
          const float gz = gz_g[c];
          cf[NL + c] = make_float2(wm * gz * a.re, wm * gz * a.im);
          // (d/dx - i d/dy), m' = m: bp = L(l+1, m+1) gm[l^2 + l + m]
          const cplx<float> vp = Lg[(l + 1) * (l + 2) / 2 + m + 1];
          const float gp = gm_g[l * l + l + m];
          const float bpr = gp * vp.re, bpi = gp * vp.im;
          // m' = -m (m > 0): source order 1 - m, times (-1)^m for S^{-m}
          float bnr = 0.f, bni = 0.f;
          if (m > 0) {
            const float gn = gm_g[l * l + l - m];
            cplx<float> u;
            if (m == 1) u = Lg[(l + 1) * (l + 2) / 2];
            else {
              const cplx<float> v = Lg[(l + 1) * (l + 2) / 2 + m - 1];
              u = ((m - 1) & 1) ? cmake<float>(-v.re, v.im) : cmake<float>(v.re, -v.im);
            }
            const float sg = (m & 1) ? -gn : gn;
            bnr = sg * u.re;
            bni = sg * u.im;
          }
          // real part bp S + bn conj(S): (bpr + bnr) Re S + (bni - bpi) Im S;
          // imaginary part: (bpi + bni) Re S + (bpr - bnr) Im S
          cf[NL + NM + c] = make_float2(bpr + bnr, bni - bpi);
          cf[NL + 2 * NM + c] = make_float2(bpi + bni, bpr - bnr);
        }
    }
    __syncwarp();
    if (act && slot >= g0 && slot < g0 + kWinSlots) {
      const float2 *cf = coef[w][slot - g0];
      // s1[m] = S_{l-1}^m, s2[m] = S_{l-2}^m
      float s1r[P + 1], s1i[P + 1], s2r[P + 1], s2i[P + 1];
#pragma unroll
      for (int l = 0; l <= P; ++l) {
        // the diagonal term first: S_l^l = a_l (x + i y) S_{l-1}^{l-1}
        float Sr, Si;
        if (l == 0) {
          Sr = rec[0];
          Si = 0.f;
        } else {
          const float a = rec[2 * (l * (l + 1) / 2 + l)];
          Sr = a * (x * s1r[l - 1] - y * s1i[l - 1]);
          Si = a * (x * s1i[l - 1] + y * s1r[l - 1]);
        }
        float dr[P + 1], di[P + 1];
        dr[l] = Sr;
        di[l] = Si;
#pragma unroll
        for (int m = 0; m < l; ++m) {
          const float2 cc = *reinterpret_cast<const float2 *>(&rec[2 * (l * (l + 1) / 2 + m)]);
          const float t0 = cc.x * z, t1 = cc.y * r2;
          const float pr = m + 1 < l ? s2r[m] : 0.f, pi = m + 1 < l ? s2i[m] : 0.f;
          dr[m] = t0 * s1r[m] - t1 * pr;
          di[m] = t0 * s1i[m] - t1 * pi;
        }
#pragma unroll
        for (int m = 0; m <= l; ++m) {
          const int c = l * (l + 1) / 2 + m;
          const float Sr_ = dr[m], Si_ = di[m];
          const float2 Lv = cf[c];
          phi += fmaf(Lv.x, Sr_, -Lv.y * Si_);
          if (FIELD && l < P) {
            const float2 a = cf[NL + c];
            dz += fmaf(a.x, Sr_, -a.y * Si_);
            const float2 gr = cf[NL + NM + c], gi = cf[NL + 2 * NM + c];
            gre += fmaf(gr.x, Sr_, gr.y * Si_);
            gim += fmaf(gi.x, Sr_, gi.y * Si_);
          }
          if (m < l) {
            s2r[m] = s1r[m];
            s2i[m] = s1i[m];
          }
          s1r[m] = Sr_;
          s1i[m] = Si_;
        }
      }
    }
  }
  if (act) {
    acc_pot[j] += (double)phi;
    if (FIELD) {
      acc_fld[3 * j] += (double)(gre * ih);
      acc_fld[3 * j + 1] += (double)(-gim * ih);
      acc_fld[3 * j + 2] += (double)(dz * ih);
    }
  }
}

__global__ void k_scatter(int64_t n, const int *__restrict__ perm, const double *__restrict__ acc_pot,
                          const double *__restrict__ acc_fld, double *__restrict__ pot,
                          double *__restrict__ fld) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  if (pot) pot[o] = acc_pot[i];
  if (fld) {
    fld[3 * (int64_t)o] = acc_fld[3 * i];
    fld[3 * (int64_t)o + 1] = acc_fld[3 * i + 1];
    fld[3 * (int64_t)o + 2] = acc_fld[3 * i + 2];
  }
}

// counters of aran_solver3d_get_stats from the lists
__global__ void k_stats(int nn, int nleaves, const int *__restrict__ begin, const int *__restrict__ end,
                        const int *__restrict__ parent, const int *__restrict__ leaf_node,
                        const int *__restrict__ near_off, const int *__restrict__ near_rng,
                        int nsemi, const int *__restrict__ semi_leaf,
                        unsigned long long *__restrict__ st) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long m2m = 0, p2p2 = 0;
  if (i < nn && end[i] > begin[i] && parent[i] >= 0) m2m = 1;
  if (i < nsemi) {
    // semifar_func counts the coarse leaf's points once for p2l and m2p
    int a = leaf_node[semi_leaf[i]];
    atomicAdd(&st[2], (unsigned long long)(end[a] - begin[a]));
  }
  if (i < nleaves) {
    int node = leaf_node[i];
    long long nt = end[node] - begin[node];
    for (int r = near_off[i]; r < near_off[i + 1]; ++r)
      for (int lf = near_rng[2 * r]; lf < near_rng[2 * r + 1]; ++lf) {
        int sn = leaf_node[lf];
        long long ns = end[sn] - begin[sn];
        if (sn == node) p2p2 += (unsigned long long)(nt * (nt + 1));  // 2 * n(n+1)/2
        else p2p2 += (unsigned long long)(nt * ns);                  // counted from both sides
      }
  }
  if (m2m) atomicAdd(&st[0], m2m);
  if (p2p2) atomicAdd(&st[1], p2p2);
}

template <typename T>
DirOffsets offsets(int p, int kind) {
  DirOffsets d;
  d.ef = dir_offset(p, kind, 0);
  d.of = dir_offset(p, kind, 1);
  d.ei = dir_offset(p, kind, 2);
  d.oi = dir_offset(p, kind, 3);
  d.ph = dir_offset(p, kind, 4);
  d.rp = dir_offset(p, kind, 5);
  d.stride = dir_offset(p, kind, 6);
  return d;
}

// M2M into the parents of depths dhi down to dlo (deepest first)
template <typename T>
void m2m_levels(AranGpuSolver3d *s, OpTables<T> &tb, cplx<T> *mult, int dhi, int dlo,
                cudaStream_t st) {
  DevTree &t = s->tree;
  const int p = s->cfg.order;
  const int nm = tri(p), nl = tri(p + 1);
  if constexpr (sizeof(T) == 4)
    if (launch_m2m_lanes(s, tb, mult, dhi, dlo, st)) return;
  DirOffsets D = offsets<T>(p, 1);
  size_t sm = ((2 * nl + 15) & ~15) + (size_t)8 * 3 * nm * sizeof(cplx<T>) + 64;
  smem_opt_in(k_m2m_rotate<T>, sm);
  for (int d = dhi; d >= dlo; --d) {
    if (d < 0 || d > t.nlevels - 2 || t.level_internal[d] == 0) continue;
    int off = t.level_off[d], cnt = t.level_off[d + 1] - off;
    k_m2m_rotate<T><<<cnt, 256, sm, st>>>(cnt, off, t.child.ptr, t.begin.ptr, t.end.ptr, p,
                                          tb.dir_m2m.ptr, D, tb.vm.ptr, tb.lm.ptr, mult);
    ACHECK(cudaGetLastError());
    s->launches++;
  }
}

// L2L into the nodes of depths dlo up to dhi (from depth 3: locals of depths
// 0-1 are zero, no far pairs above depth 2)
template <typename T>
void l2l_levels(AranGpuSolver3d *s, OpTables<T> &tb, cplx<T> *loc, int dlo, int dhi,
                cudaStream_t st) {
  DevTree &t = s->tree;
  const int p = s->cfg.order;
  const int nl = tri(p + 1);
  if constexpr (sizeof(T) == 4)
    if (launch_l2l_lanes(s, tb, loc, dlo, dhi, st)) return;
  DirOffsets D = offsets<T>(p, 2);
  const int WPB = 4;
  size_t sm = ((2 * nl + 15) & ~15) + (size_t)WPB * 2 * nl * sizeof(cplx<T>) + 64;
  smem_opt_in(k_l2l_rotate<T>, sm);
  for (int d = dlo < 3 ? 3 : dlo; d <= dhi && d < t.nlevels; ++d) {
    int off = t.level_off[d], cnt = t.level_off[d + 1] - off;
    k_l2l_rotate<T><<<ceil_div(cnt, WPB), WPB * 32, sm, st>>>(
        cnt, off, t.parent.ptr, t.child.ptr, t.begin.ptr, t.end.ptr, p, tb.dir_l2l.ptr, D,
        tb.vl.ptr, tb.lm.ptr, loc);
    ACHECK(cudaGetLastError());
    s->launches++;
  }
}

// b[i] = (float) a[i] (WIDEN false) or b[i] (+)= (double) a[i] (WIDEN true)
template <bool WIDEN, bool ADD>
__global__ void k_convert(int64_t n, const void *__restrict__ a, void *__restrict__ b) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (WIDEN) {
    double v = (double)static_cast<const float *>(a)[i];
    double *o = static_cast<double *>(b);
    o[i] = ADD ? o[i] + v : v;
  } else {
    static_cast<float *>(b)[i] = (float)static_cast<const double *>(a)[i];
  }
}

template <bool WIDEN, bool ADD>
void convert(AranGpuSolver3d *s, int64_t n, const void *a, void *b, cudaStream_t st) {
  if (n <= 0) return;
  k_convert<WIDEN, ADD><<<ceil_div(n, 256), 256, 0, st>>>(n, a, b);
  ACHECK(cudaGetLastError());
  s->launches++;
}

template <typename T>
void run_passes_t(AranGpuSolver3d *s, OpTables<T> &tb, DBuf<T> &multb, DBuf<T> &locb,
                  const real4<T> *rel) {
  cudaStream_t st = s->s0;
  DevTree &t = s->tree;
  const int p = s->cfg.order;
  const int nm = tri(p), nl = tri(p + 1);
  const bool field = s->cfg.field != 0;
  const bool kk = s->cfg.flavour == ARAN_FLAVOUR_KKYLIN;
  multb.reserve((size_t)t.nnodes * nm * 2);
  locb.reserve((size_t)t.nnodes * nl * 2);
  cplx<T> *mult = reinterpret_cast<cplx<T> *>(multb.ptr);
  cplx<T> *loc = reinterpret_cast<cplx<T> *>(locb.ptr);
  s->acc_pot.reserve(t.n);
  s->acc_fld.reserve(3 * t.n);
  // FP64 root levels of the mixed rotation path: nodes of depth <= R keep
  // FP64 expansions (the first n_root nodes, level-major order); M2M into
  // them, M2L at them and L2L between them run in FP64
  const int R = (sizeof(T) == 4 && !kk && s->root64_depth >= 0)
                    ? (s->root64_depth < t.nlevels - 1 ? s->root64_depth : t.nlevels - 1)
                    : -1;
  const int n_root = R >= 0 ? t.level_off[R + 1] : 0;
  const int n_root_src = R >= 0 ? t.level_off[R + 2 < t.nlevels ? R + 2 : t.nlevels] : 0;
  int n_root_parents = 0;   // parents of depth < R: their children have depth <= R
  for (int d = 1; d < R; ++d) n_root_parents += t.level_internal[d];
  cplx<double> *mult64 = nullptr, *loc64 = nullptr;
  if (R >= 0) {
    build_tables_fp64(s);
    s->mult64.reserve((size_t)n_root_src * nm * 2);
    s->loc64.reserve((size_t)n_root * nl * 2);
    mult64 = reinterpret_cast<cplx<double> *>(s->mult64.ptr);
    loc64 = reinterpret_cast<cplx<double> *>(s->loc64.ptr);
  }

  // near field on the second stream, as soon as the lists exist
  ACHECK(cudaStreamWaitEvent(s->s1, s->ev[2 * Stage::LISTS + 1], 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P], s->s1));
  launch_p2p(s, s->s1);
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P + 1], s->s1));

  // clear (aran/aransolver3d.c:399-410)
  ACHECK(cudaMemsetAsync(multb.ptr, 0, (size_t)t.nnodes * nm * 2 * sizeof(T), st));
  ACHECK(cudaMemsetAsync(locb.ptr, 0, (size_t)t.nnodes * nl * 2 * sizeof(T), st));
  if (R >= 0) ACHECK(cudaMemsetAsync(s->loc64.ptr, 0, (size_t)n_root * nl * 2 * sizeof(double), st));

  // P2M
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M], st));
  {
    const int WPB = 4;
    if (sizeof(T) == 4 && p == 12) {
      k_p2m_bfly<12><<<ceil_div(t.nleaves, WPB), WPB * 32, 0, st>>>(
          t.nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr, t.depth.ptr,
          reinterpret_cast<const real4<float> *>(rel), reinterpret_cast<const float *>(tb.rec.ptr),
          reinterpret_cast<const float *>(tb.p2mf.ptr), s->scale_e,
          reinterpret_cast<float *>(mult));
    } else {
      size_t sm = (2 * nl + p + 2) * sizeof(T) + (size_t)WPB * nm * sizeof(cplx<T>) + 64;
      smem_opt_in(k_p2m<T>, sm);
      k_p2m<T><<<ceil_div(t.nleaves, WPB), WPB * 32, sm, st>>>(
          t.nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr, t.depth.ptr, rel, p, tb.rec.ptr,
          tb.p2mf.ptr, s->scale_e, mult);
    }
    ACHECK(cudaGetLastError());
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M + 1], st));
  // M2M, deepest level first
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M], st));
  if (kk) kkylin_pass(s, 0);
  else if (R < 0) m2m_levels<T>(s, tb, mult, t.nlevels - 2, 0, st);
  else {
    // FP32 up to the children of depth-R parents, widened, then FP64; the
    // FP64 multipoles of depths <= R go back to FP32 for the semifar M2P
    m2m_levels<T>(s, tb, mult, t.nlevels - 2, R + 1, st);
    convert<true, false>(s, (int64_t)n_root_src * nm * 2, multb.ptr, s->mult64.ptr, st);
    m2m_levels<double>(s, s->t64, mult64, R, 0, st);
    convert<false, false>(s, (int64_t)n_root * nm * 2, s->mult64.ptr, multb.ptr, st);
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M + 1], st));
  // M2L over every node of depth >= 2
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L], st));
  if (kk) kkylin_pass(s, 1);
  else if (R < 0) launch_m2l(s, sizeof(T) == 8, 0, t.n_parents, st);
  else {
    launch_m2l(s, true, 0, n_root_parents, st);
    launch_m2l(s, false, n_root_parents, t.n_parents - n_root_parents, st);
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SEMI_P2L], st));
  launch_semifar_p2l(s, st);
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SEMI_P2L + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L + 1], st));
  // L2L
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L], st));
  if (kk) kkylin_pass(s, 2);
  else if (R < 0) l2l_levels<T>(s, tb, loc, 3, t.nlevels - 1, st);
  else {
    // the FP32 locals of depths <= R hold only semifar P2L terms: added to
    // the FP64 ones, carried down in FP64, narrowed back for the deeper levels
    convert<true, true>(s, (int64_t)n_root * nl * 2, locb.ptr, s->loc64.ptr, st);
    l2l_levels<double>(s, s->t64, loc64, 3, R, st);
    convert<false, false>(s, (int64_t)n_root * nl * 2, s->loc64.ptr, locb.ptr, st);
    l2l_levels<T>(s, tb, loc, R + 1, t.nlevels - 1, st);
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L + 1], st));
  // L2P after the near field has written the accumulators
  ACHECK(cudaStreamWaitEvent(st, s->ev[2 * Stage::P2P + 1], 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P], st));
  {
    constexpr int LPB = 4;   // leaves (warps) per block
    size_t sm = ((2 * nl + 1) & ~1) * sizeof(T) +
                (size_t)LPB * (nl + nm + p * p) * sizeof(cplx<T>) + 64;
    smem_opt_in(k_l2p<T, true>, sm);
    smem_opt_in(k_l2p<T, false>, sm);
    const int nb = ceil_div(t.nleaves, LPB);
    if (sizeof(T) == 4 && m2l_lane_order(p)) {
      // windows of 32 particles, the order folded in at compile time
      const int64_t nw = (t.n + 31) / 32;
      const int nbw = (int)ceil_div(nw, (int64_t)kWinWarps);
      auto run = [&](auto kern) {
        if (nbw == 0) return;
        kern<<<nbw, 32 * kWinWarps, 0, st>>>(
            t.n, t.nleaves, t.win_leaf.ptr, t.leaf_node.ptr, t.begin.ptr, t.depth.ptr,
            reinterpret_cast<const real4<float> *>(rel), reinterpret_cast<const float *>(tb.rec.ptr),
            reinterpret_cast<const float *>(tb.gz.ptr), reinterpret_cast<const float *>(tb.gm.ptr),
            s->scale_e, reinterpret_cast<const cplx<float> *>(loc), s->acc_pot.ptr, s->acc_fld.ptr);
      };
      if (field) {
        if (p == 4) run(k_l2p_win<4, true>);
        else if (p == 8) run(k_l2p_win<8, true>);
        else run(k_l2p_win<12, true>);
      } else {
        if (p == 4) run(k_l2p_win<4, false>);
        else if (p == 8) run(k_l2p_win<8, false>);
        else run(k_l2p_win<12, false>);
      }
    } else if (sizeof(T) == 4 && field && (p == 8 || p == 12)) {
      // the bench orders with the order folded in at compile time
      auto kern = p == 8 ? k_l2p<T, true, 8> : k_l2p<T, true, 12>;
      smem_opt_in(kern, sm);
      kern<<<nb, 32 * LPB, sm, st>>>(t.nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                     t.depth.ptr, rel, p, tb.rec.ptr, tb.gz.ptr, tb.gm.ptr,
                                     s->scale_e, loc, s->acc_pot.ptr, s->acc_fld.ptr);
    } else if (field)
      k_l2p<T, true><<<nb, 32 * LPB, sm, st>>>(t.nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                                 t.depth.ptr, rel, p, tb.rec.ptr, tb.gz.ptr,
                                                 tb.gm.ptr, s->scale_e, loc, s->acc_pot.ptr,
                                                 s->acc_fld.ptr);
    else
      k_l2p<T, false><<<nb, 32 * LPB, sm, st>>>(t.nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                                  t.depth.ptr, rel, p, tb.rec.ptr, tb.gz.ptr,
                                                  tb.gm.ptr, s->scale_e, loc, s->acc_pot.ptr,
                                                  s->acc_fld.ptr);
    ACHECK(cudaGetLastError());
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SEMI_M2P], st));
  launch_semifar_m2p(s, st);
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SEMI_M2P + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P + 1], st));
}

}  // namespace

void run_passes(AranGpuSolver3d *s) {
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    run_passes_t<float>(s, s->t32, s->mult32, s->loc32, s->rel32.ptr);
  else
    run_passes_t<double>(s, s->t64, s->mult64, s->loc64, s->rel64.ptr);
}

void scatter_outputs(AranGpuSolver3d *s, double *pot, double *fld) {
  const int TB = 256;
  k_scatter<<<ceil_div(s->tree.n, TB), TB, 0, s->s0>>>(s->tree.n, s->perm.ptr, s->acc_pot.ptr,
                                                        s->cfg.field ? s->acc_fld.ptr : nullptr,
                                                        pot, s->cfg.field ? fld : nullptr);
  ACHECK(cudaGetLastError());
  s->launches++;
}

void compute_stats(AranGpuSolver3d *s) {
  DevTree &t = s->tree;
  count_far_lists(s);
  s->stats_dev.reserve(3);
  ACHECK(cudaMemsetAsync(s->stats_dev.ptr, 0, 3 * sizeof(unsigned long long), s->s0));
  int nmax = t.nnodes > t.nleaves ? t.nnodes : t.nleaves;
  if (t.n_semi > nmax) nmax = t.n_semi;
  k_stats<<<ceil_div(nmax, 256), 256, 0, s->s0>>>(t.nnodes, t.nleaves, t.begin.ptr, t.end.ptr,
                                                  t.parent.ptr, t.leaf_node.ptr, t.near_off.ptr,
                                                  t.near_rng.ptr, t.n_semi, t.semi_leaf.ptr,
                                                  s->stats_dev.ptr);
  ACHECK(cudaGetLastError());
  unsigned long long h[3];
  ACHECK(cudaMemcpyAsync(h, s->stats_dev.ptr, sizeof(h), cudaMemcpyDeviceToHost, s->s0));
  ACHECK(cudaStreamSynchronize(s->s0));
  int64_t *st = s->stats;
  for (int i = 0; i < 11; ++i) st[i] = 0;
  st[0] = t.nnodes;          // zero
  st[1] = (int64_t)(h[1] / 2);  // p2p
  st[2] = t.n;               // p2m
  st[3] = (int64_t)h[0];     // m2m
  st[4] = t.n_far;           // m2l
  st[5] = (int64_t)h[0];     // l2l
  st[6] = t.n;               // l2p
  st[7] = (int64_t)h[2];     // p2l (semifar)
  st[8] = (int64_t)h[2];     // m2p (semifar)
}

namespace {
template <typename T>
__global__ void k_unscale(int nn, int p, const uint8_t *__restrict__ depth, double scale_e,
                          const cplx<T> *__restrict__ mult, const cplx<T> *__restrict__ loc,
                          double *__restrict__ om, double *__restrict__ ol) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  int nm = tri(p), nl = tri(p + 1);
  double h = scale_e / ldexp(1.0, depth[i]);
  for (int l = 0; l <= p; ++l) {
    double hm = pow(h, l), hl = 1.0 / hm;
    for (int m = 0; m <= l; ++m) {
      if (l < p && om) {
        cplx<T> v = mult[(size_t)i * nm + tri(l, m)];
        om[2 * ((size_t)i * nm + tri(l, m))] = (double)v.re * hm;
        om[2 * ((size_t)i * nm + tri(l, m)) + 1] = (double)v.im * hm;
      }
      if (ol) {
        cplx<T> v = loc[(size_t)i * nl + tri(l, m)];
        ol[2 * ((size_t)i * nl + tri(l, m))] = (double)v.re * hl;
        ol[2 * ((size_t)i * nl + tri(l, m)) + 1] = (double)v.im * hl;
      }
    }
  }
}
}  // namespace

void copy_expansions(AranGpuSolver3d *s, double *mult, double *local) {
  DevTree &t = s->tree;
  int p = s->cfg.order;
  size_t nm = tri(p), nl = tri(p + 1);
  DBuf<double> om, ol;
  om.reserve(t.nnodes * nm * 2);
  ol.reserve(t.nnodes * nl * 2);
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    k_unscale<float><<<ceil_div(t.nnodes, 128), 128, 0, s->s0>>>(
        t.nnodes, p, t.depth.ptr, s->scale_e, reinterpret_cast<cplx<float> *>(s->mult32.ptr),
        reinterpret_cast<cplx<float> *>(s->loc32.ptr), om.ptr, ol.ptr);
  else
    k_unscale<double><<<ceil_div(t.nnodes, 128), 128, 0, s->s0>>>(
        t.nnodes, p, t.depth.ptr, s->scale_e, reinterpret_cast<cplx<double> *>(s->mult64.ptr),
        reinterpret_cast<cplx<double> *>(s->loc64.ptr), om.ptr, ol.ptr);
  ACHECK(cudaGetLastError());
  if (mult) ACHECK(cudaMemcpyAsync(mult, om.ptr, t.nnodes * nm * 2 * sizeof(double), cudaMemcpyDeviceToHost, s->s0));
  if (local) ACHECK(cudaMemcpyAsync(local, ol.ptr, t.nnodes * nl * 2 * sizeof(double), cudaMemcpyDeviceToHost, s->s0));
  ACHECK(cudaStreamSynchronize(s->s0));
  om.release();
  ol.release();
}

}  // namespace aran
