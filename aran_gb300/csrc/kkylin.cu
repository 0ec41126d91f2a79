// kkylin.cu -- the K. Kylin flavour of M2M / M2L / L2L on the device
// (aran_development3d_{m2m,m2l,l2l}_kkylin, aran/arandevelopment3d.c:343-388;
// algorithms of aran/aransphericalseriesd-kkylin.c).
//
// These translations run recurrences on partial sums instead of rotating the
// series: for every output degree l the partial sums P[m][n] over the source
// degree n are built from two direct sums and a three-term recurrence in m,
// then summed over n.  They are restated here term for term, in the scaled
// storage of the device (distances in units of the level scale; outputs
// multiplied by 2^-l for M2M/L2L and 1/h for M2L), with per-direction tables
// (r, cos/sin theta, cos/sin phi and Y_j^m of the direction up to the degree
// the reference evaluates) generated once on the device in FP64.  One warp
// per target node (M2L, L2L) or parent (M2M): lane n owns the partial sums of
// source degree n in shared memory.  This flavour is kept for parity with the
// reference; the rotate flavour is the fast path.
#include "internal.cuh"

namespace aran {

namespace {

struct KkLayout {
  int Lh;       // harmonics degree
  int h;        // offset of harmonics (complex, interleaved)
  int stride;   // T per direction
};

__host__ __device__ KkLayout kk_layout(int p, int kind) {
  KkLayout k;
  k.Lh = kind == 0 ? 2 * p : p;
  k.h = 8;  // [0..4] = r, cost, sint, cosp, sinp
  k.stride = (k.h + 2 * tri(k.Lh + 1) + 3) & ~3;
  return k;
}

// Y_l^m (m >= 0, l <= L) by aran/aransphericalharmonic.c:149-184 (FP64)
__device__ void harmonics_d(int L, double cost, double sint, double cosp, double sinp,
                            const double *nrm, double *leg, double *out) {
  leg[0] = 1.;
  if (L > 0) {
    leg[tri(1, 0)] = cost;
    leg[tri(1, 1)] = -sint;
    for (int i = 2; i <= L; ++i) {
      for (int j = 0; j < i - 1; ++j)
        leg[tri(i, j)] = ((i + i - 1) * cost * leg[tri(i - 1, j)] - (i + j - 1) * leg[tri(i - 2, j)]) / (i - j);
      leg[tri(i, i - 1)] = (i + i - 1) * cost * leg[tri(i - 1, i - 1)];
      leg[tri(i, i)] = -(i + i - 1) * sint * leg[tri(i - 1, i - 1)];
    }
  }
  for (int i = 0; i <= L; ++i) {
    double er = 1., ei = 0.;
    for (int j = 0; j <= i; ++j) {
      double f = leg[tri(i, j)] * nrm[tri(i, j)];
      out[2 * tri(i, j)] = er * f;
      out[2 * tri(i, j) + 1] = ei * f;
      double nr = er * cosp - ei * sinp, ni = er * sinp + ei * cosp;
      er = nr;
      ei = ni;
    }
  }
}

template <typename T>
__global__ void k_kk_tables(int p, int kind, int ndir, double ex, double ey, double ez,
                            double *scratch, int sstride, T *out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ndir) return;
  KkLayout L = kk_layout(p, kind);
  T *o = out + (size_t)k * L.stride;
  double v[3];
  if (kind == 0) {
    int dx = k % 7 - 3, dy = (k / 7) % 7 - 3, dz = k / 49 - 3;
    if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1) {
      for (int i = 0; i < L.stride; ++i) o[i] = (T)0;
      return;
    }
    v[0] = dx * ex; v[1] = dy * ey; v[2] = dz * ez;                 // target - source
  } else {
    double sgn = (kind == 1) ? -0.5 : 0.25;                         // parent-child / child-parent
    v[0] = sgn * ((k & 1) ? 1. : -1.) * ex;
    v[1] = sgn * ((k & 2) ? 1. : -1.) * ey;
    v[2] = sgn * ((k & 4) ? 1. : -1.) * ez;
  }
  // vsg_vector3d_to_spherical_internal restated (see the oracle)
  double rho2 = v[0] * v[0] + v[1] * v[1], rho = sqrt(rho2);
  double r = sqrt(rho2 + v[2] * v[2]);
  double cost = v[2] / r, sint = rho / r;
  double cosp = rho > 0. ? v[0] / rho : 1., sinp = rho > 0. ? v[1] / rho : 0.;
  if (kind == 1) {  // multipole translate gets (r, -cost, sint, -cosp, -sinp)
    cost = -cost;
    cosp = -cosp;
    sinp = -sinp;
  }
  o[0] = (T)r;
  o[1] = (T)cost;
  o[2] = (T)sint;
  o[3] = (T)cosp;
  o[4] = (T)sinp;
  o[5] = o[6] = o[7] = (T)0;
  double *nrm = scratch + (size_t)k * sstride;
  double *leg = nrm + tri(L.Lh + 1);
  double *hh = leg + tri(L.Lh + 1);
  gen_hnorm(L.Lh, nrm);
  harmonics_d(L.Lh, cost, sint, cosp, sinp, nrm, leg, hh);
  for (int i = 0; i < 2 * tri(L.Lh + 1); ++i) o[L.h + i] = (T)hh[i];
}

template <typename T>
__device__ __forceinline__ cplx<T> ld(const T *a, int i) {
  return cmake<T>(a[2 * i], a[2 * i + 1]);
}

// (-1)^m conj(z): aran/aransphericalseriesd-private.h:91-99
template <typename T>
__device__ __forceinline__ cplx<T> sph_sym(cplx<T> z, int m) {
  return (m & 1) ? cmake<T>(-z.re, z.im) : cmake<T>(z.re, -z.im);
}

template <typename T>
__device__ __forceinline__ void cfma(cplx<T> &acc, cplx<T> a, cplx<T> b, T s) {
  acc.re += s * (a.re * b.re - a.im * b.im);
  acc.im += s * (a.re * b.im + a.im * b.re);
}

template <typename T>
__device__ __forceinline__ T ipow(T x, int e) {
  T r = (T)1;
  for (int i = 0; i < e; ++i) r *= x;
  return r;
}

// All three operators are warp-cooperative: lane n owns column n of the
// partial sums P[m][n] (shared memory, row-major [m][n] with row length W),
// lane m forms the output of order m.  src/out live in shared memory.

// M2L: aran/aransphericalseriesd-kkylin.c:364-517, with the vertical case of
// aran/aransphericalseriesd-translate.c:609-676 when |sin theta| < 1e-5.
// out accumulates the (unscaled-by-1/h) local.  One half-warp per source
// (hl = lane within the half): both halves walk
// the degrees l together (the __syncwarp calls are warp-wide), each with its
// own source, table, partial sums and output (lane hl owns the source
// degrees hl and hl + 16); a half whose direction is vertical takes the
// direct case and idles through the recurrence.  The
// ratios alpha(n)/alpha(l+n) use the reciprocal table and the radial powers
// a running product instead of a division and a power per term.
template <typename T>
__device__ void kk_m2l_half(int p, bool active, const cplx<T> *src, const T *tab, const T *alpha,
                            const T *ialpha, const T *beta, const T *vt, cplx<T> *P, cplx<T> *Q,
                            cplx<T> *out, int hl) {
  const T r = tab[0], cost = tab[1], sint = tab[2], cosp = tab[3], sinp = tab[4];
  const T *H = tab + 8;
  const T inv_r = (T)1 / r;
  const int nl = tri(p + 1);
  const bool vert = active && fabs((double)sint) < 1.e-5;
  if (vert) {
    for (int c = hl; c < nl; c += 16) {
      int l = 0;
      while (tri(l + 1) <= c) ++l;
      int m = c - tri(l);
      cplx<T> sum = cmake<T>(0, 0);
      T rp = ipow(inv_r, l + m + 1);
      for (int n = m; n < p; ++n, rp *= inv_r) {
        const int k = l + n + 1;
        const T f = vt[c * p + n] * ((k % 2 == 0) ? rp * cost : rp);
        sum.re += f * src[tri(n, m)].re;
        sum.im += f * src[tri(n, m)].im;
      }
      out[c].re += sum.re;
      out[c].im += sum.im;
    }
  }
  const bool rec = active && !vert;
  const int W = p;
  const cplx<T> expp = cmake<T>(cosp, sinp);
  const T cott2 = rec ? (T)2 * cost / sint : (T)0;
  const cplx<T> two_cott_expp = cmake<T>(cott2 * cosp, cott2 * sinp);
  const cplx<T> exp2p = cmul(expp, expp);
  const T isint = rec ? (T)1 / sint : (T)0;
  cplx<T> *partial = P, *partial_m_1 = Q;
  T sign = (T)1;
  // inv_r^(l+n+1) of this lane's sources n = hl, hl + 16 (orders up to
  // 32), advanced by inv_r per degree
  T rpow[2] = {ipow(inv_r, hl + 1), ipow(inv_r, hl + 17)};
  for (int l = 0; l <= p; ++l) {
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int n = hl + 16 * k;
      if (!rec || n >= p) continue;
      const int ln = l + n;
      const T fact = rpow[k] * beta[ln] / beta[n];
      cplx<T> s0 = cmake<T>(0, 0);
      for (int o = -n; o <= n; ++o) {
        int ao = o < 0 ? -o : o;
        cplx<T> h = ld(H, tri(ln, ao));
        cplx<T> sv = src[tri(n, ao)];
        if (o < 0) {
          h = sph_sym(h, ao);
          sv = sph_sym(sv, ao);
        }
        cfma(s0, h, sv, alpha[tri(n, ao)] * ialpha[tri(ln, ao)]);
      }
      partial[n] = cmake<T>(s0.re * fact, s0.im * fact);
      if (l > 0) {
        cplx<T> s1 = cmake<T>(0, 0);
        for (int o = -n; o <= n; ++o) {
          int ao = o < 0 ? -o : o;
          int op1 = o + 1, aop1 = op1 < 0 ? -op1 : op1;
          cplx<T> h = ld(H, tri(ln, aop1));
          cplx<T> sv = src[tri(n, ao)];
          if (op1 < 0) h = sph_sym(h, aop1);
          if (o < 0) sv = sph_sym(sv, ao);
          cfma(s1, h, sv, alpha[tri(n, ao)] * ialpha[tri(ln, aop1)]);
        }
        partial[W + n] = cmake<T>(s1.re * fact, s1.im * fact);
      }
      const T tlf = (T)2 * (T)ln * inv_r * isint;
      const cplx<T> tl = cmake<T>(tlf * cosp, tlf * sinp);
      for (int m = 2; m <= l; ++m) {
        cplx<T> a = cmul(two_cott_expp, partial[(m - 1) * W + n]);
        cplx<T> b = cmul(exp2p, partial[(m - 2) * W + n]);
        cplx<T> c = cmul(tl, partial_m_1[(m - 1) * W + n]);
        partial[m * W + n] = cmake<T>(a.re + b.re - c.re, a.im + b.im - c.im);
      }
    }
    rpow[0] *= inv_r;
    rpow[1] *= inv_r;
    __syncwarp();
    if (rec) {
      const T fb = beta[l] * sign;
      for (int m = hl; m <= l; m += 16) {
        cplx<T> sum = cmake<T>(0, 0);
        for (int n = 0; n < p; ++n) {
          sum.re += partial[m * W + n].re;
          sum.im += partial[m * W + n].im;
        }
        const T f = alpha[tri(l, m)] * fb;
        out[tri(l, m)].re += sum.re * f;
        out[tri(l, m)].im += -sum.im * f;
      }
    }
    __syncwarp();
    cplx<T> *fl = partial;
    partial = partial_m_1;
    partial_m_1 = fl;
    sign = -sign;
  }
}

// M2M: multipole part of aran/aransphericalseriesd-kkylin.c:32-209 with
// (r, -cost, sint, -cosp, -sinp) already folded into the table; output
// degree l scaled by 2^-l (child -> parent units).
template <typename T>
__device__ void kk_m2m_warp(int p, const cplx<T> *src, const T *tab, const T *alpha,
                            const T *beta, cplx<T> *P, cplx<T> *Q, cplx<T> *out, int lane) {
  const T r = tab[0], cost = tab[1], sint = tab[2], cosp = tab[3], sinp = tab[4];
  const T *H = tab + 8;
  const int W = p;
  cplx<T> *partial = P, *partial_m_1 = Q;
  if (lane == 0) {
    cplx<T> v = cmul(cconj(ld(H, 0)), src[0]);
    partial[0] = v;
    out[0].re += v.re * beta[0];
    out[0].im += v.im * beta[0];
  }
  __syncwarp();
  for (int l = 1; l < p; ++l) {
    cplx<T> *fl = partial;
    partial = partial_m_1;
    partial_m_1 = fl;
    for (int n = lane; n <= l - 1; n += 32) {
      const int d = l - n;
      const T rp = ipow(r, d);
      const T fact = beta[d] / beta[n];
      cplx<T> s0 = cmake<T>(0, 0);
      for (int o = (-n > n - l ? -n : n - l); o <= (n < d ? n : d); ++o) {
        int ao = o < 0 ? -o : o;
        cplx<T> h = ld(H, tri(d, ao));
        cplx<T> sv = src[tri(n, ao)];
        if (o > 0) h = sph_sym(h, ao);
        else if (o < 0) sv = sph_sym(sv, ao);
        cfma(s0, cconj(h), sv, rp * alpha[tri(n, ao)] * alpha[tri(d, ao)]);
      }
      partial[n] = cmake<T>(s0.re * fact, s0.im * fact);
      if (l > 1) {
        cplx<T> s1 = cmake<T>(0, 0);
        int lo = -n > n - 1 ? -n : n - 1, hi = n < l + l - 1 - n ? n : l + l - 1 - n;
        for (int o = lo; o <= hi; ++o) {
          int ao = o < 0 ? -o : o;
          int e1 = l - o - 1, ae1 = e1 < 0 ? -e1 : e1;
          cplx<T> h = ld(H, tri(d, ae1));
          cplx<T> sv = src[tri(n, ao)];
          if (e1 < 0) h = sph_sym(h, ae1);
          if (o < 0) sv = sph_sym(sv, ao);
          cfma(s1, cconj(h), sv, rp * alpha[tri(n, ao)] * alpha[tri(d, ae1)]);
        }
        partial[(l - 1) * W + n] = cmake<T>(s1.re * fact, s1.im * fact);
      }
      {
        cplx<T> s2 = cmake<T>(0, 0);
        int lo = -n > n ? -n : n, hi = n < l + l - n ? n : l + l - n;
        for (int o = lo; o <= hi; ++o) {
          int ao = o < 0 ? -o : o;
          int e2 = l - o, ae2 = e2 < 0 ? -e2 : e2;
          cplx<T> h = ld(H, tri(d, ae2));
          cplx<T> sv = src[tri(n, ao)];
          if (e2 < 0) h = sph_sym(h, ae2);
          if (o < 0) sv = sph_sym(sv, ao);
          cfma(s2, cconj(h), sv, rp * alpha[tri(n, ao)] * alpha[tri(d, ae2)]);
        }
        partial[l * W + n] = cmake<T>(s2.re * fact, s2.im * fact);
      }
      const T f = (T)0.5 * r / (T)(l - n);
      const cplx<T> fse = cmake<T>(f * sint * cosp, f * sint * sinp);
      const T f2 = f * (T)2 * cost;
      for (int m = 1; m < l - 1; ++m) {
        cplx<T> a = cmul(fse, partial_m_1[(m + 1) * W + n]);
        cplx<T> b = cmul(cconj(fse), partial_m_1[(m - 1) * W + n]);
        cplx<T> c = partial_m_1[m * W + n];
        partial[m * W + n] = cmake<T>(a.re - b.re + f2 * c.re, a.im - b.im + f2 * c.im);
      }
    }
    // partial[*][l]: direct terms (column l; W = p > l)
    const T f0 = beta[0] / beta[l];
    const cplx<T> h0 = cconj(ld(H, 0));
    for (int m = lane; m <= l; m += 32) {
      cplx<T> v = cmul(h0, src[tri(l, m)]);
      T f = alpha[tri(l, m)] * f0;
      partial[m * W + l] = cmake<T>(v.re * f, v.im * f);
    }
    __syncwarp();
    const T sc = ldexp((T)1, -l);
    for (int m = lane; m <= l; m += 32) {
      cplx<T> sum = cmake<T>(0, 0);
      for (int n = 0; n <= l; ++n) {
        sum.re += partial[m * W + n].re;
        sum.im += partial[m * W + n].im;
      }
      T f = beta[l] / alpha[tri(l, m)] * sc;
      out[tri(l, m)].re += sum.re * f;
      out[tri(l, m)].im += sum.im * f;
    }
    __syncwarp();
  }
}

// L2L: aran/aransphericalseriesd-kkylin.c:211-362, output degree l scaled
// by 2^-l (parent -> child units).  Buffers (p+1) x (p+1).
template <typename T>
__device__ void kk_l2l_warp(int p, const cplx<T> *src, const T *tab, const T *alpha,
                            const T *beta, cplx<T> *P, cplx<T> *Q, cplx<T> *out, int lane) {
  const T r = tab[0], cost = tab[1], sint = tab[2], cosp = tab[3], sinp = tab[4];
  const T *H = tab + 8;
  const cplx<T> y00 = ld(H, 0);
  const int W = p + 1;
  cplx<T> *partial = P, *partial_p_1 = Q;
  for (int l = p; l >= 0; --l) {
    {
      const T fact = beta[0] / beta[l];
      for (int m = lane; m <= l; m += 32) {
        cplx<T> v = cconj(cmul(y00, src[tri(l, m)]));
        T f = fact / alpha[tri(l, m)];
        partial[m * W + l] = cmake<T>(v.re * f, v.im * f);
      }
    }
    for (int n = l + 1 + lane; n <= p; n += 32) {
      const int d = n - l;
      const T rp = ipow(r, d);
      const T fact = beta[d] / beta[n];
      cplx<T> s0 = cmake<T>(0, 0);
      for (int o = (-n > l - n ? -n : l - n); o <= (n < d ? n : d); ++o) {
        int ao = o < 0 ? -o : o;
        cplx<T> h = ld(H, tri(d, ao));
        cplx<T> sv = src[tri(n, ao)];
        if (o < 0) {
          h = sph_sym(h, ao);
          sv = sph_sym(sv, ao);
        }
        cfma(s0, cconj(h), cconj(sv), rp * alpha[tri(d, ao)] / alpha[tri(n, ao)]);
      }
      partial[n] = cmake<T>(s0.re * fact, s0.im * fact);
      if (l > 0) {
        cplx<T> s1 = cmake<T>(0, 0);
        int lo = -n > l + l - n ? -n : l + l - n;
        for (int o = lo; o <= n; ++o) {
          int ao = o < 0 ? -o : o;
          int e1 = o - l, ae1 = e1 < 0 ? -e1 : e1;
          cplx<T> h = ld(H, tri(d, ae1));
          cplx<T> sv = src[tri(n, ao)];
          if (e1 < 0) h = sph_sym(h, ae1);
          if (o < 0) sv = sph_sym(sv, ao);
          cfma(s1, cconj(h), cconj(sv), rp * alpha[tri(d, ae1)] / alpha[tri(n, ao)]);
        }
        partial[l * W + n] = cmake<T>(s1.re * fact, s1.im * fact);
      }
      const T f = (T)0.5 * r / (T)(n - l);
      const cplx<T> fse = cmake<T>(f * sint * cosp, f * sint * sinp);
      const T f2 = f * (T)2 * cost;
      for (int m = 1; m < l; ++m) {
        cplx<T> a = cmul(fse, partial_p_1[(m - 1) * W + n]);
        cplx<T> b = cmul(cconj(fse), partial_p_1[(m + 1) * W + n]);
        cplx<T> c = partial_p_1[m * W + n];
        partial[m * W + n] = cmake<T>(a.re - b.re + f2 * c.re, a.im - b.im + f2 * c.im);
      }
    }
    __syncwarp();
    const T sc = ldexp((T)1, -l);
    for (int m = lane; m <= l; m += 32) {
      cplx<T> sum = cmake<T>(0, 0);
      for (int n = l; n <= p; ++n) {
        sum.re += partial[m * W + n].re;
        sum.im += partial[m * W + n].im;
      }
      T f = beta[l] * alpha[tri(l, m)] * sc;
      out[tri(l, m)].re += sum.re * f;
      out[tri(l, m)].im += -sum.im * f;
    }
    __syncwarp();
    cplx<T> *fl = partial;
    partial = partial_p_1;
    partial_p_1 = fl;
  }
}

// shared memory per warp: src (nl) + out (nl) + P, Q ((p+1)^2 each); the
// M2L uses twice that (one set per half-warp)
__host__ __device__ inline int kk_warp_cplx(int p) { return 2 * tri(p + 1) + 2 * (p + 1) * (p + 1); }

constexpr int kKkWarps = 4;

// per half-warp of the M2L: src, out, P, Q and the direction's table
// (stride T values), in complex units
__host__ __device__ inline int kk_m2l_half_cplx(int p, int stride) {
  return kk_warp_cplx(p) + (stride + 1) / 2;
}

template <typename T>
__global__ void k_m2l_kk(int cnt, int off, const int *__restrict__ far_off,
                         const int *__restrict__ far_src, const uint16_t *__restrict__ far_dir,
                         const uint8_t *__restrict__ depth, int p, const T *__restrict__ dirs,
                         int stride, const T *__restrict__ alpha_g, const T *__restrict__ ialpha_g,
                         int nalpha, const T *__restrict__ beta, const T *__restrict__ vt,
                         double scale_e, const cplx<T> *__restrict__ mult,
                         cplx<T> *__restrict__ loc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int half = lane >> 4, hl = lane & 15;
  // alpha and 1/alpha for the block, then per warp two half sets
  T *alpha = reinterpret_cast<T *>(smem_raw);
  T *ialpha = alpha + nalpha;
  for (int i = threadIdx.x; i < nalpha; i += blockDim.x) {
    alpha[i] = alpha_g[i];
    ialpha[i] = ialpha_g[i];
  }
  __syncthreads();
  const int t = off + blockIdx.x * (int)(blockDim.x >> 5) + w;
  if (t >= off + cnt) return;
  const int j0 = far_off[t], j1 = far_off[t + 1];
  if (j0 == j1) return;
  const int nm = tri(p), nl = tri(p + 1);
  const int hsz = kk_m2l_half_cplx(p, stride);
  cplx<T> *base = reinterpret_cast<cplx<T> *>(smem_raw + ((2 * nalpha * sizeof(T) + 15) & ~(size_t)15));
  cplx<T> *src = base + (size_t)(2 * w + half) * hsz;
  cplx<T> *out = src + nl;
  cplx<T> *P = out + nl;
  cplx<T> *Q = P + (p + 1) * (p + 1);
  T *tab = reinterpret_cast<T *>(Q + (p + 1) * (p + 1));
  for (int c = hl; c < nl; c += 16) out[c] = cmake<T>(0, 0);
  for (int j = j0; j < j1; j += 2) {
    const int jj = j + half;
    const bool active = jj < j1;
    __syncwarp();
    if (active) {
      const int s = far_src[jj];
      for (int c = hl; c < nm; c += 16) src[c] = mult[(size_t)s * nm + c];
      const T *tg = dirs + (size_t)far_dir[jj] * stride;
      for (int c = hl; c < stride; c += 16) tab[c] = tg[c];
    }
    __syncwarp();
    kk_m2l_half<T>(p, active, src, tab, alpha, ialpha, beta, vt, P, Q, out, hl);
  }
  __syncwarp();
  // the two halves' locals summed
  const cplx<T> *out0 = base + (size_t)(2 * w) * hsz + nl;
  const cplx<T> *out1 = base + (size_t)(2 * w + 1) * hsz + nl;
  const T ih = (T)(ldexp(1.0, depth[t]) / scale_e);
  for (int c = lane; c < nl; c += 32)
    loc[(size_t)t * nl + c] = cmake<T>((out0[c].re + out1[c].re) * ih, (out0[c].im + out1[c].im) * ih);
}

template <typename T>
__global__ void k_m2m_kk(int cnt, int off, const int *__restrict__ child,
                         const int *__restrict__ begin, const int *__restrict__ end, int p,
                         const T *__restrict__ dirs, int stride, const T *__restrict__ alpha,
                         const T *__restrict__ beta, cplx<T> *__restrict__ mult) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int Pn = off + blockIdx.x * kKkWarps + w;
  if (Pn >= off + cnt) return;
  const int c0 = child[Pn];
  if (c0 < 0) return;
  const int nm = tri(p);
  cplx<T> *src = reinterpret_cast<cplx<T> *>(smem_raw) + (size_t)w * kk_warp_cplx(p);
  cplx<T> *out = src + tri(p + 1);
  cplx<T> *P = out + tri(p + 1);
  cplx<T> *Q = P + (p + 1) * (p + 1);
  for (int c = lane; c < nm; c += 32) out[c] = cmake<T>(0, 0);
  for (int o = 0; o < 8; ++o) {
    const int ch = c0 + o;
    if (end[ch] == begin[ch]) continue;
    __syncwarp();
    for (int c = lane; c < nm; c += 32) src[c] = mult[(size_t)ch * nm + c];
    __syncwarp();
    kk_m2m_warp<T>(p, src, dirs + (size_t)o * stride, alpha, beta, P, Q, out, lane);
  }
  __syncwarp();
  for (int c = lane; c < nm; c += 32) mult[(size_t)Pn * nm + c] = out[c];
}

template <typename T>
__global__ void k_l2l_kk(int cnt, int off, const int *__restrict__ parent,
                         const int *__restrict__ child, const int *__restrict__ begin,
                         const int *__restrict__ end, int p, const T *__restrict__ dirs, int stride,
                         const T *__restrict__ alpha, const T *__restrict__ beta,
                         cplx<T> *__restrict__ loc) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int C = off + blockIdx.x * kKkWarps + w;
  if (C >= off + cnt) return;
  if (end[C] == begin[C]) return;
  const int Pn = parent[C];
  const int o = C - child[Pn];
  const int nl = tri(p + 1);
  cplx<T> *src = reinterpret_cast<cplx<T> *>(smem_raw) + (size_t)w * kk_warp_cplx(p);
  cplx<T> *out = src + nl;
  cplx<T> *P = out + nl;
  cplx<T> *Q = P + (p + 1) * (p + 1);
  for (int c = lane; c < nl; c += 32) {
    src[c] = loc[(size_t)Pn * nl + c];
    out[c] = cmake<T>(0, 0);
  }
  __syncwarp();
  kk_l2l_warp<T>(p, src, dirs + (size_t)o * stride, alpha, beta, P, Q, out, lane);
  __syncwarp();
  for (int c = lane; c < nl; c += 32) {
    cplx<T> v = loc[(size_t)C * nl + c];
    loc[(size_t)C * nl + c] = cmake<T>(v.re + out[c].re, v.im + out[c].im);
  }
}

template <typename T>
__global__ void k_kk_scalars(int L, T *alpha, T *ialpha, T *beta, double *scratch) {
  if (blockIdx.x || threadIdx.x) return;
  gen_alpha(L, scratch);
  for (int i = 0; i < tri(L + 1); ++i) {
    alpha[i] = (T)scratch[i];
    ialpha[i] = (T)(1.0 / scratch[i]);
  }
  for (int l = 0; l <= L; ++l) beta[l] = (T)beta_l(l);
}

template <typename T>
void build_kk_t(AranGpuSolver3d *s, KkTables<T> &kk, cudaStream_t st) {
  int p = s->cfg.order;
  if (kk.p == p) return;
  kk.p = p;
  int La = 2 * p + 2;
  kk.alpha.reserve(tri(La + 1));
  kk.ialpha.reserve(tri(La + 1));
  kk.beta.reserve(La + 1);
  DBuf<double> scratch;
  int Lh = 2 * p;
  int sstride = 3 * tri(Lh + 1) + 2 * tri(Lh + 1) + 16;
  scratch.reserve((size_t)343 * sstride + tri(La + 1));
  k_kk_scalars<T><<<1, 1, 0, st>>>(La, kk.alpha.ptr, kk.ialpha.ptr, kk.beta.ptr, scratch.ptr);
  ACHECK(cudaGetLastError());
  double ext = s->scale_e;
  double ex = (s->cfg.ub[0] - s->cfg.lb[0]) / ext, ey = (s->cfg.ub[1] - s->cfg.lb[1]) / ext,
         ez = (s->cfg.ub[2] - s->cfg.lb[2]) / ext;
  for (int kind = 0; kind < 3; ++kind) {
    KkLayout L = kk_layout(p, kind);
    int ndir = kind == 0 ? 343 : 8;
    kk.stride[kind] = L.stride;
    kk.dirs[kind].reserve((size_t)ndir * L.stride);
    k_kk_tables<T><<<ceil_div(ndir, 64), 64, 0, st>>>(p, kind, ndir, ex, ey, ez, scratch.ptr,
                                                        sstride, kk.dirs[kind].ptr);
    ACHECK(cudaGetLastError());
  }
  ACHECK(cudaStreamSynchronize(st));
  scratch.release();
}


template <typename T>
static void kk_passes_t(AranGpuSolver3d *s, KkTables<T> &kk, OpTables<T> &tb, cplx<T> *mult,
                        cplx<T> *loc, int stage) {
  cudaStream_t st = s->s0;
  DevTree &t = s->tree;
  const int p = s->cfg.order;
  const int TB = 32 * kKkWarps;
  const size_t sm = (size_t)kKkWarps * kk_warp_cplx(p) * sizeof(cplx<T>);
  if (stage == 0) {  // M2M, deepest level first
    if (sm > 48 * 1024)
      smem_opt_in(k_m2m_kk<T>, sm);
    for (int d = t.nlevels - 2; d >= 0; --d) {
      if (t.level_internal[d] == 0) continue;
      int off = t.level_off[d], cnt = t.level_off[d + 1] - off;
      k_m2m_kk<T><<<ceil_div(cnt, kKkWarps), TB, sm, st>>>(cnt, off, t.child.ptr, t.begin.ptr,
                                                           t.end.ptr, p, kk.dirs[1].ptr,
                                                           kk.stride[1], kk.alpha.ptr, kk.beta.ptr,
                                                           mult);
      ACHECK(cudaGetLastError());
      s->launches++;
    }
  } else if (stage == 1) {  // M2L
    if (t.nlevels > 2) {
      // two half-warp sets of buffers per warp; fewer warps per CTA where
      // four would not fit in shared memory (FP64 at high orders)
      const int nalpha = tri(2 * p + 3);
      const size_t head = (2 * (size_t)nalpha * sizeof(T) + 15) & ~(size_t)15;
      const size_t per_warp = 2 * (size_t)kk_m2l_half_cplx(p, kk.stride[0]) * sizeof(cplx<T>);
      int dev_smem = 0;
      ACHECK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
      int wpb = kKkWarps;
      while (wpb > 1 && head + (size_t)wpb * per_warp > (size_t)dev_smem) --wpb;
      const size_t sm2 = head + (size_t)wpb * per_warp;
      smem_opt_in(k_m2l_kk<T>, sm2);
      int off = t.level_off[2], cnt = t.nnodes - off;
      k_m2l_kk<T><<<ceil_div(cnt, wpb), 32 * wpb, sm2, st>>>(cnt, off, t.far_off.ptr, t.far_src.ptr,
                                                            t.far_dir.ptr, t.depth.ptr, p,
                                                            kk.dirs[0].ptr, kk.stride[0],
                                                            kk.alpha.ptr, kk.ialpha.ptr, nalpha,
                                                            kk.beta.ptr, tb.vt.ptr, s->scale_e,
                                                            mult, loc);
      ACHECK(cudaGetLastError());
      s->launches++;
    }
  } else {  // L2L from depth 3
    if (sm > 48 * 1024)
      smem_opt_in(k_l2l_kk<T>, sm);
    for (int d = 3; d < t.nlevels; ++d) {
      int off = t.level_off[d], cnt = t.level_off[d + 1] - off;
      k_l2l_kk<T><<<ceil_div(cnt, kKkWarps), TB, sm, st>>>(cnt, off, t.parent.ptr, t.child.ptr,
                                                           t.begin.ptr, t.end.ptr, p,
                                                           kk.dirs[2].ptr, kk.stride[2],
                                                           kk.alpha.ptr, kk.beta.ptr, loc);
      ACHECK(cudaGetLastError());
      s->launches++;
    }
  }
}

}  // namespace

void build_kkylin_tables(AranGpuSolver3d *s) {
  if (s->cfg.precision == ARAN_PRECISION_MIXED) build_kk_t<float>(s, s->kk32, s->s0);
  else build_kk_t<double>(s, s->kk64, s->s0);
}

void kkylin_pass(AranGpuSolver3d *s, int stage) {
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    kk_passes_t<float>(s, s->kk32, s->t32, reinterpret_cast<cplx<float> *>(s->mult32.ptr),
                       reinterpret_cast<cplx<float> *>(s->loc32.ptr), stage);
  else
    kk_passes_t<double>(s, s->kk64, s->t64, reinterpret_cast<cplx<double> *>(s->mult64.ptr),
                        reinterpret_cast<cplx<double> *>(s->loc64.ptr), stage);
}

}  // namespace aran
