// series3d.cu -- LibAran's spherical-harmonic series API
// (aran/aransphericalseriesd.h:42-131) and the 3D development operators
// called on host developments (aran/arandevelopment3d.h:45-150).
//
// Containers are host memory in the reference layout
// (aran/aransphericalseriesd-private.h:38-70).  Every operator that computes
// runs as one launch of one warp: the inputs are copied to the device, the
// reference's algorithm runs in FP64 with the lanes sharing the independent
// outputs (rotations: one lane per output (l, m'); vertical translations:
// one lane per output (l, m); phase factors: one lane per Wigner row) and
// lane 0 running the recurrences (Wigner d, harmonics, the alpha table) and
// the O(p^2) evaluations, the result comes back.  Restated from the
// reference:
//   rotate / rotate_inverse   Wigner D = e^{-i m alpha} d(beta) e^{-i m' gamma},
//                             phases only for |angle| >= 1e-5
//                             (aranwigner.c:83-313, -rotate.c:34-153);
//   translate / to_local      rotate the translation onto z, translate along z
//                             (-translate.c:301-364,445-505,609-676), rotate
//                             back (-rotate.c:165-263); the normal and kkylin
//                             flavours compute the same operators and go the
//                             same way, to_local adding their local-part
//                             translation (-translate.c:816-834);
//   evaluate / gradient       aransphericalseriesd.c:312-546;
//   P2M / P2L                 arandevelopment3d.c:169-277.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"

#include <aran/arandevelopment3d.h>

struct _AranSphericalSeriesd {
  guint8 posdeg;
  guint8 negdeg;
  gcomplex128 *terms;
};

namespace aran {
namespace {

typedef cplx<double> zd;

size_t series_len(int pd, int nd) { return ((size_t)(pd + 1) * (pd + 2) + (size_t)nd * (nd + 1)) / 2; }

enum {
  S_ROTATE = 0, S_ROTATE_INV, S_TRANSLATE, S_TO_LOCAL, S_EVAL, S_GRAD, S_P2M, S_P2L
};
enum { F_NORMAL = 0, F_KKYLIN = 1, F_ROTATE = 2 };

struct Sv {
  int pd, nd;
  zd *c;
};

struct SeriesOp {
  int kind, flavour;
  int sp, sn, dp, dn;
  const zd *src;
  zd *dst;
  double xs[3], xd[3];    // centres, or (r, cost, sint, cosp, sinp) in xs/xd for *_internal
  double a, b, g, q;
  int internal;           // evaluate/gradient from spherical coordinates
  double *scratch;
  double *out;            // evaluate: 2; gradient: 3 (Cartesian) or 6 (dr, dt, dp complex)
};

// ---- complex helpers (device) ----
__device__ __forceinline__ zd zc(double a, double b) { return cmake(a, b); }
__device__ __forceinline__ zd zadd_(zd a, zd b) { return zc(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ zd zmul_(zd a, zd b) {
  return zc(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ zd zscl(zd a, double s) { return zc(a.re * s, a.im * s); }
__device__ __forceinline__ zd zconj(zd a) { return zc(a.re, -a.im); }
__device__ __forceinline__ zd sph_sym(zd z, int m) {   // (-1)^m conj(z)
  z = zconj(z);
  return (m & 1) ? zc(-z.re, -z.im) : z;
}

// lane of the operator's warp, and the warp-wide step of lane-strided loops
__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }
constexpr int kLanes = 32;
// (l, m) of the k-th coefficient in tri order
__device__ __forceinline__ void tri_lm(int k, int &l, int &m) {
  l = (int)((sqrt(8.0 * k + 1.0) - 1.0) * 0.5);
  while (tri(l + 1) <= k) ++l;
  while (tri(l) > k) --l;
  m = k - tri(l);
}

__device__ __forceinline__ zd *sv_pos(Sv s, int l, int m) { return s.c + tri(l) + m; }
__device__ __forceinline__ zd *sv_neg(Sv s, int l, int m) {
  return s.c + ((s.pd + 1) * (s.pd + 2) + l * (l + 1)) / 2 + m;
}

// bump allocator over the scratch block
struct Arena {
  double *p;
  __device__ double *take(size_t n) {
    double *r = p;
    p += (n + 1) & ~(size_t)1;
    return r;
  }
  __device__ zd *takez(size_t n) { return reinterpret_cast<zd *>(take(2 * n)); }
};

__device__ void sph_internal(const double v[3], double &r, double &ct, double &st, double &cp,
                             double &sp) {
  double rho2 = v[0] * v[0] + v[1] * v[1], rho = sqrt(rho2);
  r = sqrt(rho2 + v[2] * v[2]);
  if (r > 0.) { ct = v[2] / r; st = rho / r; } else { ct = 1.; st = 0.; }
  if (rho > 0.) { cp = v[0] / rho; sp = v[1] / rho; } else { cp = 1.; sp = 0.; }
}

__device__ void sph_angles(const double v[3], double &r, double &theta, double &phi) {
  double rho2 = v[0] * v[0] + v[1] * v[1];
  r = sqrt(rho2 + v[2] * v[2]);
  theta = r > 0. ? acos(v[2] / r) : 0.;
  phi = rho2 > 0. ? atan2(v[1], v[0]) : 0.;
}

// h[tri(l,m)] = N_l^m P_l^m(cos) e^{i m phi}; sh the same with P/sin(theta)
// (m >= 1; 0 for m = 0), l <= n, Condon-Shortley phase
__device__ void harmonics(int n, double ct, double st, double cp, double sp, zd *h, zd *sh) {
  double er = 1., ei = 0.;
  double cmm = sqrt(1. / (4. * kPi));   // (-1)^m sqrt((2m+1)/4pi prod (2k-1)/2k), m = 0
  double smm = 1.;                      // sin^m
  double fac = 1.;                      // prod (2k-1)/(2k)
  for (int m = 0; m <= n; ++m) {
    if (m > 0) {
      fac *= (2. * m - 1.) / (2. * m);
      double t = er * cp - ei * sp;
      ei = er * sp + ei * cp;
      er = t;
    }
    cmm = sqrt((2. * m + 1.) / (4. * kPi) * fac);
    if (m & 1) cmm = -cmm;
    double y2 = 0., y1 = cmm * smm;                    // N P at l-2, l-1
    double z2 = 0., z1 = m > 0 ? cmm * smm / (st != 0. ? st : 1.) : 0.;
    if (m > 0 && st == 0.) {                            // P/sin at the poles
      double sm1 = 1.;
      for (int k = 1; k < m; ++k) sm1 *= st;
      z1 = cmm * sm1;
    }
    for (int l = m; l <= n; ++l) {
      double y, z;
      if (l == m) { y = y1; z = z1; }
      else if (l == m + 1) {
        const double a = sqrt(2. * m + 3.) * ct;
        y = a * y1;
        z = a * z1;
      } else {
        const double a = sqrt((4. * l * l - 1.) / ((double)l * l - (double)m * m));
        const double b = sqrt(((l - 1.) * (l - 1.) - (double)m * m) / (4. * (l - 1.) * (l - 1.) - 1.));
        y = a * (ct * y1 - b * y2);
        z = a * (ct * z1 - b * z2);
      }
      if (l > m) { y2 = y1; y1 = y; z2 = z1; z1 = z; }
      h[tri(l, m)] = zc(er * y, ei * y);
      if (sh) sh[tri(l, m)] = m > 0 ? zc(er * z, ei * z) : zc(0., 0.);
    }
    smm *= st;
  }
}

// Wigner D for l <= L with the reference's phases
__device__ void wigner_full(int L, double a, double b, double g, double *wd, zd *W, zd *e) {
  const int lane = lane_id();
  if (lane == 0) gen_wigner_d(L, b, wd);
  __syncwarp();
  const int n = wig_size(L);
  for (int i = lane; i < n; i += kLanes) W[i] = zc(wd[i], 0.);
  // rows (l, m') of the Wigner blocks, one lane each
  const int nrows = tri(L + 1);
  for (int pass = 0; pass < 2; ++pass) {
    const double ang = pass == 0 ? a : g;
    if (!(fabs(ang) >= 1e-5)) continue;
    __syncwarp();
    if (lane == 0) {
      zd ex = zc(cos(ang), -sin(ang));
      e[0] = zc(1., 0.);
      for (int k = 1; k <= L; ++k) e[k] = zmul_(e[k - 1], ex);
    }
    __syncwarp();
    for (int rrow = lane; rrow < nrows; rrow += kLanes) {
      int l, mp;
      tri_lm(rrow, l, mp);
      zd *row = W + wig_off(l) + mp * (2 * l + 1) + l;
      if (pass == 0) {
        for (int m = l; m >= 1; --m) row[-m] = zmul_(row[-m], zconj(e[m]));
        for (int m = 0; m <= l; ++m) row[m] = zmul_(row[m], e[m]);
      } else {
        for (int m = -l; m <= l; ++m) row[m] = zmul_(row[m], e[mp]);
      }
    }
  }
  __syncwarp();
}

__device__ void buffer_rotate(const zd *W, int deg, const zd *src, zd *dst) {
  for (int k = lane_id(); k < tri(deg + 1); k += kLanes) {
    int l, mp;
    tri_lm(k, l, mp);
    const int o = tri(l);
    const zd *row = W + wig_off(l) + mp * (2 * l + 1) + l;
    zd sum = zc(0., 0.);
    for (int m = -l; m < 0; ++m) sum = zadd_(sum, zmul_(row[m], sph_sym(src[o - m], -m)));
    for (int m = 0; m <= l; ++m) sum = zadd_(sum, zmul_(row[m], src[o + m]));
    dst[o + mp] = zadd_(dst[o + mp], sum);
  }
  __syncwarp();
}

__device__ void rotate_series(Sv src, double a, double b, double g, Sv dst, Arena ar, bool inverse) {
  const int nd = min(dst.nd, src.nd), pd = min(dst.pd, src.pd);
  const int L = max(pd + 1, nd);
  double *wd = ar.take(wig_size(L));
  zd *W = ar.takez(wig_size(L));
  zd *e = ar.takez(L + 1);
  if (inverse) wigner_full(L, -g, -b, -a, wd, W, e);
  else wigner_full(L, a, b, g, wd, W, e);
  buffer_rotate(W, pd, sv_pos(src, 0, 0), sv_pos(dst, 0, 0));
  if (nd > 0) buffer_rotate(W, nd - 1, sv_neg(src, 0, 0), sv_neg(dst, 0, 0));
}

__device__ double alpha_lm(const double *al, int l, int m) { return al[tri(l, m)]; }
__device__ double bl_over_bn(int l, int n) { return beta_l(l) / beta_l(n); }

__device__ void local_vertical(Sv src, Sv dst, double r, double cost, const double *al) {
  for (int k = lane_id(); k < tri(dst.pd + 1); k += kLanes) {
    int l, m;
    tri_lm(k, l, m);
    {
      zd *d = sv_pos(dst, l, m);
      double rp = 1.;
      for (int n = l; n <= src.pd; ++n) {
        if (n > l) rp *= r;
        const zd s = *sv_pos(src, n, m);
        const double factor = alpha_lm(al, n - l, 0) * alpha_lm(al, l, m) / alpha_lm(al, n, m);
        const double h = ((n - l) % 2 == 0) ? 1. : cost;
        *d = zadd_(*d, zscl(s, h * factor * bl_over_bn(l, n) * rp));
      }
    }
  }
  __syncwarp();
}

__device__ void multipole_vertical(Sv src, Sv dst, double r, double cost, const double *al) {
  for (int k = lane_id(); k < tri(dst.nd); k += kLanes) {
    int l, m;
    tri_lm(k, l, m);
    {
      zd *d = sv_neg(dst, l, m);
      for (int n = m; n <= min(l, src.nd - 1); ++n) {
        double rp = 1.;
        for (int k = 0; k < l - n; ++k) rp *= r;
        const zd s = *sv_neg(src, n, m);
        const double factor = alpha_lm(al, l - n, 0) * alpha_lm(al, n, m) / alpha_lm(al, l, m);
        const double h = ((l - n) % 2 == 0) ? 1. : cost;
        *d = zadd_(*d, zscl(s, h * factor * bl_over_bn(l, n) * rp));
      }
    }
  }
  __syncwarp();
}

__device__ void m2l_vertical(Sv src, Sv dst, double r, double cost, const double *al) {
  const double ir = 1. / r;
  for (int k = lane_id(); k < tri(dst.pd + 1); k += kLanes) {
    int l, m;
    tri_lm(k, l, m);
    {
      zd sum = zc(0., 0.);
      for (int n = m; n < src.nd; ++n) {
        double rp = 1.;
        for (int k = 0; k < l + n + 1; ++k) rp *= ir;
        if (((l + n + 1) & 1) == 0) rp *= cost;
        const double tf = bl_over_bn(l, n) * alpha_lm(al, l, m) * alpha_lm(al, n, m) /
                          alpha_lm(al, l + n, 0);
        sum = zadd_(sum, zscl(*sv_neg(src, n, m), rp * tf));
      }
      if ((l + m) & 1) sum = zc(-sum.re, -sum.im);
      zd *d = sv_pos(dst, l, m);
      *d = zadd_(*d, sum);
    }
  }
  __syncwarp();
}

__device__ Sv zero_series(int pd, int nd, Arena &ar) {
  Sv s;
  s.pd = pd;
  s.nd = nd;
  const size_t n = ((size_t)(pd + 1) * (pd + 2) + (size_t)nd * (nd + 1)) / 2;
  s.c = ar.takez(n);
  for (size_t i = lane_id(); i < n; i += kLanes) s.c[i] = zc(0., 0.);
  __syncwarp();
  return s;
}

// rotate the offset onto +z (flipping through cost = -1), apply `vert`, rotate back
template <typename V>
__device__ void via_rotation(Sv src, const double xs[3], Sv dst, const double xd[3], Arena ar,
                             int tpd, int tnd, V vert) {
  double v[3] = {xd[0] - xs[0], xd[1] - xs[1], xd[2] - xs[2]};
  double cost = 1.;
  if (v[2] < 0.) {
    cost = -1.;
    v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2];
  }
  double r, theta, phi;
  sph_angles(v, r, theta, phi);
  Sv rot = zero_series(src.pd, src.nd, ar);
  rotate_series(src, -phi, theta, 0., rot, ar, false);
  Sv trans = zero_series(tpd, tnd, ar);
  vert(rot, trans, r, cost);
  rotate_series(trans, -phi, theta, 0., dst, ar, true);
}

__device__ void op_translate(const SeriesOp &o, Sv src, Sv dst, Arena ar) {
  const int La = 2 * max(max(src.pd, dst.pd), max(src.nd, dst.nd)) + 4;
  double *al = ar.take(tri(La + 1));
  if (lane_id() == 0) gen_alpha(La, al);
  __syncwarp();
  via_rotation(src, o.xs, dst, o.xd, ar, dst.pd, dst.nd, [&](Sv s, Sv d, double r, double c) {
    local_vertical(s, d, r, c, al);
    if (s.nd > 0) multipole_vertical(s, d, r, -c, al);
  });
}

__device__ void op_to_local(const SeriesOp &o, Sv src, Sv dst, Arena ar) {
  const int La = 2 * max(max(src.pd, dst.pd), max(src.nd, dst.nd)) + 4;
  double *al = ar.take(tri(La + 1));
  if (lane_id() == 0) gen_alpha(La, al);
  __syncwarp();
  if (o.flavour != F_ROTATE) {
    // normal / kkylin: the source's local part is translated as well
    Sv sp = src;
    sp.nd = 0;
    via_rotation(sp, o.xs, dst, o.xd, ar, dst.pd, 0, [&](Sv s, Sv d, double r, double c) {
      local_vertical(s, d, r, c, al);
    });
  }
  if (src.nd > 0)
    via_rotation(src, o.xs, dst, o.xd, ar, dst.pd, dst.nd, [&](Sv s, Sv d, double r, double c) {
      m2l_vertical(s, d, r, c, al);
    });
}

__device__ zd eval_internal(Sv s, double r, double ct, double st, double cp, double sp, Arena ar) {
  const int n = max(s.pd, s.nd - 1);
  zd *h = ar.takez(tri(n + 1) + 1);
  harmonics(n, ct, st, cp, sp, h, nullptr);
  zd res = zc(0., 0.);
  for (int l = s.pd; l >= 0; --l) {
    double sum = 0.;
    const zd *c = sv_pos(s, l, 0);
    for (int m = 1; m <= l; ++m) sum += zmul_(c[m], h[tri(l, m)]).re;
    zd t = zadd_(zc(2. * sum, 0.), zmul_(c[0], h[tri(l, 0)]));
    res = zadd_(zscl(res, r), t);
  }
  if (s.nd != 0) {
    zd neg = zc(0., 0.);
    const double ir = 1. / r;
    for (int l = s.nd - 1; l >= 0; --l) {
      double sum = 0.;
      const zd *c = sv_neg(s, l, 0);
      for (int m = 1; m <= l; ++m) sum += zmul_(c[m], h[tri(l, m)]).re;
      zd t = zadd_(zc(2. * sum, 0.), zmul_(c[0], h[tri(l, 0)]));
      neg = zscl(zadd_(neg, t), ir);
    }
    res = zadd_(res, neg);
  }
  return res;
}

// gradient in spherical components, aransphericalseriesd.c:419-519
__device__ void grad_internal(Sv s, double r, double ct, double st, double cp, double sp,
                              zd &dr, zd &dt, zd &dp, Arena ar) {
  const int n = max(s.pd, s.nd);
  zd *h = ar.takez(tri(n + 1) + 1);
  zd *sh = ar.takez(tri(n + 1) + 1);
  harmonics(n, ct, st, cp, sp, h, sh);
  const zd ce = zc(cp, -sp);   // conj(e^{i phi})
  dr = dt = dp = zc(0., 0.);
  for (int l = s.pd; l >= 1; --l) {
    double sumr = 0., sumt = 0., sump = 0.;
    const zd *c = sv_pos(s, l, 0);
    for (int m = 1; m <= l; ++m) {
      sumr += zmul_(h[tri(l, m)], c[m]).re;
      sumt += zmul_(sh[tri(l, m)], c[m]).re * (ct * m);
      sump += zmul_(sh[tri(l, m)], c[m]).im * m;
    }
    for (int m = 1; m <= l - 1; ++m)
      sumt += zmul_(zmul_(h[tri(l, m + 1)], c[m]), ce).re * sqrt((double)((l - m) * (l + m + 1)));
    sumr = 2. * sumr + zmul_(h[tri(l, 0)], c[0]).re;
    sumt = 2. * sumt + zmul_(zmul_(h[tri(l, 1)], c[0]), ce).re * sqrt((double)(l * (l + 1)));
    sump *= -2.;
    dr = zadd_(zscl(dr, r), zc(sumr * l, 0.));
    dt = zadd_(zscl(dt, r), zc(sumt, 0.));
    dp = zadd_(zscl(dp, r), zc(sump, 0.));
  }
  if (s.nd > 0) {
    double dr2 = 0., dt2 = 0., dp2 = 0.;
    const double ir = 1. / r;
    for (int l = s.nd - 1; l >= 1; --l) {
      double sumr = 0., sumt = 0., sump = 0.;
      const zd *c = sv_neg(s, l, 0);
      for (int m = 1; m <= l; ++m) {
        sumr += zmul_(h[tri(l, m)], c[m]).re;
        sumt += zmul_(sh[tri(l, m)], c[m]).re * (ct * m);
        sump += zmul_(sh[tri(l, m)], c[m]).im * m;
      }
      for (int m = 1; m <= l - 1; ++m)
        sumt += zmul_(zmul_(h[tri(l, m + 1)], c[m]), ce).re * sqrt((double)((l - m) * (l + m + 1)));
      sumr = 2. * sumr + zmul_(h[tri(l, 0)], c[0]).re;
      sumt = 2. * sumt + zmul_(zmul_(h[tri(l, 1)], c[0]), ce).re * sqrt((double)(l * (l + 1)));
      sump *= -2.;
      dr2 = dr2 * ir + sumr * (l + 1);
      dt2 = dt2 * ir + sumt;
      dp2 = dp2 * ir + sump;
    }
    const zd *c0 = sv_neg(s, 0, 0);
    dr = zadd_(dr, zscl(zadd_(zc(dr2 * ir, 0.), zmul_(h[0], c0[0])), -ir * ir));
    dt = zadd_(dt, zc(dt2 * ir * ir * ir, 0.));
    dp = zadd_(dp, zc(dp2 * ir * ir * ir, 0.));
  }
}

__device__ void op_p2x(const SeriesOp &o, Sv dst, Arena ar, bool local) {
  const double v[3] = {o.xs[0] - o.xd[0], o.xs[1] - o.xd[1], o.xs[2] - o.xd[2]};
  double r, ct, st, cp, sp;
  sph_internal(v, r, ct, st, cp, sp);
  const int deg = local ? dst.pd : dst.nd;
  zd *h = ar.takez(tri(deg + 1) + 1);
  harmonics(deg, ct, st, cp, sp, h, nullptr);
  if (local) {
    const double ir = 1. / r;
    double fact = o.q * ir;
    for (int l = 0; l <= deg; ++l) {
      for (int m = 0; m <= l; ++m) {
        zd t = zscl(h[tri(l, m)], fact * (4. * kPi / (l + l + 1.)));
        zd *d = sv_pos(dst, l, m);
        *d = zadd_(*d, zconj(t));
      }
      fact *= ir;
    }
  } else {
    double fact = o.q;
    for (int l = 0; l < deg; ++l) {
      for (int m = 0; m <= l; ++m) {
        zd t = zscl(h[tri(l, m)], fact * (4. * kPi / (l + l + 1.)));
        zd *d = sv_neg(dst, l, m);
        *d = zadd_(*d, zconj(t));
      }
      fact *= r;
    }
  }
}

// one warp: the rotations and translations share their outputs over the
// lanes; the O(p^2) operators run on lane 0
__global__ void __launch_bounds__(32) k_series_op(SeriesOp o) {
  if (blockIdx.x != 0) return;
  Arena ar{o.scratch};
  Sv src{o.sp, o.sn, const_cast<zd *>(o.src)};
  Sv dst{o.dp, o.dn, o.dst};
  switch (o.kind) {
    case S_ROTATE: rotate_series(src, o.a, o.b, o.g, dst, ar, false); return;
    case S_ROTATE_INV: rotate_series(src, o.a, o.b, o.g, dst, ar, true); return;
    case S_TRANSLATE: op_translate(o, src, dst, ar); return;
    case S_TO_LOCAL: op_to_local(o, src, dst, ar); return;
    default: break;
  }
  if (lane_id() != 0) return;
  switch (o.kind) {
    case S_P2M: op_p2x(o, dst, ar, false); break;
    case S_P2L: op_p2x(o, dst, ar, true); break;
    case S_EVAL:
    case S_GRAD: {
      double r, ct, st, cp, sp;
      if (o.internal) {
        r = o.xs[0]; ct = o.xs[1]; st = o.xs[2]; cp = o.xd[0]; sp = o.xd[1];
      } else {
        const double v[3] = {o.xd[0] - o.xs[0], o.xd[1] - o.xs[1], o.xd[2] - o.xs[2]};
        sph_internal(v, r, ct, st, cp, sp);
      }
      if (o.kind == S_EVAL) {
        zd v = eval_internal(src, r, ct, st, cp, sp, ar);
        o.out[0] = v.re;
        o.out[1] = v.im;
      } else {
        zd dr, dt, dp;
        grad_internal(src, r, ct, st, cp, sp, dr, dt, dp, ar);
        if (o.internal) {
          o.out[0] = dr.re; o.out[1] = dr.im; o.out[2] = dt.re;
          o.out[3] = dt.im; o.out[4] = dp.re; o.out[5] = dp.im;
        } else {
          const double a = dr.re, b = dt.re, c = dp.re;
          o.out[0] = st * cp * a + ct * cp * b - sp * c;
          o.out[1] = st * sp * a + ct * sp * b + cp * c;
          o.out[2] = ct * a - st * b;
        }
      }
      break;
    }
  }
}

// ---- host side ----
struct SeriesContext {
  std::mutex mu;
  int device = -1;
  cudaStream_t st = nullptr;
  DBuf<double> buf;
};

SeriesContext &sctx() {
  static SeriesContext *c = new SeriesContext();  // lives until exit
  return *c;
}

size_t scratch_doubles(int kind, int L) {
  const size_t wig = (size_t)((L + 2) * (L + 3) * (4 * L + 7)) / 6;
  const size_t ser = 2 * (size_t)(L + 2) * (L + 3);
  const size_t al = (size_t)(2 * L + 6) * (2 * L + 7) / 2 + 8;
  (void)kind;
  return 3 * wig + 4 * ser + al + 4 * ((size_t)(L + 2) * (L + 3) / 2) + 64;
}

// Runs one operator; dst (when given) is updated in place, out receives
// evaluate/gradient results.  Returns ARAN_OK or an error code (dst untouched).
int series_op(SeriesOp op, const AranSphericalSeriesd *src, AranSphericalSeriesd *dst,
              double *out, int nout) {
  SeriesContext &c = sctx();
  std::lock_guard<std::mutex> lk(c.mu);
  try {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
      return fail(ARAN_ERR_NO_DEVICE, std::string("no CUDA device available: ") + cudaGetErrorString(e));
    if (c.device < 0) {
      ACHECK(cudaGetDevice(&c.device));
      ACHECK(cudaStreamCreateWithFlags(&c.st, cudaStreamNonBlocking));
    }
    ACHECK(cudaSetDevice(c.device));
    int L = 2;
    if (src) L = std::max(L, std::max((int)src->posdeg, (int)src->negdeg) + 1);
    if (dst) L = std::max(L, std::max((int)dst->posdeg, (int)dst->negdeg) + 1);
    const size_t ns = src ? series_len(src->posdeg, src->negdeg) : 0;
    const size_t nd = dst ? series_len(dst->posdeg, dst->negdeg) : 0;
    const size_t scr = scratch_doubles(op.kind, L);
    c.buf.reserve(2 * ns + 2 * nd + 8 + scr);
    double *base = c.buf.ptr;
    zd *dsrc = reinterpret_cast<zd *>(base);
    zd *ddst = reinterpret_cast<zd *>(base + 2 * ns);
    double *dout = base + 2 * ns + 2 * nd;
    op.scratch = dout + 8;
    op.src = dsrc;
    op.dst = ddst;
    op.out = dout;
    if (src) {
      op.sp = src->posdeg;
      op.sn = src->negdeg;
      ACHECK(cudaMemcpyAsync(dsrc, src->terms, ns * sizeof(zd), cudaMemcpyHostToDevice, c.st));
    }
    if (dst) {
      op.dp = dst->posdeg;
      op.dn = dst->negdeg;
      ACHECK(cudaMemcpyAsync(ddst, dst->terms, nd * sizeof(zd), cudaMemcpyHostToDevice, c.st));
    }
    k_series_op<<<1, 32, 0, c.st>>>(op);
    ACHECK(cudaGetLastError());
    std::vector<zd> res(nd);
    double o[8];
    if (dst) ACHECK(cudaMemcpyAsync(res.data(), ddst, nd * sizeof(zd), cudaMemcpyDeviceToHost, c.st));
    if (nout) ACHECK(cudaMemcpyAsync(o, dout, nout * sizeof(double), cudaMemcpyDeviceToHost, c.st));
    ACHECK(cudaStreamSynchronize(c.st));
    if (dst) std::memcpy(dst->terms, res.data(), nd * sizeof(zd));
    if (nout) std::memcpy(out, o, nout * sizeof(double));
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  return ARAN_OK;
}

SeriesOp make_op(int kind, int flavour = F_NORMAL) {
  SeriesOp o;
  std::memset(&o, 0, sizeof(o));
  o.kind = kind;
  o.flavour = flavour;
  return o;
}

void set3(double *d, const VsgVector3d *v) {
  d[0] = v->x;
  d[1] = v->y;
  d[2] = v->z;
}

void translate_f(const AranSphericalSeriesd *src, const VsgVector3d *xs, AranSphericalSeriesd *dst,
                 const VsgVector3d *xd, int kind, int flavour) {
  if (!src || !xs || !dst || !xd) return;
  SeriesOp o = make_op(kind, flavour);
  set3(o.xs, xs);
  set3(o.xd, xd);
  series_op(o, src, dst, nullptr, 0);
}

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" {

// ---- containers (aran/aransphericalseriesd.c:122-298) ----
AranSphericalSeriesd *aran_spherical_seriesd_new(guint8 posdeg, guint8 negdeg) {
  AranSphericalSeriesd *s = (AranSphericalSeriesd *)std::calloc(1, sizeof(AranSphericalSeriesd));
  s->posdeg = posdeg;
  s->negdeg = negdeg;
  s->terms = (gcomplex128 *)std::calloc(series_len(posdeg, negdeg), sizeof(gcomplex128));
  return s;
}

void aran_spherical_seriesd_free(AranSphericalSeriesd *ass) {
  if (!ass) return;
  std::free(ass->terms);
  std::free(ass);
}

void aran_spherical_seriesd_copy(const AranSphericalSeriesd *src, AranSphericalSeriesd *dst) {
  if (!src || !dst) return;
  // common degrees, the rest zero
  aran_spherical_seriesd_set_zero(dst);
  const int pd = std::min(src->posdeg, dst->posdeg), nd = std::min(src->negdeg, dst->negdeg);
  for (int l = 0; l <= pd; ++l)
    for (int m = 0; m <= l; ++m) dst->terms[tri(l, m)] = src->terms[tri(l, m)];
  const size_t so = series_len(src->posdeg, 0), dof = series_len(dst->posdeg, 0);
  for (int l = 0; l < nd; ++l)
    for (int m = 0; m <= l; ++m) dst->terms[dof + tri(l, m)] = src->terms[so + tri(l, m)];
}

AranSphericalSeriesd *aran_spherical_seriesd_clone(const AranSphericalSeriesd *src) {
  if (!src) return nullptr;
  AranSphericalSeriesd *d = aran_spherical_seriesd_new(src->posdeg, src->negdeg);
  aran_spherical_seriesd_copy(src, d);
  return d;
}

gcomplex128 *aran_spherical_seriesd_get_term(AranSphericalSeriesd *ass, gint i, gint j) {
  if (!ass || j < 0) return nullptr;
  if (i >= 0) {
    if (i > ass->posdeg || j > i) return nullptr;
    return ass->terms + tri(i, j);
  }
  int l = -i - 1;
  if (l >= ass->negdeg || j > l) return nullptr;
  return ass->terms + series_len(ass->posdeg, 0) + tri(l, j);
}

guint8 aran_spherical_seriesd_get_posdeg(const AranSphericalSeriesd *ass) {
  return ass ? ass->posdeg : 0;
}
guint8 aran_spherical_seriesd_get_negdeg(const AranSphericalSeriesd *ass) {
  return ass ? ass->negdeg : 0;
}

void aran_spherical_seriesd_set_zero(AranSphericalSeriesd *ass) {
  if (ass) std::memset(ass->terms, 0, series_len(ass->posdeg, ass->negdeg) * sizeof(gcomplex128));
}

void aran_spherical_seriesd_write(const AranSphericalSeriesd *ass, FILE *file) {
  if (!ass || !file) return;
  std::fprintf(file, "[");
  for (int l = 0; l <= ass->posdeg; ++l)
    for (int m = 0; m <= l; ++m) {
      gcomplex128 t = ass->terms[tri(l, m)];
      std::fprintf(file, "[%d,%d]:(%e,%e), ", l, m, t.real(), t.imag());
    }
  const size_t o = series_len(ass->posdeg, 0);
  for (int l = 0; l < ass->negdeg; ++l)
    for (int m = 0; m <= l; ++m) {
      gcomplex128 t = ass->terms[o + tri(l, m)];
      std::fprintf(file, "[%d,%d]:(%e,%e), ", -l - 1, m, t.real(), t.imag());
    }
  std::fprintf(file, "]");
}

void aran_spherical_seriesd_add(AranSphericalSeriesd *one, AranSphericalSeriesd *other,
                                AranSphericalSeriesd *result) {
  if (!one || !other || !result || one->posdeg != result->posdeg ||
      other->posdeg != result->posdeg || one->negdeg != result->negdeg ||
      other->negdeg != result->negdeg)
    return;
  const size_t n = series_len(result->posdeg, result->negdeg);
  for (size_t k = 0; k < n; ++k) result->terms[k] = one->terms[k] + other->terms[k];
}

// ---- computing operators (one launch each) ----
gcomplex128 aran_spherical_seriesd_evaluate_internal(const AranSphericalSeriesd *ass, gdouble r,
                                                     gdouble cost, gdouble sint, gdouble cosp,
                                                     gdouble sinp) {
  double o[2] = {0., 0.};
  if (!ass) return gcomplex128(0., 0.);
  SeriesOp op = make_op(S_EVAL);
  op.internal = 1;
  op.xs[0] = r; op.xs[1] = cost; op.xs[2] = sint; op.xd[0] = cosp; op.xd[1] = sinp;
  if (series_op(op, ass, nullptr, o, 2) != ARAN_OK) return gcomplex128(0., 0.);
  return gcomplex128(o[0], o[1]);
}

gcomplex128 aran_spherical_seriesd_evaluate(const AranSphericalSeriesd *ass, const VsgVector3d *x) {
  double o[2] = {0., 0.};
  if (!ass || !x) return gcomplex128(0., 0.);
  SeriesOp op = make_op(S_EVAL);
  set3(op.xd, x);
  if (series_op(op, ass, nullptr, o, 2) != ARAN_OK) return gcomplex128(0., 0.);
  return gcomplex128(o[0], o[1]);
}

void aran_spherical_seriesd_gradient_evaluate_internal(const AranSphericalSeriesd *ass, gdouble r,
                                                       gdouble cost, gdouble sint, gdouble cosp,
                                                       gdouble sinp, gcomplex128 *dr,
                                                       gcomplex128 *dt, gcomplex128 *dp) {
  double o[6];
  if (!ass || !dr || !dt || !dp) return;
  SeriesOp op = make_op(S_GRAD);
  op.internal = 1;
  op.xs[0] = r; op.xs[1] = cost; op.xs[2] = sint; op.xd[0] = cosp; op.xd[1] = sinp;
  if (series_op(op, ass, nullptr, o, 6) != ARAN_OK) return;
  *dr = gcomplex128(o[0], o[1]);
  *dt = gcomplex128(o[2], o[3]);
  *dp = gcomplex128(o[4], o[5]);
}

void aran_spherical_seriesd_gradient_evaluate(const AranSphericalSeriesd *ass, const VsgVector3d *x,
                                              VsgVector3d *grad) {
  double o[3];
  if (!ass || !x || !grad) return;
  SeriesOp op = make_op(S_GRAD);
  set3(op.xd, x);
  if (series_op(op, ass, nullptr, o, 3) != ARAN_OK) return;
  grad->x = o[0];
  grad->y = o[1];
  grad->z = o[2];
}

void aran_spherical_seriesd_rotate(const AranSphericalSeriesd *src, gdouble alpha, gdouble beta,
                                   gdouble gamma, AranSphericalSeriesd *dst) {
  if (!src || !dst) return;
  SeriesOp op = make_op(S_ROTATE);
  op.a = alpha; op.b = beta; op.g = gamma;
  series_op(op, src, dst, nullptr, 0);
}

void aran_spherical_seriesd_rotate_inverse(const AranSphericalSeriesd *src, gdouble alpha,
                                           gdouble beta, gdouble gamma, AranSphericalSeriesd *dst) {
  if (!src || !dst) return;
  SeriesOp op = make_op(S_ROTATE_INV);
  op.a = alpha; op.b = beta; op.g = gamma;
  series_op(op, src, dst, nullptr, 0);
}

void aran_spherical_seriesd_translate(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                      AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TRANSLATE, F_NORMAL);
}
void aran_spherical_seriesd_to_local(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                     AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TO_LOCAL, F_NORMAL);
}
void aran_spherical_seriesd_translate_kkylin(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                             AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TRANSLATE, F_KKYLIN);
}
void aran_spherical_seriesd_to_local_kkylin(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                            AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TO_LOCAL, F_KKYLIN);
}
void aran_spherical_seriesd_translate_rotate(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                             AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TRANSLATE, F_ROTATE);
}
void aran_spherical_seriesd_to_local_rotate(const AranSphericalSeriesd *src, const VsgVector3d *xsrc,
                                            AranSphericalSeriesd *dst, const VsgVector3d *xdst) {
  translate_f(src, xsrc, dst, xdst, S_TO_LOCAL, F_ROTATE);
}

// ---- 3D development (aran/arandevelopment3d.c:64-568) ----
static const GType kDevelopmentType = 0x41524433;  // "ARD3"

GType aran_development3d_get_type(void) { return kDevelopmentType; }

AranDevelopment3d *aran_development3d_new(guint8 posdeg, guint8 negdeg) {
  AranDevelopment3d *d = (AranDevelopment3d *)std::malloc(sizeof(AranDevelopment3d));
  d->multipole = aran_spherical_seriesd_new(posdeg, negdeg);
  d->local = aran_spherical_seriesd_new(posdeg > negdeg ? posdeg : negdeg, 0);
  return d;
}

void aran_development3d_free(AranDevelopment3d *ad) {
  if (!ad) return;
  aran_spherical_seriesd_free(ad->multipole);
  aran_spherical_seriesd_free(ad->local);
  std::free(ad);
}

void aran_development3d_copy(const AranDevelopment3d *src, AranDevelopment3d *dst) {
  if (!src || !dst) return;
  aran_spherical_seriesd_copy(src->multipole, dst->multipole);
  aran_spherical_seriesd_copy(src->local, dst->local);
}

AranDevelopment3d *aran_development3d_clone(AranDevelopment3d *src) {
  if (!src) return nullptr;
  AranDevelopment3d *d = aran_development3d_new(src->multipole->posdeg, src->multipole->negdeg);
  aran_development3d_copy(src, d);
  return d;
}

void aran_development3d_set_zero(AranDevelopment3d *ad) {
  if (!ad) return;
  aran_spherical_seriesd_set_zero(ad->multipole);
  aran_spherical_seriesd_set_zero(ad->local);
}

void aran_development3d_write(AranDevelopment3d *ad, FILE *file) {
  if (!ad || !file) return;
  std::fprintf(file, "{multipole= ");
  aran_spherical_seriesd_write(ad->multipole, file);
  std::fprintf(file, ", local= ");
  aran_spherical_seriesd_write(ad->local, file);
  std::fprintf(file, "}");
}

void aran_development3d_p2m(const VsgVector3d *position, const gdouble charge,
                            const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst) {
  if (!position || !dst_node || !dst) return;
  SeriesOp op = make_op(S_P2M);
  set3(op.xs, position);
  set3(op.xd, &dst_node->center);
  op.q = charge;
  series_op(op, nullptr, dst->multipole, nullptr, 0);
}

void aran_development3d_p2l(const VsgVector3d *position, const gdouble charge,
                            const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst) {
  if (!position || !dst_node || !dst) return;
  SeriesOp op = make_op(S_P2L);
  set3(op.xs, position);
  set3(op.xd, &dst_node->center);
  op.q = charge;
  series_op(op, nullptr, dst->local, nullptr, 0);
}

#define ARAN_DEV3_TRANSLATE(name, part_src, part_dst, kind, flavour)                         \
  void name(const VsgPRTree3dNodeInfo *src_node, AranDevelopment3d *src,                     \
            const VsgPRTree3dNodeInfo *dst_node, AranDevelopment3d *dst) {                   \
    if (!src_node || !src || !dst_node || !dst) return;                                      \
    translate_f(src->part_src, &src_node->center, dst->part_dst, &dst_node->center, kind,     \
                flavour);                                                                    \
  }
ARAN_DEV3_TRANSLATE(aran_development3d_m2m, multipole, multipole, S_TRANSLATE, F_NORMAL)
ARAN_DEV3_TRANSLATE(aran_development3d_m2l, multipole, local, S_TO_LOCAL, F_NORMAL)
ARAN_DEV3_TRANSLATE(aran_development3d_l2l, local, local, S_TRANSLATE, F_NORMAL)
ARAN_DEV3_TRANSLATE(aran_development3d_m2m_kkylin, multipole, multipole, S_TRANSLATE, F_KKYLIN)
ARAN_DEV3_TRANSLATE(aran_development3d_m2l_kkylin, multipole, local, S_TO_LOCAL, F_KKYLIN)
ARAN_DEV3_TRANSLATE(aran_development3d_l2l_kkylin, local, local, S_TRANSLATE, F_KKYLIN)
ARAN_DEV3_TRANSLATE(aran_development3d_m2m_rotate, multipole, multipole, S_TRANSLATE, F_ROTATE)
ARAN_DEV3_TRANSLATE(aran_development3d_m2l_rotate, multipole, local, S_TO_LOCAL, F_ROTATE)
ARAN_DEV3_TRANSLATE(aran_development3d_l2l_rotate, local, local, S_TRANSLATE, F_ROTATE)
#undef ARAN_DEV3_TRANSLATE

static VsgVector3d rel_to(const VsgPRTree3dNodeInfo *node, const VsgVector3d *pos) {
  VsgVector3d v = {pos->x - node->center.x, pos->y - node->center.y, pos->z - node->center.z};
  return v;
}

gcomplex128 aran_development3d_multipole_evaluate(const VsgPRTree3dNodeInfo *devel_node,
                                                  AranDevelopment3d *devel, const VsgVector3d *pos) {
  if (!devel_node || !devel || !pos) return gcomplex128(0., 0.);
  VsgVector3d v = rel_to(devel_node, pos);
  return aran_spherical_seriesd_evaluate(devel->multipole, &v);
}

gcomplex128 aran_development3d_local_evaluate(const VsgPRTree3dNodeInfo *devel_node,
                                              AranDevelopment3d *devel, const VsgVector3d *pos) {
  if (!devel_node || !devel || !pos) return gcomplex128(0., 0.);
  VsgVector3d v = rel_to(devel_node, pos);
  return aran_spherical_seriesd_evaluate(devel->local, &v);
}

gcomplex128 aran_development3d_m2p(const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                                   const VsgVector3d *pos) {
  return aran_development3d_multipole_evaluate(devel_node, devel, pos);
}

gcomplex128 aran_development3d_l2p(const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                                   const VsgVector3d *pos) {
  return aran_development3d_local_evaluate(devel_node, devel, pos);
}

void aran_development3d_multipole_gradient_evaluate(const VsgPRTree3dNodeInfo *devel_node,
                                                    AranDevelopment3d *devel,
                                                    const VsgVector3d *pos, VsgVector3d *grad) {
  if (!devel_node || !devel || !pos || !grad) return;
  VsgVector3d v = rel_to(devel_node, pos);
  aran_spherical_seriesd_gradient_evaluate(devel->multipole, &v, grad);
}

void aran_development3d_local_gradient_evaluate(const VsgPRTree3dNodeInfo *devel_node,
                                                AranDevelopment3d *devel, const VsgVector3d *pos,
                                                VsgVector3d *grad) {
  if (!devel_node || !devel || !pos || !grad) return;
  VsgVector3d v = rel_to(devel_node, pos);
  aran_spherical_seriesd_gradient_evaluate(devel->local, &v, grad);
}

void aran_development3d_m2pv(const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                             const VsgVector3d *pos, VsgVector3d *grad) {
  aran_development3d_multipole_gradient_evaluate(devel_node, devel, pos, grad);
}

void aran_development3d_l2pv(const VsgPRTree3dNodeInfo *devel_node, AranDevelopment3d *devel,
                             const VsgVector3d *pos, VsgVector3d *grad) {
  aran_development3d_local_gradient_evaluate(devel_node, devel, pos, grad);
}

}  // extern "C"
