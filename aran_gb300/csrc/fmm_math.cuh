// fmm_math.cuh -- per-item FMM math shared by the sm_103a kernels.
//
// Everything here is __host__ __device__ so the table generators can run on
// the device (one thread per table) and the same definitions can be checked
// on the host against the oracle.
//
// Conventions (LibAran's, aran/aransphericalseriesd-private.h:38-99):
//   Y_l^m = N_l^m P_l^m(cos t) e^{i m p}, Condon-Shortley phase,
//   N_l^m = sqrt((2l+1)/4pi (l-m)!/(l+m)!) (aran/aransphericalharmonic.c:31-38);
//   a series stores m >= 0 only, term (l,m) at l(l+1)/2+m, and the m < 0 half
//   is (-1)^m conj(term(l,|m|)).
//   Multipole: M_l^m = sum q 4pi/(2l+1) r^l conj(Y_l^m), l < p
//   (aran/arandevelopment3d.c:169-216); local: degrees 0..p.
//
// Device storage is *scaled*: a node at depth d with scale h_d = 2^(E-d)
// (2^E >= the root box extent) stores Mhat_l = M_l / h^l and
// Lhat_l = L_l * h^l.  h is a power of two, so the scaling is exact in FP64
// and keeps FP32 coefficients in range at any depth.
#pragma once

#include <cstdint>
#include <cmath>

#ifndef __CUDACC__
#define __host__
#define __device__
#define __forceinline__ inline
#endif

#define FMM_HD __host__ __device__ __forceinline__

namespace aran {

constexpr int kKeyBits = 21;     // quantisation bits per axis (63-bit keys)
constexpr int kMaxOrder = 30;    // largest supported p
constexpr double kPi = 3.1415926535897932384626433832795028841971693993751;

FMM_HD int tri(int l) { return (l * (l + 1)) / 2; }
FMM_HD int tri(int l, int m) { return (l * (l + 1)) / 2 + m; }
// number of multipole / local coefficients (m >= 0) at order p
FMM_HD int n_mult(int p) { return tri(p); }           // degrees 0..p-1
FMM_HD int n_local(int p) { return tri(p + 1); }      // degrees 0..p
// packed (l+1)x(l+1) block offsets for rotation tables, degrees 0..L-1
// (l, m) of the k-th coefficient in m-major order (m = 0: l = 0..p, m = 1:
// l = 1..p, ...): the vertical stage walks coefficients in this order so the
// 32 lanes of a round share m and hence their trip count
FMM_HD void mmajor_lm(int k, int p, int &l, int &m) {
  m = 0;
  while (k > p - m) {
    k -= p + 1 - m;
    ++m;
  }
  l = m + k;
}

// Compact M2L tables.  Rotation planes: plane m (source order) holds the
// entries of the coefficients c = (l, m'), l >= m, which in tri order are
// c = tri(m) .. nc-1; plane m starts at m2l_plane_off(nc, m), entry c at
// m2l_plane_off(nc, m) + c - tri(m).
FMM_HD int m2l_plane_off(int nc, int m) { return m * nc - ((m - 1) * m * (m + 1)) / 6; }
// Vertical rows: row n (source degree) holds the m-major slots k with
// m(k) <= n, i.e. k < (n+1)(p+1) - n(n+1)/2; row n starts at m2l_vrow_off.
FMM_HD int m2l_vrow_len(int p, int n) { return (n + 1) * (p + 1) - ((n + 1) * n) / 2; }
FMM_HD int m2l_vrow_off(int p, int n) {
  return (p + 1) * (n * (n + 1) / 2) - ((n + 1) * n * (n - 1)) / 6;
}

// Stream layout of the lane-parallel M2L tables (FP32, order p), one block
// per offset, in the order the kernel consumes it:
//  * the z-phases (cos, sin) of m = 0..p;
//  * the forward rotation terms (l < p, m' <= l, m <= m'): the lower
//    triangle of each even/odd Wigner block, the upper one following from
//    E[m][m'] = (-1)^{m-m'} E[m'][m] for m, m' > 0, E[0][m] = 2 (-1)^m E[m][0]
//    and O[0][m] = 0; degree l scaled by 1/beta_l; in groups of four, each
//    group four even-part factors then four odd-part factors;
//  * the vertical factors times the offset's radial powers, which are
//    V(j, m, n) = (-1)^{j+m} beta_j / beta_n S(j, n) with S symmetric in
//    (j, n): per m, the lower triangle of S over j, n in [m, p) (rows j,
//    columns n <= j), then the row j = p;
//  * the backward rotation terms (l <= p), grouped like the forward ones,
//    column m of degree l scaled by (-1)^{l+m} beta_l, which makes each block
//    symmetric (F[m][m'] = F[m'][m] for m, m' > 0, F[0][m] = 2 F[m][0] for
//    the even part, 0 for the odd one).
__host__ __device__ constexpr int m2l_lane_tet(int l) { return l * (l + 1) * (l + 2) / 6; }
__host__ __device__ constexpr int m2l_lane_nf(int p) { return m2l_lane_tet(p); }
__host__ __device__ constexpr int m2l_lane_nb(int p) { return m2l_lane_tet(p + 1); }
// vertical terms of the orders m..p: sum over k = p - m of k (k + 3) / 2
__host__ __device__ constexpr int m2l_lane_vtail(int k) { return k * (k + 1) * (k + 5) / 6; }
__host__ __device__ constexpr int m2l_lane_nv(int p) { return m2l_lane_vtail(p); }
__host__ __device__ constexpr int m2l_lane_f(int p) { return (2 * (p + 1) + 3) & ~3; }
__host__ __device__ constexpr int m2l_lane_v(int p) {
  return m2l_lane_f(p) + 8 * ((m2l_lane_nf(p) + 3) / 4);
}
__host__ __device__ constexpr int m2l_lane_b(int p) {
  return m2l_lane_v(p) + 4 * ((m2l_lane_nv(p) + 3) / 4);
}
__host__ __device__ constexpr int m2l_lane_stride(int p) {
  return m2l_lane_b(p) + 8 * ((m2l_lane_nb(p) + 3) / 4);
}
// index of the first vertical term of order m
__host__ __device__ constexpr int m2l_lane_vpre(int p, int m) {
  return m2l_lane_vtail(p) - m2l_lane_vtail(p - m);
}
// orders with a lane-parallel M2L kernel
__host__ __device__ constexpr bool m2l_lane_order(int p) { return p == 4 || p == 8 || p == 12; }

FMM_HD int sq_off(int l) { return (l * (l + 1) * (2 * l + 1)) / 6; }  // sum_{i<l} (i+1)^2
FMM_HD int sq_size(int L) { return sq_off(L); }

template <typename T> struct cplx { T re, im; };

template <typename T> FMM_HD cplx<T> cmake(T a, T b) { cplx<T> z; z.re = a; z.im = b; return z; }
template <typename T> FMM_HD cplx<T> cadd(cplx<T> a, cplx<T> b) { return cmake(a.re + b.re, a.im + b.im); }
template <typename T> FMM_HD cplx<T> cmul(cplx<T> a, cplx<T> b) {
  return cmake(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
template <typename T> FMM_HD cplx<T> cconj(cplx<T> a) { return cmake(a.re, -a.im); }
template <typename T> FMM_HD cplx<T> cscale(cplx<T> a, T s) { return cmake(a.re * s, a.im * s); }

// ---------------------------------------------------------------------------
// Morton keys.  A point's key is the 3x21-bit interleave of its quantised
// coordinates floor((x - lb) * 2^21 / (ub - lb)), clamped to [0, 2^21).
// Bit 3b holds x, 3b+1 y, 3b+2 z.
// ---------------------------------------------------------------------------
FMM_HD uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

FMM_HD uint32_t compact3(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
  v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
  v = (v ^ (v >> 32)) & 0x1fffffull;
  return (uint32_t)v;
}

// the point's position in finest cells, (x - lb) * scale, rounded as the
// oracle rounds it
FMM_HD double cell_pos(double x, double lb, double scale) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(__dsub_rn(x, lb), scale);
#else
  return (x - lb) * scale;
#endif
}

// the finest cell of position t (cell_pos), not clamped
FMM_HD int64_t cell_index(double t) { return (int64_t)floor(t); }

// a cell index clamped into the box
FMM_HD int64_t cell_clamp(int64_t i) {
  if (i < 0) i = 0;
  if (i > (1 << kKeyBits) - 1) i = (1 << kKeyBits) - 1;
  return i;
}

// a point more than one finest cell outside the closed box (a point on the
// upper bound, or within rounding of it, is inside)
FMM_HD bool cell_outside(int64_t i) { return i < -1 || i > (1 << kKeyBits); }

// centre of the node with integer coordinates c at depth d, by repeated
// halving of the root box [lb, ub] (the oracle performs the same sequence).
FMM_HD double node_center_axis(double lb, double ub, int d, int32_t c) {
  double lo = lb, hi = ub;
  for (int b = d - 1; b >= 0; --b) {
#ifdef __CUDA_ARCH__
    double mid = __dmul_rn(__dadd_rn(lo, hi), 0.5);
#else
    double mid = (lo + hi) * 0.5;
#endif
    if ((c >> b) & 1) lo = mid; else hi = mid;
  }
#ifdef __CUDA_ARCH__
  return __dmul_rn(__dadd_rn(lo, hi), 0.5);
#else
  return (lo + hi) * 0.5;
#endif
}

// ---------------------------------------------------------------------------
// Table generators (run once per order on the device, FP64).
// ---------------------------------------------------------------------------

// N_l^m by the reference recurrence (aran/aransphericalharmonic.c:31-38).
FMM_HD void gen_hnorm(int L, double *nrm) {
  for (int l = 0; l <= L; ++l)
    for (int m = 0; m <= l; ++m) {
      double v;
      if (m == 0) v = sqrt((l + l + 1.) / (4. * kPi));
      else v = nrm[tri(l, m - 1)] / sqrt((double)((unsigned)(l - m + 1) * (unsigned)(l + m)));
      nrm[tri(l, m)] = v;
    }
}

// alpha_l^m = 1/sqrt((l-m)!(l+m)!) by aran/aransphericalseriesd.c:45-60.
FMM_HD void gen_alpha(int L, double *a) {
  for (int l = 0; l <= L; ++l)
    for (int m = 0; m <= l; ++m) {
      double v;
      if (l == 0) v = 1.;
      else if (m == 0) v = a[tri(l - 1, 0)] / l;
      else if (l == m) v = a[tri(l - 1, l - 1)] / sqrt((l + l - 1.) * (l + l));
      else v = sqrt((l - m + 1.) / (l + m)) * a[tri(l, m - 1)];
      a[tri(l, m)] = v;
    }
}

FMM_HD double beta_l(int l) { return sqrt((4. * kPi) / (l + l + 1.)); }

// Recurrence coefficients for the normalised regular solid harmonics
// S_l^m(x) = r^l Y_l^m (m >= 0), computed without trigonometry:
//   S_m^m   = a_m (x + i y) S_{m-1}^{m-1}
//   S_m+1^m = b_m z S_m^m
//   S_l^m   = c_lm z S_{l-1}^m - d_lm r^2 S_{l-2}^m
// (restating the Legendre recurrence of aran/aranlegendre.c:135-169 scaled
// by r^l N_l^m).  Layout: rec[4*tri(l,m) + {0:a_or_c, 1:b_or_d}].
FMM_HD void gen_solid_rec(int L, const double *nrm, double *rec) {
  for (int l = 0; l <= L; ++l)
    for (int m = 0; m <= l; ++m) {
      double c0 = 0., c1 = 0.;
      if (l == 0) { c0 = nrm[0]; c1 = 0.; }
      else if (m == l) { c0 = -(2. * m - 1.) * nrm[tri(m, m)] / nrm[tri(m - 1, m - 1)]; }
      else if (l == m + 1) { c0 = (2. * m + 1.) * nrm[tri(m + 1, m)] / nrm[tri(m, m)]; }
      else {
        c0 = (2. * l - 1.) / (double)(l - m) * nrm[tri(l, m)] / nrm[tri(l - 1, m)];
        c1 = (double)(l + m - 1) / (double)(l - m) * nrm[tri(l, m)] / nrm[tri(l - 2, m)];
      }
      rec[2 * tri(l, m)] = c0;
      rec[2 * tri(l, m) + 1] = c1;
    }
}

// Derivative coefficients of the regular solid harmonics S_l^m = r^l Y_l^m:
// with K_l^m = (-1)^m sqrt((2l+1)/4pi) sqrt((l-m)!(l+m)!) (K_l^-m = K_l^m),
//   d/dz S_l^m          = (K_l^m / K_{l-1}^m)         S_{l-1}^m
//   (d/dx - i d/dy) S_l^m = (K_l^m / K_{l-1}^{m-1})   S_{l-1}^{m-1}
// Stored per target degree l' = l-1 and order m' in [-l', l'] as
//   gz[tri(l')+|m'|]    = K_{l'+1}^{m'} / K_{l'}^{m'}  (m' >= 0)
//   gm[l'*l' + l' + m'] = K_{l'+1}^{m'+1} / K_{l'}^{m'}
FMM_HD void gen_grad_coefs(int L, double *gz, double *gm) {
  for (int lp = 0; lp < L; ++lp) {
    int l = lp + 1;
    for (int m = 0; m <= lp; ++m) {
      // K_l^m/K_{l-1}^m = sqrt((2l+1)/(2l-1)) sqrt((l-m)(l+m))
      gz[tri(lp, m)] = sqrt((2. * l + 1.) / (2. * l - 1.)) * sqrt((double)(l - m) * (double)(l + m));
    }
    for (int mp = -lp; mp <= lp; ++mp) {
      int m = mp + 1;  // source order at degree l
      int am = m < 0 ? -m : m, amp = mp < 0 ? -mp : mp;
      // K_l^m / K_{l-1}^{mp}: sign (-1)^{am - amp}
      double sgn = ((am + amp) & 1) ? -1. : 1.;
      // sqrt((l-am)!(l+am)! / ((l-1-amp)!(l-1+amp)!))
      double r = 1.;
      // compute ratio of factorials incrementally in log-free form
      // (l-am)!/(l-1-amp)!  and (l+am)!/(l-1+amp)!
      int a1 = l - am, b1 = l - 1 - amp, a2 = l + am, b2 = l - 1 + amp;
      double num = 1., den = 1.;
      if (a1 >= b1) { for (int k = b1 + 1; k <= a1; ++k) num *= k; }
      else { for (int k = a1 + 1; k <= b1; ++k) den *= k; }
      if (a2 >= b2) { for (int k = b2 + 1; k <= a2; ++k) num *= k; }
      else { for (int k = a2 + 1; k <= b2; ++k) den *= k; }
      r = sqrt(num / den);
      gm[lp * lp + lp + mp] = sgn * sqrt((2. * l + 1.) / (2. * l - 1.)) * r;
    }
  }
}

// ---------------------------------------------------------------------------
// Wigner small-d matrix d_l^{m,m'}(beta) for l <= L by the ten recurrence
// blocks of aran/aranwigner.c:83-246.  Output packed [l][m'][l+m]
// (m' in 0..l, m in -l..l), real (no phases: the rotation kernels apply
// e^{i m phi} separately).
// ---------------------------------------------------------------------------
FMM_HD int wig_off(int l) { return (l * (l + 1) * (4 * l - 1)) / 6; }
FMM_HD int wig_size(int L) { return ((L + 1) * (L + 2) * (4 * L + 3)) / 6; }

FMM_HD void gen_wigner_d(int L, double beta, double *w) {
#define WD(l, mp, m) w[wig_off(l) + (mp) * (2 * (l) + 1) + (l) + (m)]
  double cb = cos(beta), sb = sin(beta);
  double cb2 = cos(beta * 0.5), sb2 = sin(beta * 0.5);
  double tb2 = sb2 / cb2;
  WD(0, 0, 0) = 1.;
  if (L == 0) return;
  WD(1, 0, 0) = cb;
  WD(1, 1, -1) = sb2 * sb2;
  WD(1, 1, 0) = sb / sqrt(2.);
  WD(1, 1, 1) = cb2 * cb2;
  WD(1, 0, -1) = WD(1, 1, 0);
  WD(1, 0, 1) = -WD(1, 1, 0);
  if (L <= 1) return;
  double d100 = WD(1, 0, 0), d111 = WD(1, 1, 1), d11m1 = WD(1, 1, -1);
  for (int l = 2; l <= L; ++l) {
    double tl1 = l + l - 1., sql = l * l, sql1 = (l - 1.) * (l - 1.);
    for (int mp = 0; mp <= l - 2; ++mp) {
      double sqmp = mp * mp;
      for (int m = -mp; m <= mp; ++m) {
        double sqm = m * m;
        double a = (l * tl1) / sqrt((sql - sqmp) * (sql - sqm));
        double b = (d100 - ((mp * m) / (l * (l - 1.))));
        double c = sqrt((sql1 - sqmp) * (sql1 - sqm)) / ((l - 1.) * tl1);
        WD(l, mp, m) = a * (b * WD(l - 1, mp, m) - c * WD(l - 2, mp, m));
      }
    }
    WD(l, l, l) = d111 * WD(l - 1, l - 1, l - 1);
    WD(l, l - 1, l - 1) = (l * d100 - l + 1.) * WD(l - 1, l - 1, l - 1);
    WD(l, l, -l) = d11m1 * WD(l - 1, l - 1, -(l - 1));
    WD(l, l - 1, -(l - 1)) = (l * d100 + l - 1.) * WD(l - 1, l - 1, -(l - 1));
    for (int mp = l; mp >= 1; --mp)
      WD(l, mp - 1, l) = -sqrt((l + mp) / (l - mp + 1.)) * tb2 * WD(l, mp, l);
    for (int mp = l - 1; mp >= 1; --mp) {
      double a = sqrt(((double)l + mp) / (((double)l + l) * (l - mp + 1.)));
      WD(l, mp - 1, l - 1) = (l * cb - mp + 1.) * a * WD(l, mp, l) / d111;
    }
    for (int mp = l - 1; mp <= l; ++mp)
      for (int m = 0; m < mp; ++m)
        WD(l, mp, m) = (((mp + m) & 1) ? -1. : 1.) * WD(l, m, mp);
    for (int m = 0; m < l; ++m)
      WD(l, l, -m - 1) = sqrt((l - m) / (l + m + 1.)) * tb2 * WD(l, l, -m);
    for (int m = 0; m < l; ++m) {
      double a = sqrt(((double)l - m) / (((double)l + l) * (l + m + 1.)));
      WD(l, l - 1, -m - 1) = (l * cb + m + 1.) * a * WD(l, l, -m) / d111;
    }
    for (int mp = 0; mp <= l; ++mp)
      for (int m = mp + 1; m <= l; ++m) {
        WD(l, mp, m) = (((m + mp) & 1) ? -1. : 1.) * WD(l, m, mp);
        WD(l, mp, -m) = WD(l, m, -mp);
      }
  }
#undef WD
}

// Even/odd rotation blocks.  For a "real" series (c^{-m} = (-1)^m conj c^m)
// rotated by y(beta) after the z-phase, with d = d_l^{m,m'}(beta) as stored by
// gen_wigner_d ([l][m'][l+m]):
//   Re out^{m'} = sum_{m>=0} E[m'][m] Re in^m,  Im out^{m'} = sum O[m'][m] Im in^m
//   E[m'][0] = O[m'][0] = d^{0,m'}, and for m > 0
//   E[m'][m] = d^{m,m'} + (-1)^m d^{-m,m'},  O[m'][m] = d^{m,m'} - (-1)^m d^{-m,m'}.
// Blocks for degree l are (l+1)x(l+1) at sq_off(l), row m', column m, for
// degrees 0..L-1.  The inverse rotation of LibAran looks up the angles
// (-gamma, -beta, -alpha) (aran/aransphericalseriesd-rotate.c:130-153), so its
// blocks come from gen_wigner_d at -beta.
FMM_HD void wigner_to_eo(int L, const double *w, double *E, double *O) {
  for (int l = 0; l < L; ++l) {
    int base = sq_off(l);
    for (int mp = 0; mp <= l; ++mp)
      for (int m = 0; m <= l; ++m) {
        double dp = w[wig_off(l) + mp * (2 * l + 1) + l + m];
        double dn = w[wig_off(l) + mp * (2 * l + 1) + l - m];
        double e, o;
        if (m == 0) { e = dp; o = dp; }
        else {
          double sg = (m & 1) ? -1. : 1.;
          e = dp + sg * dn;
          o = dp - sg * dn;
        }
        E[base + mp * (l + 1) + m] = e;
        O[base + mp * (l + 1) + m] = o;
      }
  }
}

}  // namespace aran
