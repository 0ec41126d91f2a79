// tables.cu -- operator tables generated on the device in FP64.
//
// LibAran builds its tables lazily on the host (alpha/beta:
// aran/aransphericalseriesd.c:40-60; vertical translation:
// aran/aransphericalseriesd-translate.c:117-297; Wigner matrices per angle
// triple: aran/aranwigner.c:83-313, cached by aran/aranwignerrepo.c:57-82).
// Here they are generated once per (order, box aspect) on the GPU:
//  * scalar tables (one thread): solid-harmonic recurrence, P2M factors,
//    vertical M2L/M2M/L2L factors, gradient factors;
//  * direction tables (one thread per direction): the even/odd Wigner blocks
//    for the rotation at theta and at -theta, the z-phases e^{i m phi} and
//    the radial powers of every translation the tree can produce: the 343
//    same-depth M2L offsets and the 8 child<->parent octants.
// The FP32 path gets an FP32 copy of the same FP64 values.
#include "internal.cuh"

namespace aran {

namespace {

struct DirLayout {
  int Lf, Li, nrp;
  int ef, of, ei, oi, ph, rp, vv, stride;
};

__host__ __device__ DirLayout dir_layout(int p, int kind) {
  DirLayout d;
  if (kind == 0) {  // M2L: (E, O) interleaved, [m][coefficient] planes
    d.Lf = p; d.Li = p + 1; d.nrp = 2 * p + 2;
    d.ef = 0;
    d.of = -1;
    d.ei = 2 * m2l_plane_off(tri(d.Lf), d.Lf);
    d.oi = -1;
    d.ph = d.ei + 2 * m2l_plane_off(tri(d.Li), d.Li);
    d.rp = d.ph + 2 * (p + 1);
    // vertical factors times the radial powers of this offset, m-major
    // slot k of the local, source degree n: vv[m2l_vrow_off(p, n) + k]
    d.vv = ((d.rp + d.nrp) + 3) & ~3;
    d.stride = ((d.vv + m2l_vrow_off(p, p)) + 3) & ~3;
    return d;
  } else if (kind == 1) { d.Lf = p; d.Li = p; d.nrp = p + 1; }          // M2M
  else { d.Lf = p + 1; d.Li = p + 1; d.nrp = p + 2; }                 // L2L
  d.ef = 0;
  d.of = d.ef + sq_size(d.Lf);
  d.ei = d.of + sq_size(d.Lf);
  d.oi = d.ei + sq_size(d.Li);
  d.ph = d.oi + sq_size(d.Li);
  d.rp = d.ph + 2 * (p + 1);
  d.vv = -1;
  d.stride = ((d.rp + d.nrp) + 3) & ~3;
  return d;
}

template <typename T>
__global__ void k_scalar_tables(int p, double *scratch, T *rec, T *p2mf, T *vt, T *vm, T *vl,
                                T *gz, T *gm, uint8_t *lm) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  int La = 2 * p + 2;
  double *nrm = scratch;                   // tri(p+2)
  double *alpha = nrm + tri(p + 2);        // tri(La+1)
  double *rec64 = alpha + tri(La + 1);     // 2 tri(p+2)
  double *gz64 = rec64 + 2 * tri(p + 2);   // tri(p+1)
  double *gm64 = gz64 + tri(p + 1);        // (p+1)^2
  gen_hnorm(p + 1, nrm);
  gen_alpha(La, alpha);
  gen_solid_rec(p, nrm, rec64);
  for (int i = 0; i < 2 * tri(p + 1); ++i) rec[i] = (T)rec64[i];
  for (int l = 0; l <= p; ++l) p2mf[l] = (T)(4. * kPi / (l + l + 1.));
  for (int l = 0; l <= p; ++l)
    for (int m = 0; m <= l; ++m) {
      lm[2 * tri(l, m)] = (uint8_t)l;
      lm[2 * tri(l, m) + 1] = (uint8_t)m;
      // M2L vertical: (-1)^{l+m} beta_l/beta_n alpha_l^m alpha_n^m / alpha_{l+n}^0
      // (aran/aransphericalseriesd-translate.c:259-268,664-672)
      for (int n = 0; n < p; ++n) {
        double v = 0.;
        if (n >= m) {
          double normaliz = beta_l(l) / beta_l(n);
          double factor = alpha[tri(l, m)] * alpha[tri(n, m)];
          v = normaliz * factor / alpha[tri(l + n, 0)];
          if ((l + m) & 1) v = -v;
        }
        vt[tri(l, m) * p + n] = (T)v;
      }
      // L2L vertical (aran/aransphericalseriesd-translate.c:338-361), 2^-l folded
      for (int n = 0; n <= p; ++n) {
        double v = 0.;
        if (n >= l) {
          double factor = alpha[tri(n - l, 0)] * alpha[tri(l, m)] / alpha[tri(n, m)];
          v = factor * (beta_l(l) / beta_l(n)) * ldexp(1., -l);
        }
        vl[tri(l, m) * (p + 1) + n] = (T)v;
      }
      // M2M vertical (aran/aransphericalseriesd-translate.c:477-503), 2^-l folded
      if (l < p)
        for (int n = 0; n < p; ++n) {
          double v = 0.;
          if (n >= m && n <= l) {
            double factor = alpha[tri(l - n, 0)] * alpha[tri(n, m)] / alpha[tri(l, m)];
            v = factor * (beta_l(l) / beta_l(n)) * ldexp(1., -l);
          }
          vm[tri(l, m) * p + n] = (T)v;
        }
    }
  gen_grad_coefs(p, gz64, gm64);
  for (int i = 0; i < tri(p); ++i) gz[i] = (T)gz64[i];
  for (int i = 0; i < p * p; ++i) gm[i] = (T)gm64[i];
}

// M2L: the vertical factors (sign folded) times the offset's radial powers,
// so the translation along z takes one factor per term
template <typename T>
__global__ void k_m2l_vertical(int p, int ndir, int stride, int rp_off, int vv_off,
                               const T *__restrict__ vt, T *__restrict__ dirs) {
  const int nl = tri(p + 1);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)ndir * nl * p) return;
  const int d = (int)(i / (nl * p)), e = (int)(i % (nl * p));
  const int k = e % nl, n = e / nl;
  if (k >= m2l_vrow_len(p, n)) return;   // slot of order m > n: not stored
  int l, m;
  mmajor_lm(k, p, l, m);
  T *tb = dirs + (size_t)d * stride;
  tb[vv_off + m2l_vrow_off(p, n) + k] = vt[tri(l, m) * p + n] * tb[rp_off + l + n + 1];
}

// lane-parallel M2L stream tables (layout: m2l_lane_* in fmm_math.cuh),
// gathered from the FP32 offset tables: same factors, consumption order
__global__ void k_m2l_lane_tables(int p, int ndir, const float *__restrict__ src, DirLayout D,
                                  float *__restrict__ dst) {
  const int stride = m2l_lane_stride(p);
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= (int64_t)ndir * stride) return;
  const int d = (int)(i / stride), e = (int)(i % stride);
  const float *s = src + (size_t)d * D.stride;
  const int F = m2l_lane_f(p), V = m2l_lane_v(p), B = m2l_lane_b(p);
  // q-th float of a grouped rotation stream: term 4 (q / 8) + q % 4, part
  // (q / 4) % 2; term t = tet(l) + m'(m'+1)/2 + m is row m', column m of
  // degree l
  auto rot = [&](int q, int nterm, int nc, int base, bool back) -> float {
    const int t = 4 * (q >> 3) + (q & 3), part = (q >> 2) & 1;
    if (t >= nterm) return 0.f;
    int l = 0;
    while (m2l_lane_tet(l + 1) <= t) ++l;
    int r = t - m2l_lane_tet(l), mp = 0;
    while (tri(mp + 1) <= r) ++mp;
    const int m = r - tri(mp);
    const double f = back ? (((l + m) & 1) ? -beta_l(l) : beta_l(l)) : 1. / beta_l(l);
    return (float)(f * s[base + 2 * (m2l_plane_off(nc, m) + tri(l, mp) - tri(m)) + part]);
  };
  float v = 0.f;
  if (e < F) {
    if (e < 2 * (p + 1)) v = s[D.ph + e];
  } else if (e < V) {
    v = rot(e - F, m2l_lane_nf(p), tri(p), D.ef, false);
  } else if (e < B) {
    const int t = e - V;
    if (t < m2l_lane_nv(p)) {
      int m = 0;
      while (m2l_lane_vpre(p, m + 1) <= t) ++m;
      const int r = t - m2l_lane_vpre(p, m), k = p - m;
      int j, n;
      if (r < tri(k)) {          // lower triangle: row j, column n <= j
        int jj = 0;
        while (tri(jj + 1) <= r) ++jj;
        j = m + jj;
        n = m + (r - tri(jj));
      } else {                   // row j = p
        j = p;
        n = m + (r - tri(k));
      }
      const int slot = m * (p + 1) - m * (m - 1) / 2 + (j - m);   // m-major slot of (j, m)
      const double sg = ((j + m) & 1) ? -1. : 1.;
      v = (float)(sg * beta_l(n) / beta_l(j) * s[D.vv + m2l_vrow_off(p, n) + slot]);
    }
  } else {
    v = rot(e - B, m2l_lane_nb(p), tri(p + 1), D.ei, true);
  }
  dst[i] = v;
}

// one thread per direction: kind 0 = M2L offset code, 1 = M2M octant, 2 = L2L octant
template <typename T>
__global__ void k_dir_tables(int p, int kind, int ndir, double ex, double ey, double ez,
                             double *scratch, int scratch_stride, T *out) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ndir) return;
  DirLayout L = dir_layout(p, kind);
  T *o = out + (size_t)k * L.stride;
  double v[3];
  if (kind == 0) {
    int dx = k % 7 - 3, dy = (k / 7) % 7 - 3, dz = k / 49 - 3;
    if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1) {
      for (int i = 0; i < L.stride; ++i) o[i] = (T)0;
      return;
    }
    v[0] = dx * ex; v[1] = dy * ey; v[2] = dz * ez;
  } else {
    double sgn = (kind == 1) ? -0.5 : 0.25;  // parent-child (M2M) / child-parent (L2L)
    v[0] = sgn * ((k & 1) ? 1. : -1.) * ex;
    v[1] = sgn * ((k & 2) ? 1. : -1.) * ey;
    v[2] = sgn * ((k & 4) ? 1. : -1.) * ez;
  }
  double cost = 1.;
  if (v[2] < 0.) { cost = -1.; v[0] = -v[0]; v[1] = -v[1]; v[2] = -v[2]; }
  double rho2 = v[0] * v[0] + v[1] * v[1];
  double r = sqrt(rho2 + v[2] * v[2]);
  double theta = acos(v[2] / r);
  double phi = rho2 > 0. ? atan2(v[1], v[0]) : 0.;
  int Lmax = L.Lf > L.Li ? L.Lf : L.Li;
  double *w = scratch + (size_t)k * scratch_stride;
  double *wm = w + wig_size(Lmax);
  double *eo = wm + wig_size(Lmax);
  gen_wigner_d(Lmax, theta, w);
  gen_wigner_d(Lmax, -theta, wm);
  // M2L blocks go in planes of the source order m: plane m holds, for every
  // output coefficient c = (l, m') in tri order, the (E, O) pair that
  // multiplies source (l, m) (zero when m > l), so the lanes of a warp, one
  // output coefficient each, read consecutive words at every step m
  auto put_cm = [&](int Lb, int base) {
    const int nc = tri(Lb);
    for (int l = 0; l < Lb; ++l)
      for (int mp = 0; mp <= l; ++mp)
        for (int m = 0; m <= l; ++m) {
          int src = sq_off(l) + mp * (l + 1) + m;
          int dst = m2l_plane_off(nc, m) + tri(l, mp) - tri(m);
          o[base + 2 * dst] = (T)eo[src];
          o[base + 2 * dst + 1] = (T)eo[sq_size(Lb) + src];
        }
  };
  wigner_to_eo(L.Lf, w, eo, eo + sq_size(L.Lf));
  if (kind == 0)
    put_cm(L.Lf, L.ef);
  else
    for (int i = 0; i < 2 * sq_size(L.Lf); ++i) o[L.ef + i] = (T)eo[i];
  wigner_to_eo(L.Li, wm, eo, eo + sq_size(L.Li));
  if (kind == 0)
    put_cm(L.Li, L.ei);
  else
    for (int i = 0; i < 2 * sq_size(L.Li); ++i) o[L.ei + i] = (T)eo[i];
  for (int m = 0; m <= p; ++m) {
    o[L.ph + 2 * m] = (T)cos(m * phi);
    o[L.ph + 2 * m + 1] = (T)sin(m * phi);
  }
  if (kind == 0) {
    // rp[k] = cost^{k-1} r^-k (aran/aransphericalseriesd-translate.c:632-650)
    double inv = 1. / r, pw = 1.;
    for (int i = 0; i < L.nrp; ++i) {
      double val = pw;
      if (i % 2 == 0) val *= cost;
      o[L.rp + i] = (T)val;
      pw *= inv;
    }
  } else {
    double base = (kind == 1 ? -cost : cost) * r, pw = 1.;
    for (int i = 0; i < L.nrp; ++i) {
      o[L.rp + i] = (T)pw;
      pw *= base;
    }
  }
}

template <typename T>
void build_tables_t(AranGpuSolver3d *s, OpTables<T> &tb, cudaStream_t st) {
  int p = s->cfg.order;
  tb.p = p;
  tb.rec.reserve(2 * tri(p + 1));
  tb.p2mf.reserve(p + 1);
  tb.vt.reserve(tri(p + 1) * p);
  tb.vm.reserve(tri(p) * p + 1);
  tb.vl.reserve(tri(p + 1) * (p + 1));
  tb.gz.reserve(tri(p) + 1);
  tb.gm.reserve(p * p + 1);
  tb.lm.reserve(2 * tri(p + 1));
  int La = 2 * p + 2;
  DBuf<double> scratch;
  size_t sc1 = tri(p + 2) + tri(La + 1) + 2 * tri(p + 2) + tri(p + 1) + (p + 1) * (p + 1) + 16;
  int Lmax = p + 1;
  int dstride = 2 * wig_size(Lmax) + 4 * sq_size(Lmax) + 16;
  size_t sc2 = (size_t)343 * dstride;
  scratch.reserve(sc1 > sc2 ? sc1 : sc2);
  k_scalar_tables<T><<<1, 1, 0, st>>>(p, scratch.ptr, tb.rec.ptr, tb.p2mf.ptr, tb.vt.ptr,
                                      tb.vm.ptr, tb.vl.ptr, tb.gz.ptr, tb.gm.ptr, tb.lm.ptr);
  ACHECK(cudaGetLastError());
  ACHECK(cudaStreamSynchronize(st));
  double ext = s->scale_e;
  double ex = (s->cfg.ub[0] - s->cfg.lb[0]) / ext, ey = (s->cfg.ub[1] - s->cfg.lb[1]) / ext,
         ez = (s->cfg.ub[2] - s->cfg.lb[2]) / ext;
  for (int kind = 0; kind < 3; ++kind) {
    DirLayout L = dir_layout(p, kind);
    int ndir = kind == 0 ? 343 : 8;
    DBuf<T> &dst = kind == 0 ? tb.dir_m2l : (kind == 1 ? tb.dir_m2m : tb.dir_l2l);
    (kind == 0 ? tb.stride_m2l : (kind == 1 ? tb.stride_m2m : tb.stride_l2l)) = L.stride;
    dst.reserve((size_t)ndir * L.stride);
    k_dir_tables<T><<<ceil_div(ndir, 64), 64, 0, st>>>(p, kind, ndir, ex, ey, ez, scratch.ptr,
                                                        dstride, dst.ptr);
    ACHECK(cudaGetLastError());
    if (kind == 0) {
      const int64_t ne = (int64_t)ndir * tri(p + 1) * p;
      k_m2l_vertical<T><<<ceil_div(ne, 256), 256, 0, st>>>(p, ndir, L.stride, L.rp, L.vv,
                                                            tb.vt.ptr, dst.ptr);
      ACHECK(cudaGetLastError());
      if (sizeof(T) == 4 && m2l_lane_order(p)) {
        const int64_t nl = (int64_t)ndir * m2l_lane_stride(p);
        tb.dir_lanes.reserve(nl);
        k_m2l_lane_tables<<<ceil_div(nl, 256), 256, 0, st>>>(
            p, ndir, reinterpret_cast<const float *>(dst.ptr), L,
            reinterpret_cast<float *>(tb.dir_lanes.ptr));
        ACHECK(cudaGetLastError());
      }
    }
    ACHECK(cudaStreamSynchronize(st));
  }
  if constexpr (sizeof(T) == 4) {
    build_oct_lane_tables(tb, st);
    ACHECK(cudaStreamSynchronize(st));
  }
  scratch.release();
}

}  // namespace

int dir_offset(int p, int kind, int what) {
  DirLayout L = dir_layout(p, kind);
  switch (what) {
    case 0: return L.ef;
    case 1: return L.of;
    case 2: return L.ei;
    case 3: return L.oi;
    case 4: return L.ph;
    case 5: return L.rp;
    case 7: return L.vv;
    default: return L.stride;
  }
}

void build_tables(AranGpuSolver3d *s) {
  if (s->cfg.precision == ARAN_PRECISION_MIXED) build_tables_t<float>(s, s->t32, s->s0);
  else build_tables_t<double>(s, s->t64, s->s0);
}

void build_tables_fp64(AranGpuSolver3d *s) {
  if (s->t64.p != s->cfg.order) build_tables_t<double>(s, s->t64, s->s0);
}

}  // namespace aran
