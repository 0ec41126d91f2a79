// semifar.cu -- the semifar interactions of aran/aransolver3d.c:357-396:
// a coarse leaf A against a deeper node D that does not touch it (and holds
// more points than the threshold) exchanges P2L and M2P instead of P2P.
//
//   P2L  every point x of A: L_l^m(D) += q 4pi/(2l+1) r^{-l-1} conj Y_l^m
//        (aran_development3d_p2l, arandevelopment3d.c:227-277), before L2L;
//   M2P  every point x of A takes D's multipole: potential
//        sum_l r^{-l-1} (M_l^0 Y_l^0 + 2 Re sum_m M_l^m Y_l^m) and its
//        gradient in spherical components (aran_spherical_seriesd_gradient_
//        evaluate, aransphericalseriesd.c:419-546, as used by
//        aran_development3d_m2pv), after L2P.
//
// One warp per pair (P2L) or per leaf (M2P); lane m walks the column m of
// the normalised Legendre functions N_l^m P_l^m and N_l^m P_l^m / sin(theta)
// upward in l, so a point costs O(p^2) with O(1) state per lane.  FP64
// throughout; the expansions are read and written in the solver's scaled
// storage (multipole / h^l, local * h^l with h the node size).
#include "internal.cuh"

namespace aran {
namespace {

constexpr double kFourPi = 12.566370614359172953850573533118;

struct Sph {
  double r, ct, st, cp, sp;
};

__device__ __forceinline__ Sph to_sph(double x, double y, double z) {
  Sph s;
  double rho2 = x * x + y * y, rho = sqrt(rho2);
  s.r = sqrt(rho2 + z * z);
  s.ct = s.r > 0. ? z / s.r : 1.;
  s.st = s.r > 0. ? rho / s.r : 0.;
  s.cp = rho > 0. ? x / rho : 1.;
  s.sp = rho > 0. ? y / rho : 0.;
  return s;
}

// N_m^m P_m^m / sin^m(theta) = (-1)^m sqrt((2m+1)/(4pi) prod_{k<=m} (2k-1)/(2k))
__device__ __forceinline__ double diag_coef(int m) {
  double v = (2. * m + 1.) / kFourPi;
  for (int k = 1; k <= m; ++k) v *= (2. * k - 1.) / (2. * k);
  v = sqrt(v);
  return (m & 1) ? -v : v;
}

__device__ __forceinline__ double ipow(double x, int e) {
  double r = 1.;
  for (int k = 0; k < e; ++k) r *= x;
  return r;
}

__device__ __forceinline__ void cpow_m(double c, double s, int m, double &er, double &ei) {
  er = 1.;
  ei = 0.;
  for (int k = 0; k < m; ++k) {
    double t = er * c - ei * s;
    ei = er * s + ei * c;
    er = t;
  }
}

__device__ __forceinline__ double wsum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// P2L, one warp per semifar pair; the pair's contribution is summed in
// shared memory (lane m owns the column m) and added to D's local.
template <typename T>
__global__ void k_semifar_p2l(int npairs, const int *__restrict__ semi_leaf,
                              const int *__restrict__ semi_node, const int *__restrict__ leaf_node,
                              const int *__restrict__ begin, const int *__restrict__ end,
                              const uint8_t *__restrict__ depth, const double *__restrict__ center,
                              const double *__restrict__ sx, const double *__restrict__ sy,
                              const double *__restrict__ sz, const double *__restrict__ sq,
                              double scale_e, int p, cplx<T> *__restrict__ loc) {
  extern __shared__ double sbuf[];
  const int nl = tri(p + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int pr = blockIdx.x * (blockDim.x >> 5) + w;
  if (pr >= npairs) return;
  double *acc = sbuf + (size_t)w * 2 * nl;
  for (int c = lane; c < 2 * nl; c += 32) acc[c] = 0.;
  __syncwarp();
  const int D = semi_node[pr], A = leaf_node[semi_leaf[pr]];
  const double h = scale_e * ldexp(1.0, -(int)depth[D]), ih = 1. / h;
  const double cx = center[3 * D], cy = center[3 * D + 1], cz = center[3 * D + 2];
  const int m = lane;
  const double dmm = m <= p ? diag_coef(m) : 0.;
  for (int i = begin[A]; i < end[A]; ++i) {
    Sph s = to_sph((sx[i] - cx) * ih, (sy[i] - cy) * ih, (sz[i] - cz) * ih);
    if (m > p) continue;
    const double q = sq[i] * ih, ir = 1. / s.r;
    double er, ei;
    cpow_m(s.cp, s.sp, m, er, ei);
    double y2 = 0., y1 = dmm * ipow(s.st, m);        // N_l^m P_l^m at l-2, l-1 (= m)
    double rp = ipow(ir, m + 1);                      // r^{-l-1}
    for (int l = m; l <= p; ++l) {
      double y;
      if (l == m) y = y1;
      else if (l == m + 1) y = sqrt(2. * m + 3.) * s.ct * y1;
      else {
        double a = sqrt((4. * l * l - 1.) / ((double)l * l - (double)m * m));
        double b = sqrt(((l - 1.) * (l - 1.) - (double)m * m) / (4. * (l - 1.) * (l - 1.) - 1.));
        y = a * (s.ct * y1 - b * y2);
      }
      if (l > m) {
        y2 = y1;
        y1 = y;
      }
      const double f = q * (kFourPi / (2. * l + 1.)) * rp * y;
      acc[2 * tri(l, m)] += f * er;      // conj(e^{i m phi})
      acc[2 * tri(l, m) + 1] -= f * ei;
      rp *= ir;
    }
  }
  __syncwarp();
  T *dst = reinterpret_cast<T *>(loc + (size_t)D * nl);
  for (int c = lane; c < 2 * nl; c += 32) atomicAdd(dst + c, (T)acc[c]);
}

// M2P, one warp per leaf with semifar nodes: potential (and gradient) of
// every semifar node's multipole at every point of the leaf.
template <typename T, bool FIELD>
__global__ void k_semifar_m2p(int nleaves, const int *__restrict__ semi_off,
                              const int *__restrict__ semi_node, const int *__restrict__ leaf_node,
                              const int *__restrict__ begin, const int *__restrict__ end,
                              const uint8_t *__restrict__ depth, const double *__restrict__ center,
                              const double *__restrict__ sx, const double *__restrict__ sy,
                              const double *__restrict__ sz, double scale_e, int p,
                              const cplx<T> *__restrict__ mult, double *__restrict__ acc_pot,
                              double *__restrict__ acc_fld) {
  extern __shared__ double sbuf[];
  const int nm = tri(p);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int L = blockIdx.x * (blockDim.x >> 5) + w;
  if (L >= nleaves) return;
  const int k0 = semi_off[L], k1 = semi_off[L + 1];
  if (k0 == k1) return;
  double *Mc = sbuf + (size_t)w * 2 * nm;
  const int A = leaf_node[L];
  const int m = lane;
  const double dmm = m < p ? diag_coef(m) : 0.;
  for (int k = k0; k < k1; ++k) {
    const int D = semi_node[k];
    __syncwarp();
    for (int c = lane; c < nm; c += 32) {
      cplx<T> v = mult[(size_t)D * nm + c];
      Mc[2 * c] = (double)v.re;
      Mc[2 * c + 1] = (double)v.im;
    }
    __syncwarp();
    const double h = scale_e * ldexp(1.0, -(int)depth[D]), ih = 1. / h;
    const double cx = center[3 * D], cy = center[3 * D + 1], cz = center[3 * D + 2];
    for (int i = begin[A]; i < end[A]; ++i) {
      Sph s = to_sph((sx[i] - cx) * ih, (sy[i] - cy) * ih, (sz[i] - cz) * ih);
      const double ir = 1. / s.r;
      double er = 0., ei = 0.;
      if (m < p) cpow_m(s.cp, s.sp, m, er, ei);
      const double wm = m == 0 ? 1. : 2.;
      double pot = 0., dr = 0., dt = 0., dp = 0.;
      double y2 = 0., y1 = 0., z2 = 0., z1 = 0.;     // Y and Y / sin(theta) columns
      double rp = ir;                                 // r^{-l-1}
      for (int l = 0; l < p; ++l) {
        double y = 0., z = 0.;
        if (m < p) {
          if (l == m) {
            y = dmm * ipow(s.st, m);
            z = m > 0 ? dmm * ipow(s.st, m - 1) : 0.;
          } else if (l == m + 1) {
            const double a = sqrt(2. * m + 3.) * s.ct;
            y = a * y1;
            z = a * z1;
          } else if (l > m + 1) {
            const double a = sqrt((4. * l * l - 1.) / ((double)l * l - (double)m * m));
            const double b = sqrt(((l - 1.) * (l - 1.) - (double)m * m) / (4. * (l - 1.) * (l - 1.) - 1.));
            y = a * (s.ct * y1 - b * y2);
            z = a * (s.ct * z1 - b * z2);
          }
          if (l >= m) {
            y2 = y1;
            y1 = y;
            z2 = z1;
            z1 = z;
          }
        }
        // h = e^{i m phi} N P, hn = the same at order m + 1 (next lane)
        const double hr = er * y, hi = ei * y;
        const double hnr = __shfl_down_sync(0xffffffffu, hr, 1);
        const double hni = __shfl_down_sync(0xffffffffu, hi, 1);
        if (m <= l && m < p) {
          const double cr = Mc[2 * tri(l, m)], ci = Mc[2 * tri(l, m) + 1];
          const double re_hc = hr * cr - hi * ci;
          pot += rp * wm * re_hc;
          if (FIELD) {
            const double rq = rp * ir;               // r^{-l-2}
            dr -= (l + 1.) * rq * wm * re_hc;
            // (h_{l,m+1} c e^{-i phi}) real part
            const double tr = hnr * cr - hni * ci, ti = hnr * ci + hni * cr;
            const double re_next = tr * s.cp + ti * s.sp;
            if (m >= 1) {
              const double shr = er * z, shi = ei * z;
              const double re_sc = shr * cr - shi * ci, im_sc = shr * ci + shi * cr;
              double t = re_sc * s.ct * m;
              if (m <= l - 1) t += re_next * sqrt((double)(l - m) * (double)(l + m + 1));
              dt += rq * 2. * t;
              dp += rq * (-2.) * im_sc * m;
            } else if (l >= 1) {
              dt += rq * re_next * sqrt((double)l * (double)(l + 1));
            }
          }
        }
        rp *= ir;
      }
      pot = wsum(pot);
      if (FIELD) {
        dr = wsum(dr);
        dt = wsum(dt);
        dp = wsum(dp);
      }
      if (lane == 0) {
        acc_pot[i] += pot * ih;
        if (FIELD) {
          const double g2 = ih * ih;
          acc_fld[3 * (size_t)i] += (s.st * s.cp * dr + s.ct * s.cp * dt - s.sp * dp) * g2;
          acc_fld[3 * (size_t)i + 1] += (s.st * s.sp * dr + s.ct * s.sp * dt + s.cp * dp) * g2;
          acc_fld[3 * (size_t)i + 2] += (s.ct * dr - s.st * dt) * g2;
        }
      }
    }
  }
}

template <typename T>
void p2l_t(AranGpuSolver3d *s, const cplx<T> *, cplx<T> *loc, cudaStream_t st) {
  DevTree &t = s->tree;
  const int p = s->cfg.order, WPB = 4;
  size_t sm = (size_t)WPB * 2 * tri(p + 1) * sizeof(double);
  smem_opt_in(k_semifar_p2l<T>, sm);
  k_semifar_p2l<T><<<ceil_div(t.n_semi, WPB), WPB * 32, sm, st>>>(
      t.n_semi, t.semi_leaf.ptr, t.semi_node.ptr, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
      t.depth.ptr, t.center.ptr, s->sx.ptr, s->sy.ptr, s->sz.ptr, s->sq.ptr, s->scale_e, p, loc);
  ACHECK(cudaGetLastError());
  s->launches++;
}

template <typename T>
void m2p_t(AranGpuSolver3d *s, const cplx<T> *mult, cudaStream_t st) {
  DevTree &t = s->tree;
  const int p = s->cfg.order, WPB = 4;
  size_t sm = (size_t)WPB * 2 * tri(p) * sizeof(double);
  if (s->cfg.field) {
    smem_opt_in(k_semifar_m2p<T, true>, sm);
    k_semifar_m2p<T, true><<<ceil_div(t.nleaves, WPB), WPB * 32, sm, st>>>(
        t.nleaves, t.semi_off.ptr, t.semi_node.ptr, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
        t.depth.ptr, t.center.ptr, s->sx.ptr, s->sy.ptr, s->sz.ptr, s->scale_e, p, mult,
        s->acc_pot.ptr, s->acc_fld.ptr);
  } else {
    smem_opt_in(k_semifar_m2p<T, false>, sm);
    k_semifar_m2p<T, false><<<ceil_div(t.nleaves, WPB), WPB * 32, sm, st>>>(
        t.nleaves, t.semi_off.ptr, t.semi_node.ptr, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
        t.depth.ptr, t.center.ptr, s->sx.ptr, s->sy.ptr, s->sz.ptr, s->scale_e, p, mult,
        s->acc_pot.ptr, s->acc_fld.ptr);
  }
  ACHECK(cudaGetLastError());
  s->launches++;
}

}  // namespace

void launch_semifar_p2l(AranGpuSolver3d *s, cudaStream_t st) {
  if (s->cfg.semifar_threshold <= 0 || s->tree.n_semi == 0) return;
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    p2l_t<float>(s, nullptr, reinterpret_cast<cplx<float> *>(s->loc32.ptr), st);
  else
    p2l_t<double>(s, nullptr, reinterpret_cast<cplx<double> *>(s->loc64.ptr), st);
}

void launch_semifar_m2p(AranGpuSolver3d *s, cudaStream_t st) {
  if (s->cfg.semifar_threshold <= 0 || s->tree.n_semi == 0) return;
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    m2p_t<float>(s, reinterpret_cast<const cplx<float> *>(s->mult32.ptr), st);
  else
    m2p_t<double>(s, reinterpret_cast<const cplx<double> *>(s->mult64.ptr), st);
}

}  // namespace aran
