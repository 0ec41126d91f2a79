// compat2d.cu -- LibAran's 2D public API (aran/aransolver2d.h,
// aran/arandevelopment2d.h, aran/aranlaurentseriesd.h and the
// vsg_prtree2d_new_full tree constructor) on the GPU library.
//
// The Laurent-series containers are host memory with the reference layout
// (degrees posdeg .. -negdeg, aranlaurentseriesd.c:37-43).  Every operator
// that computes (evaluate, translate, to_taylor and the development
// operators built on them) runs as one small launch on the GPU: one thread
// per output term, each repeating the reference's loop for that term in the
// same order (aranlaurentseriesd.c:47-73,311-452; arandevelopment2d.c:167-221).
// aran_solver2d_solve runs the forest solver of solver2d.cu on one system.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "internal.cuh"

#include <aran/aranprofiledb.h>
#include <aran/aransolver2d.h>

struct _AranLaurentSeriesd {
  guint8 posdeg;
  guint8 negdeg;
  gcomplex128 *terms;   // posdeg + negdeg + 1, degree i at posdeg - i
};

struct _VsgPRTree2d {
  VsgVector2d lb, ub;
  guint maxbox;
  gdouble tolerance;
};

struct _AranSolver2d {
  VsgPRTree2d *tree = nullptr;
  AranDevelopment2d *devel = nullptr;
  AranZeroFunc zero = nullptr;
  AranParticle2ParticleFunc2d p2p = nullptr;
  AranParticle2MultipoleFunc2d p2m = nullptr;
  AranMultipole2MultipoleFunc2d m2m = nullptr;
  AranMultipole2LocalFunc2d m2l = nullptr;
  AranLocal2LocalFunc2d l2l = nullptr;
  AranLocal2ParticleFunc2d l2p = nullptr;
  AranParticle2LocalFunc2d p2l = nullptr;
  AranMultipole2ParticleFunc2d m2p = nullptr;
  guint semifar_threshold = 0;
  std::vector<VsgPoint2> points;
  bool layout = false;
  size_t off_pos = 0, off_q = 0, off_acc = 0;
  AranGpuSolver2d *gpu = nullptr;
  AranGpuConfig2d gpu_cfg;
  int64_t stats[11] = {};
  guint depth = 0;
  // virtual leaves, children order, operator costs (< 0: unknown), and
  // whether the last solve ran on exactly the current points
  VsgPRTree2dNFIsleafFunc nf_isleaf = nullptr;
  gpointer nf_isleaf_data = nullptr;
  bool hilbert = false;
  double p2p_time = -1, p2m_time = -1, p2l_time = -1, l2p_time = -1, m2p_time = -1,
         m2m_time = -1, m2l_time = -1, l2l_time = -1;
  bool solved_current = false;
};

namespace aran {
namespace {

const GType kDevelopment2dType = 0x41524432;  // "ARD2"

enum { OP_TRANSLATE = 0, OP_TO_TAYLOR = 1, OP_EVALUATE = 2, OP_P2M = 3, OP_P2L = 4 };

typedef cplx<double> zd;

__device__ __forceinline__ zd zmul2(zd a, zd b) {
  return cmake(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ zd zadd2(zd a, zd b) { return cmake(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ zd zsc(zd a, double s) { return cmake(a.re * s, a.im * s); }
__device__ __forceinline__ zd zrecip(zd a) {
  double r2 = a.re * a.re + a.im * a.im;
  return cmake(a.re / r2, -a.im / r2);
}

// One operator on reference-layout series (index posdeg - degree).
// z: zdst - zsrc (translate / to_taylor), the evaluation point (evaluate) or
// position - centre (p2m / p2l).  q: the charge of p2m / p2l.
__global__ void k_laurent_op(int kind, int sp, int sn, const zd *__restrict__ src, zd z, int dp,
                             int dn, zd *__restrict__ dst, const double *__restrict__ binom,
                             int nb, double q) {
  const int t = threadIdx.x;
  if (kind == OP_EVALUATE) {
    if (t != 0) return;
    zd pos = src[0];
    for (int i = 1; i <= sp; ++i) pos = zadd2(zmul2(pos, z), src[i]);
    zd neg = cmake(0.0, 0.0);
    if (sn != 0) {
      zd invz = zrecip(z);
      neg = src[sp + sn];
      for (int i = sn - 1; i > 0; --i) neg = zadd2(zmul2(neg, invz), src[sp + i]);
      neg = zmul2(neg, invz);
    }
    dst[0] = zadd2(pos, neg);
    return;
  }
  if (kind == OP_P2M) {
    // dst degree -i += q z^{i-1}, i = 1 .. dn - 1
    int i = t + 1;
    if (i >= dn) return;
    zd tmp = cmake(q, 0.0);
    for (int k = 1; k < i; ++k) tmp = zmul2(tmp, z);
    dst[dp + i] = zadd2(dst[dp + i], tmp);
    return;
  }
  if (kind == OP_P2L) {
    // dst degree i += -q z^{-(i+1)}, i = 0 .. dp
    int i = t;
    if (i > dp) return;
    zd inv = zrecip(z);
    zd tmp = cmake(-q, 0.0);
    for (int k = 0; k <= i; ++k) tmp = zmul2(tmp, inv);
    dst[dp - i] = zadd2(dst[dp - i], tmp);
    return;
  }
  // translate / to_taylor: non-negative part (aran_taylor_translate)
  if (t <= dp) {
    int i = t;
    zd sum = src[0];
    for (int j = sp - 1; j >= i; --j) sum = zadd2(zmul2(sum, z), zsc(src[sp - j], binom[j * nb + i]));
    dst[dp - i] = zadd2(dst[dp - i], sum);
  }
  if (sn <= 0) return;
  if (kind == OP_TRANSLATE) {
    int i = t + 1;
    if (i > dn) return;
    zd mz = cmake(-z.re, -z.im);
    int jm = i < sn ? i : sn;
    zd sum = cmake(0.0, 0.0);
    for (int j = 1; j < jm; ++j) sum = zmul2(zadd2(sum, zsc(src[sp + j], binom[(i - 1) * nb + j - 1])), mz);
    dst[dp + i] = zadd2(dst[dp + i], zadd2(sum, src[sp + jm]));
  } else {
    int i = t;
    if (i > dp) return;
    zd inv = zrecip(z);
    zd minv = cmake(-inv.re, -inv.im);
    zd pw = cmake(1.0, 0.0);
    for (int k = 0; k < i; ++k) pw = zmul2(pw, minv);
    zd sum = cmake(0.0, 0.0);
    for (int j = sn - 1; j >= 1; --j)
      sum = zmul2(zadd2(sum, zsc(src[sp + j], binom[(i + j - 1) * nb + j - 1])), inv);
    dst[dp - i] = zadd2(dst[dp - i], zmul2(sum, pw));
  }
}

// process-wide launch context for the per-call operators (serialised)
struct OpContext {
  std::mutex mu;
  int device = -1;
  cudaStream_t st = nullptr;
  DBuf<zd> buf;
  DBuf<double> binom;
  int nb = 0;
};

OpContext &op_ctx() {
  static OpContext *c = new OpContext();  // lives until exit
  return *c;
}

// Runs one operator; returns ARAN_OK and updates dst (or writes the value
// to *value for evaluate), or an error code with dst untouched.
int laurent_op(int kind, int sp, int sn, const gcomplex128 *src, std::complex<double> z, int dp,
               int dn, gcomplex128 *dst, double q, gcomplex128 *value) {
  OpContext &c = op_ctx();
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
    int need = std::max(std::max(sp, dn), dp + sn) + 2;
    if (need > c.nb) {
      int nb = std::max(need, 64);
      std::vector<double> b((size_t)nb * nb, 0.0);
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j <= i; ++j)
          b[(size_t)i * nb + j] = (j == 0 || j == i) ? 1.0 : b[(size_t)(i - 1) * nb + j] + b[(size_t)(i - 1) * nb + j - 1];
      c.binom.reserve(b.size());
      ACHECK(cudaMemcpyAsync(c.binom.ptr, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice, c.st));
      ACHECK(cudaStreamSynchronize(c.st));
      c.nb = nb;
    }
    const int ns = src ? sp + sn + 1 : 0;
    const int nd = kind == OP_EVALUATE ? 1 : dp + dn + 1;
    c.buf.reserve(ns + nd);
    zd *dsrc = c.buf.ptr, *ddst = c.buf.ptr + ns;
    if (ns) ACHECK(cudaMemcpyAsync(dsrc, src, ns * sizeof(zd), cudaMemcpyHostToDevice, c.st));
    if (kind != OP_EVALUATE) ACHECK(cudaMemcpyAsync(ddst, dst, nd * sizeof(zd), cudaMemcpyHostToDevice, c.st));
    int threads = std::max(dp + 1, dn + 1);
    threads = ((threads + 31) / 32) * 32;
    zd zz = cmake(z.real(), z.imag());
    k_laurent_op<<<1, threads, 0, c.st>>>(kind, sp, sn, dsrc, zz, dp, dn, ddst, c.binom.ptr, c.nb, q);
    ACHECK(cudaGetLastError());
    if (kind == OP_EVALUATE) {
      zd v;
      ACHECK(cudaMemcpyAsync(&v, ddst, sizeof(zd), cudaMemcpyDeviceToHost, c.st));
      ACHECK(cudaStreamSynchronize(c.st));
      *value = gcomplex128(v.re, v.im);
    } else {
      std::vector<gcomplex128> out(nd);
      ACHECK(cudaMemcpyAsync(out.data(), ddst, nd * sizeof(zd), cudaMemcpyDeviceToHost, c.st));
      ACHECK(cudaStreamSynchronize(c.st));
      std::memcpy(dst, out.data(), nd * sizeof(gcomplex128));
    }
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  return ARAN_OK;
}

std::complex<double> cz(const VsgVector2d &v) { return std::complex<double>(v.x, v.y); }

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" {

// ---- libvsg 2D tree description ----
VsgPRTree2d *vsg_prtree2d_new_full(const VsgVector2d *lbound, const VsgVector2d *ubound,
                                   VsgPoint2dLocFunc, VsgPoint2dDistFunc, VsgRegion2dLocFunc,
                                   guint maxbox) {
  if (!lbound || !ubound) return nullptr;
  VsgPRTree2d *t = new VsgPRTree2d();
  t->lb = *lbound;
  t->ub = *ubound;
  t->maxbox = maxbox > 0 ? maxbox : 1;
  t->tolerance = 0.;
  return t;
}

void vsg_prtree2d_free(VsgPRTree2d *prtree) { delete prtree; }

gint vsg_vector2d_vector2d_locfunc(const VsgVector2d *candidate, const VsgVector2d *center) {
  return (candidate->x > center->x ? 1 : 0) | (candidate->y > center->y ? 2 : 0);
}

gdouble vsg_vector2d_dist(const VsgVector2d *one, const VsgVector2d *other) {
  double dx = one->x - other->x, dy = one->y - other->y;
  return sqrt(dx * dx + dy * dy);
}

// ---- Laurent series (aran/aranlaurentseriesd.c:98-280) ----
AranLaurentSeriesd *aran_laurent_seriesd_new(guint8 posdeg, guint8 negdeg) {
  AranLaurentSeriesd *s = (AranLaurentSeriesd *)std::calloc(1, sizeof(AranLaurentSeriesd));
  s->posdeg = posdeg;
  s->negdeg = negdeg;
  s->terms = (gcomplex128 *)std::calloc((size_t)posdeg + negdeg + 1, sizeof(gcomplex128));
  return s;
}

void aran_laurent_seriesd_free(AranLaurentSeriesd *als) {
  if (!als) return;
  std::free(als->terms);
  std::free(als);
}

void aran_laurent_seriesd_copy(const AranLaurentSeriesd *src, AranLaurentSeriesd *dst) {
  if (!src || !dst) return;
  // term by term over the common degrees (aranlaurentseriesd.c:150-170)
  for (int i = -(int)dst->negdeg; i <= (int)dst->posdeg; ++i) {
    gcomplex128 v = (i >= -(int)src->negdeg && i <= (int)src->posdeg) ? src->terms[src->posdeg - i]
                                                                       : gcomplex128(0., 0.);
    dst->terms[dst->posdeg - i] = v;
  }
}

AranLaurentSeriesd *aran_laurent_seriesd_clone(AranLaurentSeriesd *src) {
  if (!src) return nullptr;
  AranLaurentSeriesd *d = aran_laurent_seriesd_new(src->posdeg, src->negdeg);
  aran_laurent_seriesd_copy(src, d);
  return d;
}

gcomplex128 *aran_laurent_seriesd_get_term(AranLaurentSeriesd *als, gint i) {
  if (!als || i < -(int)als->negdeg || i > (int)als->posdeg) return nullptr;
  return als->terms + (als->posdeg - i);
}

guint8 aran_laurent_seriesd_get_posdeg(AranLaurentSeriesd *als) { return als ? als->posdeg : 0; }
guint8 aran_laurent_seriesd_get_negdeg(AranLaurentSeriesd *als) { return als ? als->negdeg : 0; }

void aran_laurent_seriesd_set_zero(AranLaurentSeriesd *als) {
  if (als) std::memset(als->terms, 0, ((size_t)als->posdeg + als->negdeg + 1) * sizeof(gcomplex128));
}

void aran_laurent_seriesd_add(AranLaurentSeriesd *one, AranLaurentSeriesd *other,
                              AranLaurentSeriesd *result) {
  // all three of the same degrees (aranlaurentseriesd.c:262-267)
  if (!one || !other || !result || one->posdeg != result->posdeg ||
      other->posdeg != result->posdeg || one->negdeg != result->negdeg ||
      other->negdeg != result->negdeg)
    return;
  for (int k = 0; k <= (int)result->posdeg + result->negdeg; ++k)
    result->terms[k] = one->terms[k] + other->terms[k];
}

void aran_laurent_seriesd_write(AranLaurentSeriesd *als, FILE *file) {
  if (!als || !file) return;
  std::fprintf(file, "[");
  for (int i = -(int)als->negdeg; i <= (int)als->posdeg; ++i) {
    gcomplex128 t = als->terms[als->posdeg - i];
    std::fprintf(file, i < als->posdeg ? "%d:(%e,%e), " : "%d:(%e,%e)] ", i, t.real(), t.imag());
  }
}

gcomplex128 aran_laurent_seriesd_evaluate(AranLaurentSeriesd *als, gcomplex128 z) {
  gcomplex128 v(0., 0.);
  if (!als) return v;
  laurent_op(OP_EVALUATE, als->posdeg, als->negdeg, als->terms, z, 0, 0, nullptr, 0., &v);
  return v;
}

void aran_laurent_seriesd_translate(AranLaurentSeriesd *src, gcomplex128 zsrc,
                                    AranLaurentSeriesd *dst, gcomplex128 zdst) {
  if (!src || !dst) return;
  laurent_op(OP_TRANSLATE, src->posdeg, src->negdeg, src->terms, zdst - zsrc, dst->posdeg,
             dst->negdeg, dst->terms, 0., nullptr);
}

void aran_laurent_seriesd_to_taylor(AranLaurentSeriesd *src, gcomplex128 zsrc,
                                    AranLaurentSeriesd *dst, gcomplex128 zdst) {
  if (!src || !dst) return;
  laurent_op(OP_TO_TAYLOR, src->posdeg, src->negdeg, src->terms, zdst - zsrc, dst->posdeg,
             dst->negdeg, dst->terms, 0., nullptr);
}

// ---- 2D development (aran/arandevelopment2d.c:64-346) ----
GType aran_development2d_get_type(void) { return kDevelopment2dType; }

AranDevelopment2d *aran_development2d_new(guint8 posdeg, guint8 negdeg) {
  AranDevelopment2d *d = (AranDevelopment2d *)std::malloc(sizeof(AranDevelopment2d));
  d->multipole = aran_laurent_seriesd_new(posdeg, negdeg);
  d->local = aran_laurent_seriesd_new(posdeg > negdeg ? posdeg : negdeg, 0);
  return d;
}

void aran_development2d_free(AranDevelopment2d *ad) {
  if (!ad) return;
  aran_laurent_seriesd_free(ad->multipole);
  aran_laurent_seriesd_free(ad->local);
  std::free(ad);
}

void aran_development2d_copy(const AranDevelopment2d *src, AranDevelopment2d *dst) {
  if (!src || !dst) return;
  aran_laurent_seriesd_copy(src->multipole, dst->multipole);
  aran_laurent_seriesd_copy(src->local, dst->local);
}

AranDevelopment2d *aran_development2d_clone(AranDevelopment2d *src) {
  if (!src) return nullptr;
  AranDevelopment2d *d = aran_development2d_new(src->multipole->posdeg, src->multipole->negdeg);
  aran_development2d_copy(src, d);
  return d;
}

void aran_development2d_set_zero(AranDevelopment2d *ad) {
  if (!ad) return;
  aran_laurent_seriesd_set_zero(ad->multipole);
  aran_laurent_seriesd_set_zero(ad->local);
}

void aran_development2d_write(AranDevelopment2d *ad, FILE *file) {
  if (!ad || !file) return;
  std::fprintf(file, "{multipole= ");
  aran_laurent_seriesd_write(ad->multipole, file);
  std::fprintf(file, ", local= ");
  aran_laurent_seriesd_write(ad->local, file);
  std::fprintf(file, "}");
}

void aran_development2d_p2m(VsgVector2d *position, gdouble charge,
                            const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst) {
  if (!position || !dst_node || !dst) return;
  AranLaurentSeriesd *m = dst->multipole;
  laurent_op(OP_P2M, 0, 0, nullptr, cz(*position) - cz(dst_node->center), m->posdeg, m->negdeg,
             m->terms, charge, nullptr);
}

void aran_development2d_p2l(VsgVector2d *position, gdouble charge,
                            const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst) {
  if (!position || !dst_node || !dst) return;
  AranLaurentSeriesd *l = dst->local;
  laurent_op(OP_P2L, 0, 0, nullptr, cz(*position) - cz(dst_node->center), l->posdeg, l->negdeg,
             l->terms, charge, nullptr);
}

void aran_development2d_m2m(const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                            const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst) {
  if (!src_node || !src || !dst_node || !dst) return;
  aran_laurent_seriesd_translate(src->multipole, cz(src_node->center), dst->multipole,
                                 cz(dst_node->center));
}

void aran_development2d_m2l(const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                            const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst) {
  if (!src_node || !src || !dst_node || !dst) return;
  aran_laurent_seriesd_to_taylor(src->multipole, cz(src_node->center), dst->local,
                                 cz(dst_node->center));
}

void aran_development2d_l2l(const VsgPRTree2dNodeInfo *src_node, AranDevelopment2d *src,
                            const VsgPRTree2dNodeInfo *dst_node, AranDevelopment2d *dst) {
  if (!src_node || !src || !dst_node || !dst) return;
  aran_laurent_seriesd_translate(src->local, cz(src_node->center), dst->local,
                                 cz(dst_node->center));
}

gcomplex128 aran_development2d_multipole_evaluate(const VsgPRTree2dNodeInfo *devel_node,
                                                  AranDevelopment2d *devel, const VsgVector2d *pos) {
  if (!devel_node || !devel || !pos) return gcomplex128(0., 0.);
  return aran_laurent_seriesd_evaluate(devel->multipole, cz(*pos) - cz(devel_node->center));
}

gcomplex128 aran_development2d_local_evaluate(const VsgPRTree2dNodeInfo *devel_node,
                                              AranDevelopment2d *devel, const VsgVector2d *pos) {
  if (!devel_node || !devel || !pos) return gcomplex128(0., 0.);
  return aran_laurent_seriesd_evaluate(devel->local, cz(*pos) - cz(devel_node->center));
}

gcomplex128 aran_development2d_m2p(const VsgPRTree2dNodeInfo *devel_node, AranDevelopment2d *devel,
                                   const VsgVector2d *pos) {
  return aran_development2d_multipole_evaluate(devel_node, devel, pos);
}

gcomplex128 aran_development2d_l2p(const VsgPRTree2dNodeInfo *devel_node, AranDevelopment2d *devel,
                                   const VsgVector2d *pos) {
  return aran_development2d_local_evaluate(devel_node, devel, pos);
}

// ---- 2D solver (aran/aransolver2d.c) ----
namespace {

int leaf_pred2(const AranGpuNodeView *v, void *data) {
  AranSolver2d *s = (AranSolver2d *)data;
  VsgPRTree2dNodeInfo info;
  std::memset(&info, 0, sizeof(info));
  info.center = {v->center[0], v->center[1]};
  info.lbound = {v->lbound[0], v->lbound[1]};
  info.ubound = {v->ubound[0], v->ubound[1]};
  info.point_count = (guint)v->point_count;
  info.depth = (guint)v->depth;
  return s->nf_isleaf(&info, s->nf_isleaf_data) ? 1 : 0;
}

// the GPU solver of the solver's order and leaf capacity, with its
// virtual-leaf predicate
int gpu_solver2(AranSolver2d *solver) {
  AranGpuConfig2d cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.maxbox = (int)solver->tree->maxbox;
  cfg.order = solver->devel->multipole->negdeg;
  cfg.max_depth = 0;
  if (!solver->gpu || std::memcmp(&cfg, &solver->gpu_cfg, sizeof(cfg)) != 0) {
    if (solver->gpu) aran_gpu_solver2d_destroy(solver->gpu);
    solver->gpu = nullptr;
    solver->solved_current = false;
    int rc = aran_gpu_solver2d_create(&cfg, &solver->gpu);
    if (rc != ARAN_OK) return rc;
    solver->gpu_cfg = cfg;
  }
  return aran_gpu_solver2d_set_leaf_predicate(solver->gpu, solver->nf_isleaf ? leaf_pred2 : nullptr,
                                              solver);
}

void gather2(AranSolver2d *solver, size_t off_pos, size_t off_q, std::vector<double> &xy,
             std::vector<double> &q) {
  const size_t n = solver->points.size();
  xy.resize(2 * n);
  q.resize(n);
  for (size_t i = 0; i < n; ++i) {
    const char *pt = (const char *)solver->points[i];
    const VsgVector2d *v = (const VsgVector2d *)(pt + off_pos);
    xy[2 * i] = v->x;
    xy[2 * i + 1] = v->y;
    q[i] = off_q == (size_t)-1 ? 0.0 : *(const double *)(pt + off_q);
  }
}

// Hilbert index of cell (x, y) of a 2^bits grid (J. Skilling's transpose
// algorithm, AIP Conf. Proc. 707 (2004) 381, for two axes)
uint64_t hilbert2(uint32_t x, uint32_t y, int bits) {
  uint32_t X[2] = {x, y};
  const uint32_t M = 1u << (bits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 2; ++i) {
      if (X[i] & Q) X[0] ^= P;
      else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  X[1] ^= X[0];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[1] & Q) t ^= Q - 1;
  X[0] ^= t;
  X[1] ^= t;
  uint64_t h = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < 2; ++i) h = (h << 1) | ((X[i] >> b) & 1u);
  return h;
}

}  // namespace

AranSolver2d *aran_solver2d_new(VsgPRTree2d *prtree, GType devel_type, gpointer devel,
                                AranZeroFunc zero) {
  AranSolver2d *s = new AranSolver2d();
  if (!prtree) {
    VsgVector2d lb = {-1., -1.}, ub = {1., 1.};
    prtree = vsg_prtree2d_new_full(&lb, &ub, nullptr, nullptr, nullptr, 1);
  }
  s->tree = prtree;
  aran_solver2d_set_development(s, devel_type, devel, zero);
  return s;
}

void aran_solver2d_free(AranSolver2d *solver) {
  if (!solver) return;
  if (solver->gpu) aran_gpu_solver2d_destroy(solver->gpu);
  vsg_prtree2d_free(solver->tree);
  aran_development2d_free(solver->devel);
  delete solver;
}

void aran_solver2d_set_development(AranSolver2d *solver, GType devel_type, gpointer devel,
                                   AranZeroFunc zero) {
  if (!solver) return;
  if (devel && devel_type != kDevelopment2dType) {
    set_error("aran_solver2d_set_development: only ARAN_TYPE_DEVELOPMENT2D is supported");
    return;
  }
  if (solver->devel && solver->devel != devel) aran_development2d_free(solver->devel);
  solver->devel = (AranDevelopment2d *)devel;
  solver->zero = zero;
}

void aran_solver2d_set_functions_full(AranSolver2d *solver, AranParticle2ParticleFunc2d p2p,
                                      AranParticle2MultipoleFunc2d p2m,
                                      AranMultipole2MultipoleFunc2d m2m,
                                      AranMultipole2LocalFunc2d m2l, AranLocal2LocalFunc2d l2l,
                                      AranLocal2ParticleFunc2d l2p, AranParticle2LocalFunc2d p2l,
                                      AranMultipole2ParticleFunc2d m2p, guint semifar_threshold) {
  if (!solver) return;
  solver->p2p = p2p;
  solver->p2m = p2m;
  solver->m2m = m2m;
  solver->m2l = m2l;
  solver->l2l = l2l;
  solver->l2p = l2p;
  solver->p2l = p2l;
  solver->m2p = m2p;
  solver->semifar_threshold = semifar_threshold;
}

void aran_solver2d_set_functions(AranSolver2d *solver, AranParticle2ParticleFunc2d p2p,
                                 AranParticle2MultipoleFunc2d p2m,
                                 AranMultipole2MultipoleFunc2d m2m, AranMultipole2LocalFunc2d m2l,
                                 AranLocal2LocalFunc2d l2l, AranLocal2ParticleFunc2d l2p) {
  aran_solver2d_set_functions_full(solver, p2p, p2m, m2m, m2l, l2l, l2p, nullptr, nullptr, 0);
}

void aran_solver2d_reinit_stats(AranSolver2d *solver) {
  if (solver) std::memset(solver->stats, 0, sizeof(solver->stats));
}

void aran_solver2d_get_stats(AranSolver2d *solver, glong *zero_count, glong *p2p_count,
                             glong *p2m_count, glong *m2m_count, glong *m2l_count,
                             glong *l2l_count, glong *l2p_count, glong *p2l_count,
                             glong *m2p_count, glong *p2p_remote_count,
                             glong *m2l_remote_count) {
  if (!solver) return;
  glong *out[11] = {zero_count, p2p_count, p2m_count, m2m_count, m2l_count, l2l_count,
                    l2p_count, p2l_count, m2p_count, p2p_remote_count, m2l_remote_count};
  for (int i = 0; i < 11; ++i)
    if (out[i]) *out[i] = (glong)solver->stats[i];
}

gdouble aran_solver2d_get_tolerance(AranSolver2d *solver) {
  return solver ? solver->tree->tolerance : -1.;
}

void aran_solver2d_set_tolerance(AranSolver2d *solver, gdouble tolerance) {
  if (solver) solver->tree->tolerance = tolerance;
}

void aran_solver2d_get_bounds(AranSolver2d *solver, VsgVector2d *lbound, VsgVector2d *ubound) {
  if (!solver) return;
  if (lbound) *lbound = solver->tree->lb;
  if (ubound) *ubound = solver->tree->ub;
}

guint aran_solver2d_depth(const AranSolver2d *solver) { return solver ? solver->depth : 0; }

guint aran_solver2d_point_count(const AranSolver2d *solver) {
  return solver ? (guint)solver->points.size() : 0;
}

void aran_solver2d_insert_point(AranSolver2d *solver, VsgPoint2 point) {
  if (!solver || !point) return;
  solver->points.push_back(point);
  solver->solved_current = false;
}

gboolean aran_solver2d_insert_point_local(AranSolver2d *solver, VsgPoint2 point) {
  if (!solver || !point) return FALSE;
  aran_solver2d_insert_point(solver, point);
  return TRUE;
}

gboolean aran_solver2d_remove_point(AranSolver2d *solver, VsgPoint2 point) {
  if (!solver) return FALSE;
  for (size_t i = 0; i < solver->points.size(); ++i)
    if (solver->points[i] == point) {
      solver->points.erase(solver->points.begin() + i);
      solver->solved_current = false;
      return TRUE;
    }
  return FALSE;
}

void aran_solver2d_foreach_point(AranSolver2d *solver, GFunc func, gpointer user_data) {
  if (!solver || !func) return;
  for (VsgPoint2 p : solver->points) func(p, user_data);
}

void aran_solver2d_set_cauchy_layout(AranSolver2d *solver, size_t pos_offset,
                                     size_t density_offset, size_t accum_offset) {
  if (!solver) return;
  solver->layout = true;
  solver->off_pos = pos_offset;
  solver->off_q = density_offset;
  solver->off_acc = accum_offset;
}

int aran_solver2d_solve_try(AranSolver2d *solver) {
  if (!solver) return fail(ARAN_ERR_INVALID, "aran_solver2d_solve: solver is NULL");
  if (!solver->layout)
    return fail(ARAN_ERR_INVALID, "aran_solver2d_solve: call aran_solver2d_set_cauchy_layout first");
  if (!solver->devel || solver->devel->multipole->negdeg < 1)
    return fail(ARAN_ERR_INVALID, "aran_solver2d_solve: no development (aran_development2d_new (0, p))");
  if (solver->devel->multipole->posdeg != 0)
    return fail(ARAN_ERR_UNSUPPORTED,
                "aran_solver2d_solve: the GPU path takes developments aran_development2d_new (0, p)");
  if (!solver->p2p || !solver->p2m || !solver->l2p)
    return fail(ARAN_ERR_INVALID, "aran_solver2d_solve: the GPU path needs p2p, p2m and l2p");
  if ((void *)solver->m2m != (void *)&aran_development2d_m2m ||
      (void *)solver->m2l != (void *)&aran_development2d_m2l ||
      (void *)solver->l2l != (void *)&aran_development2d_l2l)
    return fail(ARAN_ERR_UNSUPPORTED,
                "aran_solver2d_solve: m2m/m2l/l2l must be aran_development2d_m2m/m2l/l2l");
  const int64_t n = (int64_t)solver->points.size();
  if (n == 0) return ARAN_OK;
  int rc = gpu_solver2(solver);
  if (rc != ARAN_OK) return rc;
  std::vector<double> xy, q, acc(2 * n);
  gather2(solver, solver->off_pos, solver->off_q, xy, q);
  int64_t offs[2] = {0, n};
  double box[4] = {solver->tree->lb.x, solver->tree->lb.y, solver->tree->ub.x, solver->tree->ub.y};
  rc = aran_gpu_solver2d_solve(solver->gpu, 1, offs, box, xy.data(), q.data(), acc.data(),
                               ARAN_MEM_HOST);
  if (rc != ARAN_OK) return rc;
  solver->solved_current = true;
  for (int64_t i = 0; i < n; ++i) {
    double *a = (double *)((char *)solver->points[i] + solver->off_acc);  // gcomplex128: re, im
    a[0] += acc[2 * i];
    a[1] += acc[2 * i + 1];
  }
  int64_t st[11];
  if (aran_gpu_solver2d_get_stats(solver->gpu, st) == ARAN_OK)
    for (int k = 0; k < 11; ++k) solver->stats[k] += st[k];
  int64_t info[5];
  if (aran_gpu_solver2d_tree_info(solver->gpu, info) == ARAN_OK) solver->depth = (guint)info[4];
  return ARAN_OK;
}

void aran_solver2d_solve(AranSolver2d *solver) { (void)aran_solver2d_solve_try(solver); }

void aran_solver2d_get_functions_full(AranSolver2d *solver, AranParticle2ParticleFunc2d *p2p,
                                      AranParticle2MultipoleFunc2d *p2m,
                                      AranMultipole2MultipoleFunc2d *m2m,
                                      AranMultipole2LocalFunc2d *m2l, AranLocal2LocalFunc2d *l2l,
                                      AranLocal2ParticleFunc2d *l2p,
                                      AranParticle2LocalFunc2d *p2l,
                                      AranMultipole2ParticleFunc2d *m2p,
                                      guint *semifar_threshold) {
  (void)p2p;   // not written, like the 3D twin (aran/aransolver3d.c:676-684)
  if (!solver) return;
  if (p2m) *p2m = solver->p2m;
  if (m2m) *m2m = solver->m2m;
  if (m2l) *m2l = solver->m2l;
  if (l2l) *l2l = solver->l2l;
  if (l2p) *l2p = solver->l2p;
  if (p2l) *p2l = solver->p2l;
  if (m2p) *m2p = solver->m2p;
  if (semifar_threshold) *semifar_threshold = solver->semifar_threshold;
}

void aran_solver2d_db_profile_operators(AranSolver2d *solver, gdouble order) {
  if (!solver) return;
  if (solver->p2p) solver->p2p_time = aran_profile_db_address_eval((gpointer)solver->p2p, 0.);
  if (solver->p2m) solver->p2m_time = aran_profile_db_address_eval((gpointer)solver->p2m, order);
  if (solver->p2l) solver->p2l_time = aran_profile_db_address_eval((gpointer)solver->p2l, order);
  if (solver->l2p) solver->l2p_time = aran_profile_db_address_eval((gpointer)solver->p2p, order);
  if (solver->m2p) solver->m2p_time = aran_profile_db_address_eval((gpointer)solver->m2p, order);
  if (solver->m2m) solver->m2m_time = aran_profile_db_address_eval((gpointer)solver->m2m, order);
  if (solver->m2l) solver->m2l_time = aran_profile_db_address_eval((gpointer)solver->m2l, order);
  if (solver->l2l) solver->l2l_time = aran_profile_db_address_eval((gpointer)solver->l2l, order);
  std::fprintf(stderr, "db_p2p_time %p = %g\n", (void *)solver->p2p, solver->p2p_time);
  std::fprintf(stderr, "db_p2m_time %p = %g\n", (void *)solver->p2m, solver->p2m_time);
  std::fprintf(stderr, "db_p2l_time %p = %g\n", (void *)solver->p2l, solver->p2l_time);
  std::fprintf(stderr, "db_m2m_time %p = %g\n", (void *)solver->m2m, solver->m2m_time);
  std::fprintf(stderr, "db_m2l_time %p = %g\n", (void *)solver->m2l, solver->m2l_time);
  std::fprintf(stderr, "db_l2l_time %p = %g\n", (void *)solver->l2l, solver->l2l_time);
  std::fprintf(stderr, "db_l2p_time %p = %g\n", (void *)solver->l2p, solver->l2p_time);
  std::fprintf(stderr, "db_m2p_time %p = %g\n", (void *)solver->m2p, solver->m2p_time);
}

void aran_solver2d_profile_operators(AranSolver2d *solver, AranParticleInitFunc2d point_init,
                                     gpointer p1, gpointer p2) {
  (void)point_init;
  (void)p1;
  (void)p2;
  if (!solver || !solver->devel || solver->devel->multipole->negdeg < 1) return;
  AranGpuConfig2d cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.maxbox = (int)solver->tree->maxbox < 8 ? 8 : (int)solver->tree->maxbox;
  cfg.order = solver->devel->multipole->negdeg;
  const int64_t n = 100000;
  std::vector<double> xy(2 * n), q(n, 1.0 / n), acc(2 * n);
  uint64_t st = 0x9E3779B97F4A7C15ull;
  auto u = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return (double)(st >> 11) * (1.0 / 9007199254740992.0);
  };
  const VsgVector2d lb = solver->tree->lb, ub = solver->tree->ub;
  for (int64_t i = 0; i < n; ++i) {
    xy[2 * i] = lb.x + (ub.x - lb.x) * u();
    xy[2 * i + 1] = lb.y + (ub.y - lb.y) * u();
  }
  AranGpuSolver2d *g = nullptr;
  if (aran_gpu_solver2d_create(&cfg, &g) != ARAN_OK) return;
  int64_t offs[2] = {0, n}, c[11];
  double box[4] = {lb.x, lb.y, ub.x, ub.y}, ms[16];
  bool ok = true;
  for (int rep = 0; rep < 2 && ok; ++rep)
    ok = aran_gpu_solver2d_solve(g, 1, offs, box, xy.data(), q.data(), acc.data(),
                                 ARAN_MEM_HOST) == ARAN_OK;
  ok = ok && aran_gpu_solver2d_timings(g, ms) == ARAN_OK &&
       aran_gpu_solver2d_get_stats(g, c) == ARAN_OK;
  aran_gpu_solver2d_destroy(g);
  if (!ok) return;
  auto per = [](double stage_ms, int64_t count) { return count > 0 ? 1e-3 * stage_ms / count : -1.0; };
  solver->p2p_time = per(ms[9], c[1]);
  solver->p2m_time = per(ms[4], c[2]);
  solver->m2m_time = per(ms[5], c[3]);
  solver->m2l_time = per(ms[6], c[4]);
  solver->l2l_time = per(ms[7], c[5]);
  solver->l2p_time = per(ms[8], c[6]);
}

guint aran_solver2d_optimal_semifar_threshold(AranSolver2d *solver) {
  if (!solver) return G_MAXUINT;
  if (solver->p2l_time < 0. || solver->m2p_time < 0. || !(solver->p2p_time > 0.))
    return G_MAXUINT;
  const double t = (solver->p2l_time + solver->m2p_time) / solver->p2p_time;
  return t >= (double)G_MAXUINT ? G_MAXUINT : (guint)t;
}

void aran_solver2d_set_children_order_hilbert(AranSolver2d *solver) {
  if (solver) solver->hilbert = true;
}

void aran_solver2d_set_children_order_default(AranSolver2d *solver) {
  if (solver) solver->hilbert = false;
}

void aran_solver2d_set_nf_isleaf(AranSolver2d *solver, VsgPRTree2dNFIsleafFunc isleaf,
                                 gpointer user_data) {
  if (!solver) return;
  solver->nf_isleaf = isleaf;
  solver->nf_isleaf_data = user_data;
  solver->solved_current = false;
}

void aran_solver2d_traverse(AranSolver2d *solver, GTraverseType order, VsgPRTree2dFunc func,
                            gpointer user_data) {
  if (!solver || !func || solver->points.empty() || !solver->devel) return;
  if (gpu_solver2(solver) != ARAN_OK) return;
  aran::Forest2dHost h;
  const int64_t n = (int64_t)solver->points.size();
  if (!solver->solved_current) {
    std::vector<double> xy, q;
    gather2(solver, 0, (size_t)-1, xy, q);
    int64_t offs[2] = {0, n};
    double box[4] = {solver->tree->lb.x, solver->tree->lb.y, solver->tree->ub.x,
                     solver->tree->ub.y};
    if (aran::solve2d_impl(solver->gpu, 1, offs, box, xy.data(), q.data(), nullptr,
                           ARAN_MEM_HOST, true) != ARAN_OK)
      return;
  }
  if (aran::forest2d_to_host(solver->gpu, h, solver->solved_current) != ARAN_OK) return;
  const int nn = h.nnodes, p = h.p;
  std::vector<VsgPRTree2dNodeInfo> info(nn);
  std::vector<GSList> cells(n);
  std::vector<AranDevelopment2d *> devs(nn, nullptr);
  for (int i = 0; i < nn; ++i) {
    VsgPRTree2dNodeInfo &f = info[i];
    std::memset(&f, 0, sizeof(f));
    f.center = {h.center[2 * (size_t)i], h.center[2 * (size_t)i + 1]};
    const double *bx = h.sysbox.data() + 6 * (size_t)h.sys[i];
    double lo[2], hi[2];
    for (int a = 0; a < 2; ++a) {
      lo[a] = bx[a];
      hi[a] = bx[2 + a];
      for (int b = h.depth[i] - 1; b >= 0; --b) {
        const double mid = (lo[a] + hi[a]) * 0.5;
        if ((h.ij[2 * (size_t)i + a] >> b) & 1) lo[a] = mid;
        else hi[a] = mid;
      }
    }
    f.lbound = {lo[0], lo[1]};
    f.ubound = {hi[0], hi[1]};
    f.point_count = (guint)(h.end[i] - h.begin[i]);
    f.isleaf = h.child[i] < 0;
    f.depth = h.depth[i];
    f.id = (guint)i;
    f.father_info = h.parent[i] >= 0 ? &info[h.parent[i]] : nullptr;
    if (f.isleaf && h.end[i] > h.begin[i]) {
      for (int k = h.begin[i]; k < h.end[i]; ++k) {
        cells[k].data = solver->points[h.perm[k]];
        cells[k].next = k + 1 < h.end[i] ? &cells[k + 1] : nullptr;
      }
      f.point_list = &cells[h.begin[i]];
    }
    // developments aran_development2d_new (0, p): multipole term z^-t and
    // local term z^k of the node after a solve, zero before
    AranDevelopment2d *d = aran_development2d_new(0, (guint8)p);
    if (!h.mult.empty())
      for (int t = 0; t <= p; ++t) {
        const size_t k = ((size_t)i * (p + 1) + t) * 2;
        *aran_laurent_seriesd_get_term(d->multipole, -t) = gcomplex128(h.mult[k], h.mult[k + 1]);
        *aran_laurent_seriesd_get_term(d->local, t) = gcomplex128(h.loc[k], h.loc[k + 1]);
      }
    devs[i] = d;
    f.user_data = d;
  }
  auto kids = [&](int i, int out[4]) {
    for (int o = 0; o < 4; ++o) out[o] = h.child[i] + o;
    if (solver->hilbert) {
      uint64_t key[4];
      for (int o = 0; o < 4; ++o) {
        const int c = h.child[i] + o;
        key[o] = hilbert2((uint32_t)h.ij[2 * (size_t)c], (uint32_t)h.ij[2 * (size_t)c + 1],
                          h.depth[c]);
      }
      std::sort(out, out + 4,
                [&](int a, int b) { return key[a - h.child[i]] < key[b - h.child[i]]; });
    }
  };
  if (order == G_LEVEL_ORDER) {
    std::vector<int> level{0}, next;
    while (!level.empty()) {
      next.clear();
      for (int i : level) {
        func(&info[i], user_data);
        if (h.child[i] >= 0) {
          int k[4];
          kids(i, k);
          next.insert(next.end(), k, k + 4);
        }
      }
      level.swap(next);
    }
  } else {
    std::vector<std::pair<int, int>> stack{{0, 0}};
    std::vector<std::array<int, 4>> order_of(nn);
    while (!stack.empty()) {
      auto &top = stack.back();
      const int i = top.first;
      const bool leaf = h.child[i] < 0;
      if (top.second == 0) {
        if (!leaf) kids(i, order_of[i].data());
        if (order == G_PRE_ORDER || (leaf && order == G_IN_ORDER)) func(&info[i], user_data);
      }
      if (leaf || top.second == 4) {
        if (order == G_POST_ORDER) func(&info[i], user_data);
        stack.pop_back();
        continue;
      }
      if (order == G_IN_ORDER && top.second == 1) func(&info[i], user_data);
      const int c = order_of[i][top.second++];
      stack.push_back({c, 0});
    }
  }
  for (auto *d : devs) aran_development2d_free(d);
}

void aran_solver2d_foreach_point_custom(AranSolver2d *solver, VsgRegion2 selector,
                                        VsgRegion2Point2LocFunc locfunc, GFunc func,
                                        gpointer user_data) {
  if (!solver || !locfunc || !func) return;
  struct Ctx {
    VsgRegion2 sel;
    VsgRegion2Point2LocFunc loc;
    GFunc fn;
    gpointer data;
  } ctx{selector, locfunc, func, user_data};
  aran_solver2d_traverse(
      solver, G_PRE_ORDER,
      [](const VsgPRTree2dNodeInfo *node, gpointer d) {
        Ctx *c = (Ctx *)d;
        if (!node->isleaf) return;
        for (GSList *l = node->point_list; l; l = l->next)
          if (c->loc(c->sel, l->data) == VSG_RLOC2_MASK) c->fn(l->data, c->data);
      },
      &ctx);
}

}  // extern "C"
