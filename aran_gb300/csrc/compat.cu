// compat.cu -- LibAran's public 3D solver API (aran/aransolver3d.h,
// aran/aran.h and the vsg_prtree3d_new_full tree constructor) implemented on
// the GPU solver, so a program written against LibAran keeps its calls.  See
// include/aran/aransolver3d.h for the contract; the development and series
// operators are in series3d.cu.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "internal.cuh"

#include <aran/aranprofiledb.h>
#include <aran/aransolver3d.h>

struct _VsgPRTree3d {
  VsgVector3d lb, ub;
  guint maxbox;
  gdouble tolerance;
};

struct _AranSolver3d {
  VsgPRTree3d *tree = nullptr;
  AranDevelopment3d *devel = nullptr;
  AranZeroFunc zero = nullptr;
  AranParticle2ParticleFunc3d p2p = nullptr;
  AranParticle2MultipoleFunc3d p2m = nullptr;
  AranMultipole2MultipoleFunc3d m2m = nullptr;
  AranMultipole2LocalFunc3d m2l = nullptr;
  AranLocal2LocalFunc3d l2l = nullptr;
  AranLocal2ParticleFunc3d l2p = nullptr;
  AranParticle2LocalFunc3d p2l = nullptr;
  AranMultipole2ParticleFunc3d m2p = nullptr;
  guint semifar_threshold = 0;
  std::vector<VsgPoint3> points;
  int kind = -1;
  size_t off_pos = 0, off_q = 0, off_res = 0;
  int precision = ARAN_PRECISION_FP64;
  AranGpuSolver3d *gpu = nullptr;
  AranGpuConfig3d gpu_cfg;
  int64_t stats[11] = {};
  guint depth = 0;
  // virtual leaves (aran_solver3d_set_nf_isleaf)
  VsgPRTree3dNFIsleafFunc nf_isleaf = nullptr;
  gpointer nf_isleaf_data = nullptr;
  bool hilbert = false;
  // operator costs (db_profile_operators / profile_operators); < 0: unknown
  double p2p_time = -1, p2m_time = -1, p2l_time = -1, l2p_time = -1, m2p_time = -1,
         m2m_time = -1, m2l_time = -1, l2l_time = -1;
  // the last solve ran on exactly the current points (their expansions are
  // those of the GPU solver's last solve)
  bool solved_current = false;
  // find_point grid: cell of side `cell` -> points (VsgVector3d at offset 0)
  double cell = -1.;
  std::map<std::tuple<int64_t, int64_t, int64_t>, std::vector<VsgPoint3>> grid;
};

namespace {

const VsgVector3d *pos0(VsgPoint3 p) { return (const VsgVector3d *)p; }

// grid cell of a position: side = tolerance (1 when the tolerance is 0, the
// search then compares exact positions)
std::tuple<int64_t, int64_t, int64_t> cell_of(double side, const VsgVector3d *v) {
  return std::make_tuple((int64_t)std::floor(v->x / side), (int64_t)std::floor(v->y / side),
                         (int64_t)std::floor(v->z / side));
}

void grid_sync(AranSolver3d *s) {
  const double tol = s->tree->tolerance;
  const double side = tol > 0 ? tol : 1.0;
  if (side == s->cell) return;
  s->grid.clear();
  s->cell = side;
  for (VsgPoint3 p : s->points) s->grid[cell_of(side, pos0(p))].push_back(p);
}

// Hilbert index of cell (x, y, z) of a 2^bits grid: J. Skilling, "Programming
// the Hilbert curve", AIP Conf. Proc. 707 (2004) 381 -- axes to transposed
// index, then the bits interleaved
uint64_t hilbert_index(uint32_t x, uint32_t y, uint32_t z, int bits) {
  uint32_t X[3] = {x, y, z};
  const uint32_t M = 1u << (bits - 1);
  for (uint32_t Q = M; Q > 1; Q >>= 1) {
    const uint32_t P = Q - 1;
    for (int i = 0; i < 3; ++i) {
      if (X[i] & Q) X[0] ^= P;
      else {
        const uint32_t t = (X[0] ^ X[i]) & P;
        X[0] ^= t;
        X[i] ^= t;
      }
    }
  }
  for (int i = 1; i < 3; ++i) X[i] ^= X[i - 1];
  uint32_t t = 0;
  for (uint32_t Q = M; Q > 1; Q >>= 1)
    if (X[2] & Q) t ^= Q - 1;
  for (int i = 0; i < 3; ++i) X[i] ^= t;
  uint64_t h = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < 3; ++i) h = (h << 1) | ((X[i] >> b) & 1u);
  return h;
}

gboolean nf_isleaf_adapter(const AranGpuNodeView *v, void *data) {
  AranSolver3d *s = (AranSolver3d *)data;
  VsgPRTree3dNodeInfo info;
  std::memset(&info, 0, sizeof(info));
  info.center = {v->center[0], v->center[1], v->center[2]};
  info.lbound = {v->lbound[0], v->lbound[1], v->lbound[2]};
  info.ubound = {v->ubound[0], v->ubound[1], v->ubound[2]};
  info.point_count = (guint)v->point_count;
  info.depth = (guint)v->depth;
  return s->nf_isleaf(&info, s->nf_isleaf_data);
}

int leaf_pred_adapter(const AranGpuNodeView *v, void *data) { return nf_isleaf_adapter(v, data) ? 1 : 0; }

// the GPU configuration of the solver's current functions and tree; flavour
// < 0 and a message when the operators do not run on the GPU
int gpu_config(AranSolver3d *solver, AranGpuConfig3d *cfg) {
  if (!solver->devel || aran_spherical_seriesd_get_negdeg(solver->devel->multipole) < 1) {
    aran::set_error("aran_solver3d: no development (aran_development3d_new (0, p))");
    return ARAN_ERR_INVALID;
  }
  auto is = [](void *f, void *g) { return f == g; };
  int flavour = -1;
  if (is((void *)solver->m2m, (void *)&aran_development3d_m2m_rotate) &&
      is((void *)solver->m2l, (void *)&aran_development3d_m2l_rotate) &&
      is((void *)solver->l2l, (void *)&aran_development3d_l2l_rotate))
    flavour = ARAN_FLAVOUR_ROTATE;
  else if (is((void *)solver->m2m, (void *)&aran_development3d_m2m_kkylin) &&
           is((void *)solver->m2l, (void *)&aran_development3d_m2l_kkylin) &&
           is((void *)solver->l2l, (void *)&aran_development3d_l2l_kkylin))
    flavour = ARAN_FLAVOUR_KKYLIN;
  else if (is((void *)solver->m2m, (void *)&aran_development3d_m2m) &&
           is((void *)solver->m2l, (void *)&aran_development3d_m2l) &&
           is((void *)solver->l2l, (void *)&aran_development3d_l2l))
    flavour = ARAN_FLAVOUR_NORMAL;
  if (flavour < 0) {
    aran::set_error("aran_solver3d_solve: m2m/m2l/l2l must be one flavour of this library's "
                    "operators (normal, kkylin or rotate); user translations do not run on "
                    "the GPU");
    return ARAN_ERR_UNSUPPORTED;
  }
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->lb[0] = solver->tree->lb.x;
  cfg->lb[1] = solver->tree->lb.y;
  cfg->lb[2] = solver->tree->lb.z;
  cfg->ub[0] = solver->tree->ub.x;
  cfg->ub[1] = solver->tree->ub.y;
  cfg->ub[2] = solver->tree->ub.z;
  cfg->maxbox = (int)solver->tree->maxbox;
  cfg->order = aran_spherical_seriesd_get_negdeg(solver->devel->multipole);
  cfg->flavour = flavour;
  cfg->field = solver->kind == ARAN_NEWTON_FIELD;
  cfg->precision = solver->precision;
  cfg->max_depth = 0;
  // semifar only with p2l and m2p (aransolver3d.c:1152-1160): G_MAXUINT
  // turns it off, 0 asks for the optimal threshold
  if (solver->p2l && solver->m2p && solver->semifar_threshold != G_MAXUINT) {
    guint t = solver->semifar_threshold ? solver->semifar_threshold
                                        : aran_solver3d_optimal_semifar_threshold(solver);
    cfg->semifar_threshold = t > 0x7fffffffu ? 0 : (int)t;
  }
  return ARAN_OK;
}

// the GPU solver of cfg, made anew when the configuration changed; the
// virtual-leaf predicate follows the LibAran solver's
int gpu_solver(AranSolver3d *solver, const AranGpuConfig3d &cfg) {
  if (!solver->gpu || std::memcmp(&cfg, &solver->gpu_cfg, sizeof(cfg)) != 0) {
    if (solver->gpu) aran_gpu_solver3d_destroy(solver->gpu);
    solver->gpu = nullptr;
    solver->solved_current = false;
    int rc = aran_gpu_solver3d_create(&cfg, &solver->gpu);
    if (rc != ARAN_OK) return rc;
    solver->gpu_cfg = cfg;
  }
  return aran_gpu_solver3d_set_leaf_predicate(solver->gpu,
                                              solver->nf_isleaf ? leaf_pred_adapter : nullptr,
                                              solver);
}

void gather(AranSolver3d *solver, size_t off_pos, size_t off_q, std::vector<double> &xyz,
            std::vector<double> &q) {
  const size_t n = solver->points.size();
  xyz.resize(3 * n);
  q.resize(n);
  for (size_t i = 0; i < n; ++i) {
    const char *pt = (const char *)solver->points[i];
    const VsgVector3d *v = (const VsgVector3d *)(pt + off_pos);
    xyz[3 * i] = v->x;
    xyz[3 * i + 1] = v->y;
    xyz[3 * i + 2] = v->z;
    q[i] = off_q == (size_t)-1 ? 0.0 : *(const double *)(pt + off_q);
  }
}

}  // namespace


extern "C" {

void aran_init(void) {
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaSetDevice(dev);
}

VsgPRTree3d *vsg_prtree3d_new_full(const VsgVector3d *lbound, const VsgVector3d *ubound,
                                   VsgPoint3dLocFunc, VsgPoint3dDistFunc, VsgRegion3dLocFunc,
                                   guint maxbox) {
  if (!lbound || !ubound) return nullptr;
  VsgPRTree3d *t = new VsgPRTree3d();
  t->lb = *lbound;
  t->ub = *ubound;
  t->maxbox = maxbox > 0 ? maxbox : 1;
  t->tolerance = 0.;
  return t;
}

void vsg_prtree3d_free(VsgPRTree3d *prtree) { delete prtree; }

gint vsg_vector3d_vector3d_locfunc(const VsgVector3d *candidate, const VsgVector3d *center) {
  return (candidate->x > center->x ? 1 : 0) | (candidate->y > center->y ? 2 : 0) |
         (candidate->z > center->z ? 4 : 0);
}

gdouble vsg_vector3d_dist(const VsgVector3d *one, const VsgVector3d *other) {
  double dx = one->x - other->x, dy = one->y - other->y, dz = one->z - other->z;
  return sqrt(dx * dx + dy * dy + dz * dz);
}

// ---- solver (aran/aransolver3d.c) ----
AranSolver3d *aran_solver3d_new(VsgPRTree3d *prtree, GType devel_type, gpointer devel,
                                AranZeroFunc zero) {
  AranSolver3d *s = new AranSolver3d();
  if (!prtree) {
    // aran/aransolver3d.c:514-523: default tree [-1,1]^3
    VsgVector3d lb = {-1., -1., -1.}, ub = {1., 1., 1.};
    prtree = vsg_prtree3d_new_full(&lb, &ub, nullptr, nullptr, nullptr, 1);
  }
  s->tree = prtree;
  aran_solver3d_set_development(s, devel_type, devel, zero);
  return s;
}

void aran_solver3d_free(AranSolver3d *solver) {
  if (!solver) return;
  if (solver->gpu) aran_gpu_solver3d_destroy(solver->gpu);
  vsg_prtree3d_free(solver->tree);
  aran_development3d_free(solver->devel);
  delete solver;
}

void aran_solver3d_set_development(AranSolver3d *solver, GType devel_type, gpointer devel,
                                   AranZeroFunc zero) {
  if (!solver) return;
  if (devel && devel_type != aran_development3d_get_type()) {
    aran::set_error("aran_solver3d_set_development: only ARAN_TYPE_DEVELOPMENT3D is supported");
    return;
  }
  if (solver->devel && solver->devel != devel) aran_development3d_free(solver->devel);
  solver->devel = (AranDevelopment3d *)devel;
  solver->zero = zero;
}

void aran_solver3d_set_functions_full(AranSolver3d *solver, AranParticle2ParticleFunc3d p2p,
                                      AranParticle2MultipoleFunc3d p2m,
                                      AranMultipole2MultipoleFunc3d m2m,
                                      AranMultipole2LocalFunc3d m2l, AranLocal2LocalFunc3d l2l,
                                      AranLocal2ParticleFunc3d l2p, AranParticle2LocalFunc3d p2l,
                                      AranMultipole2ParticleFunc3d m2p, guint semifar_threshold) {
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

void aran_solver3d_set_functions(AranSolver3d *solver, AranParticle2ParticleFunc3d p2p,
                                 AranParticle2MultipoleFunc3d p2m,
                                 AranMultipole2MultipoleFunc3d m2m, AranMultipole2LocalFunc3d m2l,
                                 AranLocal2LocalFunc3d l2l, AranLocal2ParticleFunc3d l2p) {
  aran_solver3d_set_functions_full(solver, p2p, p2m, m2m, m2l, l2l, l2p, nullptr, nullptr, 0);
}

void aran_solver3d_reinit_stats(AranSolver3d *solver) {
  if (solver) std::memset(solver->stats, 0, sizeof(solver->stats));
}

void aran_solver3d_get_stats(AranSolver3d *solver, glong *zero_count, glong *p2p_count,
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

gdouble aran_solver3d_get_tolerance(AranSolver3d *solver) {
  return solver ? solver->tree->tolerance : -1.;
}

void aran_solver3d_set_tolerance(AranSolver3d *solver, gdouble tolerance) {
  if (solver) solver->tree->tolerance = tolerance;
}

void aran_solver3d_get_bounds(AranSolver3d *solver, VsgVector3d *lbound, VsgVector3d *ubound) {
  if (!solver) return;
  if (lbound) *lbound = solver->tree->lb;
  if (ubound) *ubound = solver->tree->ub;
}

guint aran_solver3d_depth(const AranSolver3d *solver) { return solver ? solver->depth : 0; }

guint aran_solver3d_point_count(const AranSolver3d *solver) {
  return solver ? (guint)solver->points.size() : 0;
}

void aran_solver3d_insert_point(AranSolver3d *solver, VsgPoint3 point) {
  if (!solver || !point) return;
  solver->points.push_back(point);
  solver->solved_current = false;
  if (solver->cell > 0) solver->grid[cell_of(solver->cell, pos0(point))].push_back(point);
}

gboolean aran_solver3d_insert_point_local(AranSolver3d *solver, VsgPoint3 point) {
  if (!solver || !point) return FALSE;
  aran_solver3d_insert_point(solver, point);
  return TRUE;
}

gboolean aran_solver3d_remove_point(AranSolver3d *solver, VsgPoint3 point) {
  if (!solver) return FALSE;
  for (size_t i = 0; i < solver->points.size(); ++i)
    if (solver->points[i] == point) {
      solver->points.erase(solver->points.begin() + i);
      solver->solved_current = false;
      if (solver->cell > 0) {
        auto &v = solver->grid[cell_of(solver->cell, pos0(point))];
        v.erase(std::find(v.begin(), v.end(), point));
      }
      return TRUE;
    }
  return FALSE;
}

VsgPoint3 aran_solver3d_find_point(AranSolver3d *solver, VsgPoint3 selector) {
  if (!solver || !selector) return nullptr;
  grid_sync(solver);
  const double tol = solver->tree->tolerance;
  const VsgVector3d *v = pos0(selector);
  auto c = cell_of(solver->cell, v);
  const int64_t r = tol > 0 ? 1 : 0;
  for (int64_t dz = -r; dz <= r; ++dz)
    for (int64_t dy = -r; dy <= r; ++dy)
      for (int64_t dx = -r; dx <= r; ++dx) {
        auto it = solver->grid.find(std::make_tuple(std::get<0>(c) + dx, std::get<1>(c) + dy,
                                                    std::get<2>(c) + dz));
        if (it == solver->grid.end()) continue;
        for (VsgPoint3 p : it->second) {
          const VsgVector3d *w = pos0(p);
          if (tol > 0 ? vsg_vector3d_dist(v, w) <= tol
                      : (w->x == v->x && w->y == v->y && w->z == v->z))
            return p;
        }
      }
  return nullptr;
}

void aran_solver3d_get_functions_full(AranSolver3d *solver, AranParticle2ParticleFunc3d *p2p,
                                      AranParticle2MultipoleFunc3d *p2m,
                                      AranMultipole2MultipoleFunc3d *m2m,
                                      AranMultipole2LocalFunc3d *m2l, AranLocal2LocalFunc3d *l2l,
                                      AranLocal2ParticleFunc3d *l2p,
                                      AranParticle2LocalFunc3d *p2l,
                                      AranMultipole2ParticleFunc3d *m2p,
                                      guint *semifar_threshold) {
  (void)p2p;   // not written, as in aran/aransolver3d.c:676-684
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

void aran_solver3d_set_children_order_hilbert(AranSolver3d *solver) {
  if (solver) solver->hilbert = true;
}

void aran_solver3d_set_children_order_default(AranSolver3d *solver) {
  if (solver) solver->hilbert = false;
}

void aran_solver3d_set_nf_isleaf(AranSolver3d *solver, VsgPRTree3dNFIsleafFunc isleaf,
                                 gpointer user_data) {
  if (!solver) return;
  solver->nf_isleaf = isleaf;
  solver->nf_isleaf_data = user_data;
  solver->solved_current = false;
}

void aran_solver3d_traverse(AranSolver3d *solver, GTraverseType order, VsgPRTree3dFunc func,
                            gpointer user_data) {
  if (!solver || !func || solver->points.empty()) return;
  AranGpuConfig3d cfg;
  int rc = gpu_config(solver, &cfg);
  if (rc == ARAN_OK) rc = gpu_solver(solver, cfg);
  if (rc != ARAN_OK) return;
  AranGpuSolver3d *g = solver->gpu;
  const int p = cfg.order;
  std::vector<double> em, el;
  try {
    if (!solver->solved_current) {
      std::vector<double> xyz, q;
      gather(solver, 0, (size_t)-1, xyz, q);
      aran::build_tree_only(g, (int64_t)solver->points.size(), xyz.data(), q.data());
    } else {
      const size_t nn = g->tree.nnodes;
      em.resize(nn * p * (p + 1));
      el.resize(nn * (p + 1) * (p + 2));
      aran::copy_expansions(g, em.data(), el.data());
    }
  } catch (const aran::CudaError &ce) {
    aran::from_cuda(ce);
    return;
  } catch (const aran::InputError &ie) {
    aran::set_error(ie.msg);
    return;
  }
  aran::DevTree &t = g->tree;
  const int nn = t.nnodes;
  std::vector<int> beg(nn), end(nn), child(nn), parent(nn), ijk(3 * (size_t)nn), perm(t.n);
  std::vector<uint8_t> dep(nn);
  std::vector<double> ctr(3 * (size_t)nn);
  cudaMemcpy(beg.data(), t.begin.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(end.data(), t.end.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(child.data(), t.child.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(parent.data(), t.parent.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(ijk.data(), t.ijk.ptr, 3 * (size_t)nn * sizeof(int), cudaMemcpyDeviceToHost);
  cudaMemcpy(dep.data(), t.depth.ptr, nn, cudaMemcpyDeviceToHost);
  cudaMemcpy(ctr.data(), t.center.ptr, 3 * (size_t)nn * sizeof(double), cudaMemcpyDeviceToHost);
  if (cudaMemcpy(perm.data(), g->perm.ptr, t.n * sizeof(int), cudaMemcpyDeviceToHost) !=
      cudaSuccess) {
    aran::set_error("aran_solver3d_traverse: copying the tree failed");
    return;
  }
  // node infos (father_info pointers into the same array), point lists of
  // the leaves, developments
  std::vector<VsgPRTree3dNodeInfo> info(nn);
  std::vector<GSList> cells(t.n);
  std::vector<AranDevelopment3d *> devs(nn, nullptr);
  for (int i = 0; i < nn; ++i) {
    VsgPRTree3dNodeInfo &f = info[i];
    std::memset(&f, 0, sizeof(f));
    f.center = {ctr[3 * (size_t)i], ctr[3 * (size_t)i + 1], ctr[3 * (size_t)i + 2]};
    double lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = cfg.lb[a];
      hi[a] = cfg.ub[a];
      for (int b = dep[i] - 1; b >= 0; --b) {
        const double mid = (lo[a] + hi[a]) * 0.5;
        if ((ijk[3 * (size_t)i + a] >> b) & 1) lo[a] = mid;
        else hi[a] = mid;
      }
    }
    f.lbound = {lo[0], lo[1], lo[2]};
    f.ubound = {hi[0], hi[1], hi[2]};
    f.point_count = (guint)(end[i] - beg[i]);
    f.isleaf = child[i] < 0;
    f.depth = dep[i];
    f.id = (guint)i;
    f.father_info = parent[i] >= 0 ? &info[parent[i]] : nullptr;
    if (f.isleaf && end[i] > beg[i]) {
      for (int k = beg[i]; k < end[i]; ++k) {
        cells[k].data = solver->points[perm[k]];
        cells[k].next = k + 1 < end[i] ? &cells[k + 1] : nullptr;
      }
      f.point_list = &cells[beg[i]];
    }
    AranDevelopment3d *d = aran_development3d_new(0, (guint8)p);
    if (!em.empty()) {
      for (int l = 0; l < p; ++l)
        for (int m = 0; m <= l; ++m) {
          const size_t k = (size_t)i * p * (p + 1) / 2 + l * (l + 1) / 2 + m;
          *aran_spherical_seriesd_get_term(d->multipole, -l - 1, m) = gcomplex128(em[2 * k], em[2 * k + 1]);
        }
      for (int l = 0; l <= p; ++l)
        for (int m = 0; m <= l; ++m) {
          const size_t k = (size_t)i * (p + 1) * (p + 2) / 2 + l * (l + 1) / 2 + m;
          *aran_spherical_seriesd_get_term(d->local, l, m) = gcomplex128(el[2 * k], el[2 * k + 1]);
        }
    }
    devs[i] = d;
    f.user_data = d;
  }
  // children in octant order x + 2y + 4z (the tree's) or along the Hilbert curve
  auto kids = [&](int i, int out[8]) {
    for (int o = 0; o < 8; ++o) out[o] = child[i] + o;
    if (solver->hilbert) {
      uint64_t h[8];
      for (int o = 0; o < 8; ++o) {
        const int c = child[i] + o;
        h[o] = hilbert_index((uint32_t)ijk[3 * (size_t)c], (uint32_t)ijk[3 * (size_t)c + 1],
                             (uint32_t)ijk[3 * (size_t)c + 2], dep[c]);
      }
      std::sort(out, out + 8, [&](int a, int b) { return h[a - child[i]] < h[b - child[i]]; });
    }
  };
  if (order == G_LEVEL_ORDER) {
    std::vector<int> level{0}, next;
    while (!level.empty()) {
      next.clear();
      for (int i : level) {
        func(&info[i], user_data);
        if (child[i] >= 0) {
          int k[8];
          kids(i, k);
          next.insert(next.end(), k, k + 8);
        }
      }
      level.swap(next);
    }
  } else {
    // iterative depth-first walk: (node, next child position)
    std::vector<std::pair<int, int>> stack{{0, 0}};
    std::vector<std::array<int, 8>> order_of(nn);
    while (!stack.empty()) {
      auto &top = stack.back();
      const int i = top.first;
      const bool leaf = child[i] < 0;
      if (top.second == 0) {
        if (!leaf) kids(i, order_of[i].data());
        if (order == G_PRE_ORDER || (leaf && order == G_IN_ORDER)) func(&info[i], user_data);
      }
      if (leaf || top.second == 8) {
        if (order == G_POST_ORDER) func(&info[i], user_data);
        stack.pop_back();
        continue;
      }
      if (order == G_IN_ORDER && top.second == 1) func(&info[i], user_data);
      const int c = order_of[i][top.second++];
      stack.push_back({c, 0});
    }
  }
  for (auto *d : devs) aran_development3d_free(d);
}

void aran_solver3d_foreach_point_custom(AranSolver3d *solver, VsgRegion3 selector,
                                        VsgRegion3Point3LocFunc locfunc, GFunc func,
                                        gpointer user_data) {
  if (!solver || !locfunc || !func) return;
  struct Ctx {
    VsgRegion3 sel;
    VsgRegion3Point3LocFunc loc;
    GFunc fn;
    gpointer data;
  } ctx{selector, locfunc, func, user_data};
  aran_solver3d_traverse(
      solver, G_PRE_ORDER,
      [](const VsgPRTree3dNodeInfo *node, gpointer d) {
        Ctx *c = (Ctx *)d;
        if (!node->isleaf) return;
        for (GSList *l = node->point_list; l; l = l->next)
          if (c->loc(c->sel, l->data) == VSG_RLOC3_MASK) c->fn(l->data, c->data);
      },
      &ctx);
}

void aran_solver3d_db_profile_operators(AranSolver3d *solver, gdouble order) {
  if (!solver) return;
  // aran/aransolver3d.c:687-740, with its lookup of the l2p cost under the
  // p2p address kept
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

void aran_solver3d_profile_operators(AranSolver3d *solver, AranParticleInitFunc3d point_init,
                                     gpointer p1, gpointer p2) {
  (void)point_init;
  (void)p1;
  (void)p2;
  if (!solver) return;
  AranGpuConfig3d cfg;
  if (gpu_config(solver, &cfg) != ARAN_OK) return;
  cfg.semifar_threshold = 1;   // semifar interactions wherever the traversal allows them
  cfg.maxbox = cfg.maxbox < 8 ? 8 : cfg.maxbox;
  // calibration set: 200,000 particles of a Plummer sphere (scale radius
  // 1/40 of the box, cut at half the box) centred in the tree's box
  const int64_t n = 200000;
  std::vector<double> xyz(3 * n), q(n, 1.0 / n), pot(n), fld(3 * n);
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  double ext = 0, c[3];
  for (int a = 0; a < 3; ++a) {
    ext = std::fmax(ext, cfg.ub[a] - cfg.lb[a]);
    c[a] = 0.5 * (cfg.lb[a] + cfg.ub[a]);
  }
  for (int64_t i = 0; i < n;) {
    const double r = (ext / 40) / std::sqrt(std::pow(u(rng), -2.0 / 3.0) - 1.0);
    if (!(r <= 0.5 * ext * 0.999)) continue;
    const double z = (1.0 - 2.0 * u(rng)) * r, ph = 2.0 * M_PI * u(rng);
    const double rho = std::sqrt(std::fmax(r * r - z * z, 0.0));
    xyz[3 * i] = c[0] + rho * std::cos(ph);
    xyz[3 * i + 1] = c[1] + rho * std::sin(ph);
    xyz[3 * i + 2] = c[2] + z;
    ++i;
  }
  AranGpuSolver3d *g = nullptr;
  if (aran_gpu_solver3d_create(&cfg, &g) != ARAN_OK) return;
  double ms[16];
  int64_t st[11];
  bool ok = true;
  for (int rep = 0; rep < 2 && ok; ++rep)
    ok = aran_gpu_solver3d_solve(g, n, xyz.data(), q.data(), pot.data(),
                                 cfg.field ? fld.data() : nullptr, ARAN_MEM_HOST) == ARAN_OK;
  ok = ok && aran_gpu_solver3d_timings(g, ms) == ARAN_OK &&
       aran_gpu_solver3d_get_stats(g, st) == ARAN_OK;
  aran_gpu_solver3d_destroy(g);
  if (!ok) return;
  // seconds per operation: stage time over its count (P2P per unordered pair
  // as the reference's p2p callback handles one pair); the semifar stages
  // run inside the M2L and L2P spans
  auto per = [](double stage_ms, int64_t count) { return count > 0 ? 1e-3 * stage_ms / count : -1.0; };
  solver->p2p_time = per(ms[9], st[1]);
  solver->p2m_time = per(ms[4], st[2]);
  solver->m2m_time = per(ms[5], st[3]);
  solver->m2l_time = per(ms[6] - ms[12], st[4]);
  solver->l2l_time = per(ms[7], st[5]);
  solver->l2p_time = per(ms[8] - ms[13], st[6]);
  solver->p2l_time = per(ms[12], st[7]);
  solver->m2p_time = per(ms[13], st[8]);
}


void aran_solver3d_foreach_point(AranSolver3d *solver, GFunc func, gpointer user_data) {
  if (!solver || !func) return;
  for (VsgPoint3 p : solver->points) func(p, user_data);
}

// (p2l + m2p) / p2p of the operator costs (aran/aransolver3d.c:1090-1127);
// G_MAXUINT while a cost is unknown
guint aran_solver3d_optimal_semifar_threshold(AranSolver3d *solver) {
  if (!solver) return G_MAXUINT;
  if (solver->p2l_time < 0. || solver->m2p_time < 0. || !(solver->p2p_time > 0.))
    return G_MAXUINT;
  const double t = (solver->p2l_time + solver->m2p_time) / solver->p2p_time;
  return t >= (double)G_MAXUINT ? G_MAXUINT : (guint)t;
}

void aran_solver3d_set_newton_layout(AranSolver3d *solver, int kind, size_t pos_offset,
                                     size_t charge_offset, size_t result_offset) {
  if (!solver) return;
  solver->kind = kind;
  solver->off_pos = pos_offset;
  solver->off_q = charge_offset;
  solver->off_res = result_offset;
}

void aran_solver3d_set_precision(AranSolver3d *solver, int precision) {
  if (solver) solver->precision = precision;
}

int aran_solver3d_solve_try(AranSolver3d *solver) {
  if (!solver) {
    aran::set_error("aran_solver3d_solve: solver is NULL");
    return ARAN_ERR_INVALID;
  }
  if (solver->kind != ARAN_NEWTON_POTENTIAL && solver->kind != ARAN_NEWTON_FIELD) {
    aran::set_error("aran_solver3d_solve: call aran_solver3d_set_newton_layout first");
    return ARAN_ERR_INVALID;
  }
  if (!solver->p2p || !solver->p2m || !solver->l2p || !solver->m2l || !solver->m2m || !solver->l2l) {
    aran::set_error("aran_solver3d_solve: the GPU path needs p2p, p2m, m2m, m2l, l2l and l2p");
    return ARAN_ERR_INVALID;
  }
  AranGpuConfig3d cfg;
  int rc = gpu_config(solver, &cfg);
  if (rc != ARAN_OK) return rc;
  const int64_t n = (int64_t)solver->points.size();
  if (n == 0) return ARAN_OK;
  rc = gpu_solver(solver, cfg);
  if (rc != ARAN_OK) return rc;
  std::vector<double> xyz, q, pot(n), fld(cfg.field ? 3 * n : 0);
  gather(solver, solver->off_pos, solver->off_q, xyz, q);
  rc = aran_gpu_solver3d_solve(solver->gpu, n, xyz.data(), q.data(), pot.data(),
                               cfg.field ? fld.data() : nullptr, ARAN_MEM_HOST);
  if (rc != ARAN_OK) return rc;
  solver->solved_current = true;
  // results accumulate into the points, as the reference callbacks do
  for (int64_t i = 0; i < n; ++i) {
    char *pt = (char *)solver->points[i];
    if (cfg.field) {
      VsgVector3d *f = (VsgVector3d *)(pt + solver->off_res);
      f->x += fld[3 * i];
      f->y += fld[3 * i + 1];
      f->z += fld[3 * i + 2];
    } else {
      double *acc = (double *)(pt + solver->off_res);  // gcomplex128: (re, im)
      acc[0] += pot[i];
    }
  }
  int64_t st[11];
  if (aran_gpu_solver3d_get_stats(solver->gpu, st) == ARAN_OK)
    for (int k = 0; k < 11; ++k) solver->stats[k] += st[k];
  int64_t info[5];
  if (aran_gpu_solver3d_tree_info(solver->gpu, info) == ARAN_OK) solver->depth = (guint)info[4];
  return ARAN_OK;
}

void aran_solver3d_solve(AranSolver3d *solver) { (void)aran_solver3d_solve_try(solver); }

}  // extern "C"
