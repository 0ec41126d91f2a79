// compat.cu -- LibAran's public 3D solver API (aran/aransolver3d.h,
// aran/aran.h and the vsg_prtree3d_new_full tree constructor) implemented on
// the GPU solver, so a program written against LibAran keeps its calls.  See
// include/aran/aransolver3d.h for the contract; the development and series
// operators are in series3d.cu.
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "internal.cuh"

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
};


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
  if (solver && point) solver->points.push_back(point);
}

gboolean aran_solver3d_remove_point(AranSolver3d *solver, VsgPoint3 point) {
  if (!solver) return FALSE;
  for (size_t i = 0; i < solver->points.size(); ++i)
    if (solver->points[i] == point) {
      solver->points.erase(solver->points.begin() + i);
      return TRUE;
    }
  return FALSE;
}

void aran_solver3d_foreach_point(AranSolver3d *solver, GFunc func, gpointer user_data) {
  if (!solver || !func) return;
  for (VsgPoint3 p : solver->points) func(p, user_data);
}

// (p2l + m2p) / p2p cost per point on the GPU kernels, from their flop
// counts: P2L 8 tri(p+1), M2P with gradient 24 tri(p), P2P 20 per pair (the
// reference times the three callbacks instead, aransolver3d.c:1090-1127)
guint aran_solver3d_optimal_semifar_threshold(AranSolver3d *solver) {
  if (!solver || !solver->devel || !solver->p2l || !solver->m2p) return G_MAXUINT;
  int p = aran_spherical_seriesd_get_negdeg(solver->devel->multipole);
  return (guint)((8 * (p + 1) * (p + 2) / 2 + 24 * p * (p + 1) / 2) / 20);
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
  if (!solver->devel || aran_spherical_seriesd_get_negdeg(solver->devel->multipole) < 1) {
    aran::set_error("aran_solver3d_solve: no development (aran_development3d_new (0, p))");
    return ARAN_ERR_INVALID;
  }
  if (!solver->p2p || !solver->p2m || !solver->l2p || !solver->m2l || !solver->m2m || !solver->l2l) {
    aran::set_error("aran_solver3d_solve: the GPU path needs p2p, p2m, m2m, m2l, l2l and l2p");
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
  const int64_t n = (int64_t)solver->points.size();
  if (n == 0) return ARAN_OK;
  AranGpuConfig3d cfg;
  std::memset(&cfg, 0, sizeof(cfg));
  cfg.lb[0] = solver->tree->lb.x;
  cfg.lb[1] = solver->tree->lb.y;
  cfg.lb[2] = solver->tree->lb.z;
  cfg.ub[0] = solver->tree->ub.x;
  cfg.ub[1] = solver->tree->ub.y;
  cfg.ub[2] = solver->tree->ub.z;
  cfg.maxbox = (int)solver->tree->maxbox;
  cfg.order = aran_spherical_seriesd_get_negdeg(solver->devel->multipole);
  cfg.flavour = flavour;
  cfg.field = solver->kind == ARAN_NEWTON_FIELD;
  cfg.precision = solver->precision;
  cfg.max_depth = 0;
  // semifar only with p2l and m2p (aransolver3d.c:1152-1160): G_MAXUINT
  // turns it off, 0 asks for the optimal threshold
  if (solver->p2l && solver->m2p && solver->semifar_threshold != G_MAXUINT) {
    guint t = solver->semifar_threshold ? solver->semifar_threshold
                                        : aran_solver3d_optimal_semifar_threshold(solver);
    cfg.semifar_threshold = t > 0x7fffffffu ? 0 : (int)t;
  }
  if (!solver->gpu || std::memcmp(&cfg, &solver->gpu_cfg, sizeof(cfg)) != 0) {
    if (solver->gpu) aran_gpu_solver3d_destroy(solver->gpu);
    solver->gpu = nullptr;
    int rc = aran_gpu_solver3d_create(&cfg, &solver->gpu);
    if (rc != ARAN_OK) return rc;
    solver->gpu_cfg = cfg;
  }
  std::vector<double> xyz(3 * n), q(n), pot(n), fld(cfg.field ? 3 * n : 0);
  for (int64_t i = 0; i < n; ++i) {
    const char *pt = (const char *)solver->points[i];
    const VsgVector3d *v = (const VsgVector3d *)(pt + solver->off_pos);
    xyz[3 * i] = v->x;
    xyz[3 * i + 1] = v->y;
    xyz[3 * i + 2] = v->z;
    q[i] = *(const double *)(pt + solver->off_q);
  }
  int rc = aran_gpu_solver3d_solve(solver->gpu, n, xyz.data(), q.data(), pot.data(),
                                   cfg.field ? fld.data() : nullptr, ARAN_MEM_HOST);
  if (rc != ARAN_OK) return rc;
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
