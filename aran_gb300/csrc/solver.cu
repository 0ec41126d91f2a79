// solver.cu -- C ABI of libaran_gpu.so and the solve orchestration.
//
// aran_gpu_solver3d_solve replaces aran_solver3d_solve
// (aran/aransolver3d.c:1135-1202) plus the per-point insertion that precedes
// it: every stage runs on the device, the host only sequences launches.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>

#include "internal.cuh"

namespace aran {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }

int consumer_wait_polls() {
  const char *v = getenv("ARAN_DEBUG_WAIT_POLLS");
  if (!v || !*v) return 1 << 20;
  long k = strtol(v, nullptr, 10);
  return k < 0 ? 0 : (k > (1 << 20) ? (1 << 20) : (int)k);
}

void scatter_outputs(AranGpuSolver3d *s, double *pot, double *fld);

void smem_raise(const void *kernel, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> limit;
  int dev = 0;
  ACHECK(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  size_t &cur = limit[{dev, kernel}];
  if (cur >= bytes) return;
  ACHECK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  cur = bytes;
}

// uploads the systems of a solve (offs/boxes NULL: one system in the
// solver's box); skipped when they equal the last solve's
void set_systems(AranGpuSolver3d *s, int nsys, const int64_t *offs, const double *boxes,
                 int64_t n) {
  std::vector<int> off(nsys + 1);
  std::vector<double> box(9 * (size_t)nsys);
  for (int k = 0; k <= nsys; ++k) off[k] = offs ? (int)offs[k] : (k ? (int)n : 0);
  for (int k = 0; k < nsys; ++k)
    for (int a = 0; a < 3; ++a) {
      double *b = box.data() + 9 * (size_t)k;
      b[a] = boxes ? boxes[6 * (size_t)k + a] : s->cfg.lb[a];
      b[3 + a] = boxes ? boxes[6 * (size_t)k + 3 + a] : s->cfg.ub[a];
      b[6 + a] = (double)(1 << kKeyBits) / (b[3 + a] - b[a]);
    }
  if (nsys == s->nsys && off == s->h_sys_off && box == s->h_sys_box && s->sys_off.ptr) return;
  s->sys_off.reserve(off.size());
  s->sys_box.reserve(box.size());
  s->nsys = nsys;
  s->h_sys_off = off;
  s->h_sys_box = box;
  ACHECK(cudaMemcpyAsync(s->sys_off.ptr, s->h_sys_off.data(), off.size() * sizeof(int),
                         cudaMemcpyHostToDevice, s->s0));
  ACHECK(cudaMemcpyAsync(s->sys_box.ptr, s->h_sys_box.data(), box.size() * sizeof(double),
                         cudaMemcpyHostToDevice, s->s0));
}

void build_tree_only(AranGpuSolver3d *s, int64_t n, const double *xyz, const double *q) {
  ACHECK(cudaSetDevice(s->device));
  cudaStream_t st = s->s0;
  ACHECK(cudaMemsetAsync(s->err_dev.ptr, 0, sizeof(int), st));
  s->io_xyz.reserve(3 * n);
  s->io_q.reserve(n);
  ACHECK(cudaMemcpyAsync(s->io_xyz.ptr, xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
  ACHECK(cudaMemcpyAsync(s->io_q.ptr, q, n * sizeof(double), cudaMemcpyHostToDevice, st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SORT], st));
  set_systems(s, 1, nullptr, nullptr, n);
  build_tree(s, n, s->io_xyz.ptr, s->io_q.ptr);
  ACHECK(cudaStreamSynchronize(st));
  s->have_tree = false;   // no lists: counters and list queries need a solve
}

namespace {

// mixed solvers of order >= kRootFp64Order start with FP64 expansions at
// depths <= kRootFp64Depth (at most 584 nodes take FP64 M2L: depths 2-3)
constexpr int kRootFp64Order = 16;
constexpr int kRootFp64Depth = 3;

int check_config(const AranGpuConfig3d *c) {
  if (!c) return fail(ARAN_ERR_INVALID, "config is NULL");
  for (int a = 0; a < 3; ++a)
    if (!(c->ub[a] > c->lb[a]) || !std::isfinite(c->lb[a]) || !std::isfinite(c->ub[a]))
      return fail(ARAN_ERR_INVALID, "bounding box must satisfy lb < ub (finite)");
  if (c->maxbox < 0) return fail(ARAN_ERR_INVALID, "maxbox must be >= 1 (0: the tuned value)");
  if (c->order < 1 || c->order > kMaxOrder)
    return fail(ARAN_ERR_INVALID, "order must be in [1, " + std::to_string(kMaxOrder) + "]");
  // the normal flavour (aransphericalseriesd-translate.c:507-834) applies the
  // same linear operators as the rotate flavour; it runs the rotation
  // kernels (O(p^3) per translation instead of O(p^4), equal to FP64 rounding)
  if (c->flavour != ARAN_FLAVOUR_ROTATE && c->flavour != ARAN_FLAVOUR_KKYLIN &&
      c->flavour != ARAN_FLAVOUR_NORMAL)
    return fail(ARAN_ERR_INVALID, "unknown flavour");
  if (c->precision != ARAN_PRECISION_FP64 && c->precision != ARAN_PRECISION_MIXED)
    return fail(ARAN_ERR_INVALID, "unknown precision");
  if (c->max_depth < 0 || c->max_depth > kKeyBits)
    return fail(ARAN_ERR_INVALID, "max_depth must be in [0, 21]");
  // the kkylin M2L scales by alpha(n, m) / alpha(l + n, m) with l + n up to
  // 2p; 1 / (2p)! leaves the FP32 range above order 16
  if (c->flavour == ARAN_FLAVOUR_KKYLIN && c->precision == ARAN_PRECISION_MIXED && c->order > 16)
    return fail(ARAN_ERR_INVALID, "mixed-precision kkylin takes orders up to 16");
  return ARAN_OK;
}

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" {

const char *aran_gpu_last_error(void) { return g_last_error.c_str(); }

const char *aran_gpu_version(void) { return "aran-gb300 0.1 (sm_103a)"; }

int aran_gpu_solver3d_create(const AranGpuConfig3d *cfg, AranGpuSolver3d **out) {
  if (!out) return fail(ARAN_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = check_config(cfg);
  if (rc) return rc;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(ARAN_ERR_NO_DEVICE, std::string("no CUDA device available: ") + cudaGetErrorString(e));
  AranGpuSolver3d *s = new AranGpuSolver3d();
  s->cfg = *cfg;
  if (cfg->maxbox == 0) {
    // leaf capacity and M2L kernel from the autotuner's database
    AranGpuTuneResult tr;
    if (aran_gpu_tune_lookup(nullptr, cfg, &tr) == 1) {
      s->cfg.maxbox = tr.maxbox;
      s->m2l_kernel = tr.m2l_kernel;
      s->m2l_nst = tr.m2l_nst;
      s->m2l_g = tr.m2l_g;
    } else {
      s->cfg.maxbox = 64;
    }
  }
  try {
    ACHECK(cudaGetDevice(&s->device));
    ACHECK(cudaStreamCreateWithFlags(&s->s0, cudaStreamNonBlocking));
    ACHECK(cudaStreamCreateWithFlags(&s->s1, cudaStreamNonBlocking));
    for (auto &ev : s->ev) ACHECK(cudaEventCreate(&ev));
    double ext = 0;
    for (int a = 0; a < 3; ++a) ext = std::fmax(ext, cfg->ub[a] - cfg->lb[a]);
    s->scale_e = std::ldexp(1.0, (int)std::ceil(std::log2(ext)));
    if (s->scale_e < ext) s->scale_e *= 2;
    build_tables(s);
    if (cfg->flavour == ARAN_FLAVOUR_KKYLIN) build_kkylin_tables(s);
    if (cfg->precision == ARAN_PRECISION_MIXED && cfg->order >= kRootFp64Order &&
        cfg->flavour != ARAN_FLAVOUR_KKYLIN) {
      s->root64_depth = kRootFp64Depth;
      build_tables_fp64(s);
    }
    s->err_dev.reserve(4);
    ACHECK(cudaHostAlloc(&s->h_small, 16 * sizeof(int), cudaHostAllocDefault));
    ACHECK(cudaMemset(s->err_dev.ptr, 0, sizeof(int)));
  } catch (const CudaError &ce) {
    int r = from_cuda(ce);
    aran_gpu_solver3d_destroy(s);
    return r;
  }
  *out = s;
  return ARAN_OK;
}

void aran_gpu_solver3d_destroy(AranGpuSolver3d *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->s0) cudaStreamSynchronize(s->s0);
  if (s->s1) cudaStreamSynchronize(s->s1);
  if (s->h_small) cudaFreeHost(s->h_small);
  DevTree &t = s->tree;
  t.key.release(); t.ijk.release(); t.depth.release(); t.begin.release(); t.end.release();
  t.child.release(); t.parent.release(); t.center.release(); t.col.release(); t.ncol.release();
  t.lf_begin.release(); t.lf_end.release(); t.far_off.release(); t.far_src.release();
  t.far_dir.release(); t.leaf_node.release(); t.win_leaf.release(); t.near_off.release();
  t.near_rng.release();
  t.m2l_targets.release();
  for (auto *tb : {&s->t64}) {
    tb->rec.release(); tb->p2mf.release(); tb->vt.release(); tb->vm.release(); tb->vl.release();
    tb->gz.release(); tb->gm.release(); tb->dir_m2l.release(); tb->dir_m2m.release();
    tb->dir_l2l.release(); tb->dir_lanes.release(); tb->lm.release();
    tb->oct_lanes[0].release(); tb->oct_lanes[1].release();
  }
  {
    auto *tb = &s->t32;
    tb->rec.release(); tb->p2mf.release(); tb->vt.release(); tb->vm.release(); tb->vl.release();
    tb->gz.release(); tb->gm.release(); tb->dir_m2l.release(); tb->dir_m2m.release();
    tb->dir_l2l.release(); tb->dir_lanes.release(); tb->lm.release();
    tb->oct_lanes[0].release(); tb->oct_lanes[1].release();
  }
  s->keys_in.release(); s->keys_out.release(); s->idx_in.release(); s->perm.release();
  s->cub_tmp.release(); s->sx.release(); s->sy.release(); s->sz.release(); s->sq.release();
  s->rel64.release(); s->rel32.release(); s->acc_pot.release(); s->acc_fld.release();
  s->io_xyz.release(); s->io_q.release(); s->io_pot.release(); s->io_fld.release();
  s->mult64.release(); s->loc64.release(); s->mult32.release(); s->loc32.release();
  s->scan_tmp.release(); s->stats_dev.release(); s->err_dev.release();
  t.leaf_be.release(); t.leaf_chi.release(); t.leaf_clo.release(); t.big_items.release();
  t.parents.release(); t.big_rng.release(); t.sys.release();
  s->sys_off.release(); s->sys_box.release(); s->tc_tab.release(); s->tc_dvec.release();
  s->kk64.release();
  s->kk32.release();
  for (auto &ev : s->ev)
    if (ev) cudaEventDestroy(ev);
  if (s->s0) cudaStreamDestroy(s->s0);
  if (s->s1) cudaStreamDestroy(s->s1);
  delete s;
}

}  // extern "C"

namespace {

int check_systems(const AranGpuSolver3d *s, int nsys, const int64_t *offs, const double *boxes,
                  int64_t n) {
  if (nsys < 1) return fail(ARAN_ERR_INVALID, "nsys must be >= 1");
  if (!offs || !boxes) return fail(ARAN_ERR_INVALID, "offsets and boxes must not be NULL");
  if (offs[0] != 0 || offs[nsys] != n)
    return fail(ARAN_ERR_INVALID, "offsets must start at 0 and end at n");
  for (int k = 0; k < nsys; ++k) {
    if (offs[k + 1] < offs[k]) return fail(ARAN_ERR_INVALID, "offsets must be non-decreasing");
    for (int a = 0; a < 3; ++a) {
      const double lo = boxes[6 * (size_t)k + a], hi = boxes[6 * (size_t)k + 3 + a];
      if (!std::isfinite(lo) || !std::isfinite(hi) || !(hi > lo))
        return fail(ARAN_ERR_INVALID, "system " + std::to_string(k) + ": box must satisfy lb < ub (finite)");
      // the operator tables are made for the solver's box extents
      if (hi - lo != s->cfg.ub[a] - s->cfg.lb[a])
        return fail(ARAN_ERR_INVALID, "system " + std::to_string(k) +
                                          ": box extents must equal the solver's ub - lb");
    }
  }
  return ARAN_OK;
}

int solve_impl(AranGpuSolver3d *s, int nsys, const int64_t *offs, const double *boxes, int64_t n,
               const double *xyz, const double *q, double *pot, double *field, int mem) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (n < 1) return fail(ARAN_ERR_INVALID, "n must be >= 1");
  if (n > (int64_t)1 << 30) return fail(ARAN_ERR_INVALID, "n exceeds 2^30 particles");
  if (!xyz || !q) return fail(ARAN_ERR_INVALID, "xyz and q must not be NULL");
  if (mem != ARAN_MEM_HOST && mem != ARAN_MEM_DEVICE) return fail(ARAN_ERR_INVALID, "bad mem kind");
  if (field && !s->cfg.field) return fail(ARAN_ERR_INVALID, "field requested from a potential-only solver");
  if (offs) {
    int rc = check_systems(s, nsys, offs, boxes, n);
    if (rc) return rc;
  }
  try {
    ACHECK(cudaSetDevice(s->device));
    s->launches = 0;
    cudaStream_t st = s->s0;
    set_systems(s, offs ? nsys : 1, offs, boxes, n);
    const double *dx = xyz, *dq = q;
    double *dpot = pot, *dfld = field;
    ACHECK(cudaEventRecord(s->ev[2 * Stage::TOTAL], st));
    ACHECK(cudaMemsetAsync(s->err_dev.ptr, 0, sizeof(int), st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::H2D], st));
    if (mem == ARAN_MEM_HOST) {
      s->io_xyz.reserve(3 * n);
      s->io_q.reserve(n);
      ACHECK(cudaMemcpyAsync(s->io_xyz.ptr, xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, st));
      ACHECK(cudaMemcpyAsync(s->io_q.ptr, q, n * sizeof(double), cudaMemcpyHostToDevice, st));
      dx = s->io_xyz.ptr;
      dq = s->io_q.ptr;
      if (pot) { s->io_pot.reserve(n); dpot = s->io_pot.ptr; }
      if (field) { s->io_fld.reserve(3 * n); dfld = s->io_fld.ptr; }
    }
    ACHECK(cudaEventRecord(s->ev[2 * Stage::H2D + 1], st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::SORT], st));
    build_tree(s, n, dx, dq);
    ACHECK(cudaEventRecord(s->ev[2 * Stage::TREE], st));  // tree start == sort end
    build_lists(s);
    run_passes(s);
    scatter_outputs(s, dpot, dfld);
    ACHECK(cudaEventRecord(s->ev[2 * Stage::D2H], st));
    if (mem == ARAN_MEM_HOST) {
      if (pot) ACHECK(cudaMemcpyAsync(pot, dpot, n * sizeof(double), cudaMemcpyDeviceToHost, st));
      if (field) ACHECK(cudaMemcpyAsync(field, dfld, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    ACHECK(cudaEventRecord(s->ev[2 * Stage::D2H + 1], st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::TOTAL + 1], st));
    ACHECK(cudaStreamSynchronize(st));
    ACHECK(cudaStreamSynchronize(s->s1));
    ACHECK(cudaGetLastError());
    s->have_tree = true;
    {
      int derr = 0;
      ACHECK(cudaMemcpy(&derr, s->err_dev.ptr, sizeof(int), cudaMemcpyDeviceToHost));
      if (derr & kErrTimeout)
        return fail(ARAN_ERR_TIMEOUT, "a bounded device-side wait gave up (M2L table copy)");
    }
    // stage times
    auto el = [&](int a0, int a1) {
      float ms = 0;
      cudaEventElapsedTime(&ms, s->ev[a0], s->ev[a1]);
      return (double)ms;
    };
    s->ms[0] = el(2 * Stage::TOTAL, 2 * Stage::TOTAL + 1);
    s->ms[1] = el(2 * Stage::SORT, 2 * Stage::SORT + 1);
    s->ms[2] = el(2 * Stage::SORT + 1, 2 * Stage::TREE + 1);
    s->ms[3] = el(2 * Stage::TREE + 1, 2 * Stage::LISTS + 1);
    s->ms[4] = el(2 * Stage::P2M, 2 * Stage::P2M + 1);
    s->ms[5] = el(2 * Stage::M2M, 2 * Stage::M2M + 1);
    s->ms[6] = el(2 * Stage::M2L, 2 * Stage::M2L + 1);
    s->ms[7] = el(2 * Stage::L2L, 2 * Stage::L2L + 1);
    s->ms[8] = el(2 * Stage::L2P, 2 * Stage::L2P + 1);
    s->ms[9] = el(2 * Stage::P2P, 2 * Stage::P2P + 1);
    s->ms[10] = el(2 * Stage::H2D, 2 * Stage::H2D + 1);
    s->ms[11] = el(2 * Stage::D2H, 2 * Stage::D2H + 1);
    s->ms[12] = el(2 * Stage::SEMI_P2L, 2 * Stage::SEMI_P2L + 1);
    s->ms[13] = el(2 * Stage::SEMI_M2P, 2 * Stage::SEMI_M2P + 1);
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  } catch (const InputError &ie) {
    // stopped after the key pass: drain the stream, no output was written
    cudaStreamSynchronize(s->s0);
    cudaStreamSynchronize(s->s1);
    s->have_tree = false;
    return fail(ARAN_ERR_INVALID, ie.msg);
  }
  return ARAN_OK;
}

}  // namespace

extern "C" {

int aran_gpu_solver3d_solve(AranGpuSolver3d *s, int64_t n, const double *xyz, const double *q,
                            double *pot, double *field, int mem) {
  return solve_impl(s, 1, nullptr, nullptr, n, xyz, q, pot, field, mem);
}

int aran_gpu_solver3d_solve_forest(AranGpuSolver3d *s, int nsys, const int64_t *offsets,
                                   const double *boxes, const double *xyz, const double *q,
                                   double *pot, double *field, int mem) {
  if (!offsets) return fail(ARAN_ERR_INVALID, "offsets must not be NULL");
  if (nsys < 1) return fail(ARAN_ERR_INVALID, "nsys must be >= 1");
  return solve_impl(s, nsys, offsets, boxes, offsets[nsys], xyz, q, pot, field, mem);
}

int aran_gpu_solver3d_get_stats(AranGpuSolver3d *s, int64_t stats[11]) {
  if (!s || !stats) return fail(ARAN_ERR_INVALID, "NULL argument");
  if (!s->have_tree) return fail(ARAN_ERR_INVALID, "no solve has run yet");
  try {
    compute_stats(s);
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  for (int i = 0; i < 11; ++i) stats[i] = s->stats[i];
  return ARAN_OK;
}

int aran_gpu_solver3d_tree_info(AranGpuSolver3d *s, int64_t info[5]) {
  if (!s || !info) return fail(ARAN_ERR_INVALID, "NULL argument");
  if (!s->have_tree) return fail(ARAN_ERR_INVALID, "no solve has run yet");
  DevTree &t = s->tree;
  try {
    count_far_lists(s);
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  info[0] = t.nnodes;
  info[1] = t.n_far;
  // directed near leaf entries: expand the ranges
  int64_t nn = 0;
  try {
    std::vector<int> off(t.nleaves + 1), rng(2 * t.n_near_rng);
    ACHECK(cudaMemcpy(off.data(), t.near_off.ptr, off.size() * sizeof(int), cudaMemcpyDeviceToHost));
    if (t.n_near_rng)
      ACHECK(cudaMemcpy(rng.data(), t.near_rng.ptr, rng.size() * sizeof(int), cudaMemcpyDeviceToHost));
    for (int64_t r = 0; r < t.n_near_rng; ++r) nn += rng[2 * r + 1] - rng[2 * r];
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  info[2] = nn;
  info[3] = t.nleaves;
  info[4] = t.nlevels - 1;
  return ARAN_OK;
}

int aran_gpu_solver3d_tree_lists(AranGpuSolver3d *s, uint64_t *node_ids, int32_t *node_begin,
                                 int32_t *node_end, uint8_t *node_leaf, uint64_t *far_pairs,
                                 uint64_t *near_pairs, int32_t *perm) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (!s->have_tree) return fail(ARAN_ERR_INVALID, "no solve has run yet");
  DevTree &t = s->tree;
  try {
    int nn = t.nnodes;
    std::vector<uint64_t> key(nn);
    std::vector<uint8_t> dep(nn);
    std::vector<int> child(nn), beg(nn), en(nn);
    ACHECK(cudaMemcpy(key.data(), t.key.ptr, nn * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(dep.data(), t.depth.ptr, nn, cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(child.data(), t.child.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(beg.data(), t.begin.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(en.data(), t.end.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<uint64_t> id(nn);
    for (int i = 0; i < nn; ++i) id[i] = (1ull << (3 * dep[i])) | key[i];
    for (int i = 0; i < nn; ++i) {
      if (node_ids) node_ids[i] = id[i];
      if (node_begin) node_begin[i] = beg[i];
      if (node_end) node_end[i] = en[i];
      if (node_leaf) node_leaf[i] = child[i] < 0 ? 1 : 0;
    }
    if (far_pairs) {
      build_far_lists(s);
      ACHECK(cudaStreamSynchronize(s->s0));
      std::vector<int> off(nn + 1), src(t.n_far);
      ACHECK(cudaMemcpy(off.data(), t.far_off.ptr, (nn + 1) * sizeof(int), cudaMemcpyDeviceToHost));
      if (t.n_far) ACHECK(cudaMemcpy(src.data(), t.far_src.ptr, t.n_far * sizeof(int), cudaMemcpyDeviceToHost));
      for (int i = 0; i < nn; ++i)
        for (int j = off[i]; j < off[i + 1]; ++j) {
          far_pairs[2 * (size_t)j] = id[i];
          far_pairs[2 * (size_t)j + 1] = id[src[j]];
        }
    }
    if (near_pairs) {
      std::vector<int> off(t.nleaves + 1), rng(2 * t.n_near_rng + 2), ln(t.nleaves);
      ACHECK(cudaMemcpy(off.data(), t.near_off.ptr, (t.nleaves + 1) * sizeof(int), cudaMemcpyDeviceToHost));
      if (t.n_near_rng) ACHECK(cudaMemcpy(rng.data(), t.near_rng.ptr, 2 * t.n_near_rng * sizeof(int), cudaMemcpyDeviceToHost));
      ACHECK(cudaMemcpy(ln.data(), t.leaf_node.ptr, t.nleaves * sizeof(int), cudaMemcpyDeviceToHost));
      size_t w = 0;
      for (int L = 0; L < t.nleaves; ++L)
        for (int r = off[L]; r < off[L + 1]; ++r)
          for (int lf = rng[2 * r]; lf < rng[2 * r + 1]; ++lf) {
            near_pairs[2 * w] = id[ln[L]];
            near_pairs[2 * w + 1] = id[ln[lf]];
            ++w;
          }
    }
    if (perm) ACHECK(cudaMemcpy(perm, s->perm.ptr, t.n * sizeof(int), cudaMemcpyDeviceToHost));
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  return ARAN_OK;
}

int aran_gpu_solver3d_expansions(AranGpuSolver3d *s, double *mult, double *local) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (!s->have_tree) return fail(ARAN_ERR_INVALID, "no solve has run yet");
  try {
    copy_expansions(s, mult, local);
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  return ARAN_OK;
}

int aran_gpu_solver3d_timings(AranGpuSolver3d *s, double ms[16]) {
  if (!s || !ms) return fail(ARAN_ERR_INVALID, "NULL argument");
  for (int i = 0; i < 16; ++i) ms[i] = s->ms[i];
  return ARAN_OK;
}

int64_t aran_gpu_solver3d_launches(AranGpuSolver3d *s) { return s ? s->launches : -1; }

int aran_gpu_solver3d_set_leaf_predicate(AranGpuSolver3d *s, AranGpuLeafPredicate pred,
                                         void *user_data) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  s->leaf_pred = pred;
  s->leaf_pred_data = pred ? user_data : nullptr;
  return ARAN_OK;
}

int aran_gpu_solver3d_set_m2l_kernel(AranGpuSolver3d *s, int kernel, int nst, int g) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (kernel < ARAN_M2L_AUTO || kernel > ARAN_M2L_TENSOR) return fail(ARAN_ERR_INVALID, "unknown M2L kernel");
  if (nst < 0 || nst > 3 || g < 0 || g > 2 || ((nst == 0) != (g == 0)))
    return fail(ARAN_ERR_INVALID, "sibling configuration: nst in 1..3 and g in 1..2, or both 0");
  s->m2l_kernel = kernel;
  s->m2l_nst = nst;
  s->m2l_g = g;
  return ARAN_OK;
}

int aran_gpu_solver3d_set_fp64_root_depth(AranGpuSolver3d *s, int depth) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (s->cfg.precision != ARAN_PRECISION_MIXED)
    return fail(ARAN_ERR_INVALID, "FP64 root levels apply to mixed-precision solvers");
  if (depth < -1 || depth > kKeyBits) return fail(ARAN_ERR_INVALID, "depth must be in [-1, 21]");
  try {
    ACHECK(cudaSetDevice(s->device));
    if (depth >= 0 && s->cfg.flavour != ARAN_FLAVOUR_KKYLIN) build_tables_fp64(s);
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  s->root64_depth = depth;
  return ARAN_OK;
}

}  // extern "C"
