// internal.cuh -- device buffers, solver state and kernel entry points shared
// by the translation units of libaran_gpu.so.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/aran_gpu.h"
#include "fmm_math.cuh"

namespace aran {

void set_error(const std::string &msg);

struct CudaError {
  cudaError_t code;
  std::string where;
};

// invalid input found on the device before any output was written
struct InputError {
  std::string msg;
};

// bits of the solver's device error word
constexpr int kErrTimeout = 1;     // a bounded mbarrier wait gave up
constexpr int kErrNonFinite = 2;   // NaN/Inf coordinate or charge
constexpr int kErrOutside = 4;     // a point outside its system's box (closed)

// sets the thread's last error and returns the status code
inline int fail(int code, const std::string &msg) {
  set_error(msg);
  return code;
}

// status code and message of a CUDA runtime failure
inline int from_cuda(const CudaError &e) {
  std::string m = std::string("CUDA error ") + cudaGetErrorName(e.code) + ": " +
                  cudaGetErrorString(e.code) + " in " + e.where;
  set_error(m);
  if (e.code == cudaErrorMemoryAllocation) return ARAN_ERR_OOM;
  if (e.code == cudaErrorNoDevice || e.code == cudaErrorInsufficientDriver) return ARAN_ERR_NO_DEVICE;
  return ARAN_ERR_CUDA;
}

#define ACHECK(call)                                                          \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess)                                                    \
      throw ::aran::CudaError{e_, std::string(#call) + " @ " + __FILE__ + ":" + \
                                      std::to_string(__LINE__)};              \
  } while (0)

// Grow-only device buffer.
template <typename T>
struct DBuf {
  T *ptr = nullptr;
  size_t cap = 0;
  void reserve(size_t n) {
    if (n <= cap) return;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    size_t c = n + n / 4 + 64;
    ACHECK(cudaMalloc(&ptr, c * sizeof(T)));
    cap = c;
  }
  // grow keeping the first `keep` elements
  void grow_keep(size_t n, size_t keep, cudaStream_t st) {
    if (n <= cap) return;
    T *old = ptr;
    size_t c = n + n / 2 + 64;
    T *np = nullptr;
    ACHECK(cudaMalloc(&np, c * sizeof(T)));
    if (old && keep) ACHECK(cudaMemcpyAsync(np, old, keep * sizeof(T), cudaMemcpyDeviceToDevice, st));
    if (old) {
      ACHECK(cudaStreamSynchronize(st));
      cudaFree(old);
    }
    ptr = np;
    cap = c;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
};

template <typename T> struct real4 { T x, y, z, q; };

// Node arrays, level-major (all nodes of depth d are contiguous).
struct DevTree {
  int64_t n = 0;
  int nnodes = 0;
  int nlevels = 0;
  int nleaves = 0;                    // non-empty leaves
  std::vector<int> level_off;        // size nlevels+1 (host)
  std::vector<int> level_internal;   // internal nodes per level (host)
  DBuf<uint64_t> key;                 // morton prefix at the node depth
  DBuf<int> ijk;                      // 3 per node
  DBuf<uint8_t> depth;
  DBuf<int> begin, end, child, parent;
  DBuf<int> sys;                      // system (tree of the forest) of the node
  DBuf<double> center;                // 3 per node
  DBuf<int> col;                      // 27 per node
  DBuf<int> ncol;
  DBuf<int> lf_begin, lf_end;         // leaf-ordinal range below the node
  DBuf<int> far_off, far_src;         // CSR over nodes
  DBuf<uint16_t> far_dir;             // offset code (dx+3)+7(dy+3)+49(dz+3)
  DBuf<int> leaf_node;                // leaf ordinal -> node
  DBuf<int> win_leaf;                 // leaf of particle 32 w (windows of 32 particles)
  DBuf<int> near_off, near_rng;       // CSR over leaves of [lf_a, lf_b) ranges (2 ints)
  DBuf<int> m2l_targets;              // nodes with non-empty far lists
  int n_m2l_targets = 0;
  DBuf<int2> leaf_be;                 // particle [begin, end) per leaf ordinal
  DBuf<float4> leaf_chi, leaf_clo;    // FP32 leaf centre split hi + lo; chi.w = close-pair r^2
  DBuf<int4> big_items;               // (leaf, lf_a, lf_b, 0): chunks of heavy near ranges
  DBuf<int> big_rng;                  // [0] chunk total, [1] range count, then heavy range indices
  DBuf<int> semi_off;                 // CSR over leaves of semifar nodes (threshold > 0)
  DBuf<int> semi_node, semi_leaf;     // per semifar pair: deep node, coarse leaf ordinal
  int n_semi = 0;
  DBuf<int> parents;                  // internal nodes of depth >= 1 (their children take M2L)
  int n_parents = 0;
  int n_big = 0;
  int64_t n_far = 0;
  bool far_counted = false;           // far_off and n_far made (count_far_lists)
  bool far_built = false;             // far_src/far_dir written (build_far_lists)
  int64_t n_near_rng = 0;
};

// Per-order operator tables (device).  Direction tables: 343 M2L offsets,
// 8 M2M octants, 8 L2L octants.
template <typename T>
struct OpTables {
  int p = -1;
  int stride_m2l = 0, stride_m2m = 0, stride_l2l = 0;
  DBuf<T> rec;      // 2*tri(p+1)
  DBuf<T> p2mf;     // p
  DBuf<T> vt;       // tri(p+1)*p   (M2L vertical, sign folded)
  DBuf<T> vm;       // tri(p)*p     (M2M vertical, 2^-l folded)
  DBuf<T> vl;       // tri(p+1)*(p+1) (L2L vertical, 2^-l folded)
  DBuf<T> gz, gm;   // gradient coefficients
  DBuf<T> dir_m2l, dir_m2m, dir_l2l;
  DBuf<T> dir_lanes; // lane-parallel M2L stream tables (FP32, m2l_lane_order)
  DBuf<float> oct_lanes[2];   // lane-parallel M2M / L2L octant-0 stream tables (FP32)
  DBuf<uint8_t> lm; // (l,m) of coefficient index, 2*tri(p+1)
};

// tables of the kkylin flavour (kkylin.cu): alpha/beta and, per direction
// (343 M2L offsets, 8 M2M and 8 L2L octants), r, cos/sin theta, cos/sin phi
// and the harmonics of the direction
template <typename T>
struct KkTables {
  int p = -1;
  DBuf<T> alpha, ialpha, beta, dirs[3];   // ialpha = 1 / alpha
  int stride[3] = {0, 0, 0};
  void release() {
    alpha.release();
    ialpha.release();
    beta.release();
    for (auto &d : dirs) d.release();
    p = -1;
  }
};

struct Stage {
  enum { TOTAL, SORT, TREE, LISTS, P2M, M2M, M2L, L2L, L2P, P2P, H2D, D2H, SEMI_P2L, SEMI_M2P,
         NSTAGE };
};

}  // namespace aran

struct AranGpuSolver3d {
  AranGpuConfig3d cfg;
  int device = 0;
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t ev[2 * aran::Stage::NSTAGE] = {};
  cudaEvent_t ev_p2p_done = nullptr, ev_lists_done = nullptr;
  double scale_e = 1.;   // 2^E >= root extent
  aran::OpTables<double> t64;
  aran::OpTables<float> t32;
  aran::KkTables<double> kk64;
  aran::KkTables<float> kk32;
  aran::DevTree tree;
  // particles (sorted)
  aran::DBuf<uint64_t> keys_in, keys_out;
  aran::DBuf<int> idx_in, perm;
  aran::DBuf<uint8_t> cub_tmp;
  aran::DBuf<double> sx, sy, sz, sq;     // sorted FP64 positions/charges
  aran::DBuf<aran::real4<double>> rel64;
  aran::DBuf<aran::real4<float>> rel32;
  aran::DBuf<double> acc_pot, acc_fld;   // sorted accumulators (FP64)
  aran::DBuf<double> io_xyz, io_q, io_pot, io_fld;  // staging for host calls
  aran::DBuf<double> mult64, loc64;
  aran::DBuf<float> mult32, loc32;
  aran::DBuf<int> scan_tmp;
  aran::DBuf<unsigned long long> stats_dev;
  aran::DBuf<int> err_dev;               // device error word (bounded waits)
  int *h_small = nullptr;                // pinned host words for the solve's small readbacks
  int64_t stats[11] = {};
  double ms[16] = {};
  int64_t launches = 0;
  bool have_tree = false;
  // mixed precision: nodes of depth <= root64_depth keep FP64 expansions
  // (M2M into them, M2L and L2L at them in FP64); -1 = none
  int root64_depth = -1;
  // host predicate keeping nodes about to be split as leaves (virtual leaves)
  AranGpuLeafPredicate leaf_pred = nullptr;
  void *leaf_pred_data = nullptr;
  // systems of the solve (a forest: one octree per system; 1 for a plain
  // solve): particle offsets (device, nsys + 1) and per system lb[3],
  // ub[3] and the key scales 2^21 / (ub - lb) (9 doubles, host and device)
  int nsys = 1;
  // M2L kernel of the FP32 part (ARAN_M2L_*) and a forced sibling
  // configuration (table slots, parents per CTA; 0 = the library's)
  int m2l_kernel = ARAN_M2L_AUTO;
  int m2l_nst = 0, m2l_g = 0;
  // dense M2L operators of the tensor-core kernel (m2l_tc.cu), made on
  // first use at order tc_p
  aran::DBuf<float> tc_tab;
  aran::DBuf<int8_t> tc_dvec;
  int tc_p = -1;
  aran::DBuf<int> sys_off;
  aran::DBuf<double> sys_box;
  std::vector<int> h_sys_off;
  std::vector<double> h_sys_box;
};

namespace aran {

// solver.cu: the tree of n host particles without lists or passes (for
// traversals of the tree); the solver's last solve results stay valid only
// if the same particles are given
void build_tree_only(AranGpuSolver3d *s, int64_t n, const double *xyz, const double *q);
// tree.cu
void build_tree(AranGpuSolver3d *s, int64_t n, const double *d_xyz, const double *d_q);
void build_lists(AranGpuSolver3d *s);
void count_far_lists(AranGpuSolver3d *s);
void build_far_lists(AranGpuSolver3d *s);
// tables.cu
void build_tables(AranGpuSolver3d *s);
void build_tables_fp64(AranGpuSolver3d *s);   // FP64 tables beside a mixed solver's FP32 ones
// offset of part `what` (0 ef, 1 of, 2 ei, 3 oi, 4 ph, 5 rp, 6 stride, 7 vv) in
// a direction table of kind 0 (M2L), 1 (M2M) or 2 (L2L) at order p
int dir_offset(int p, int kind, int what);
// passes.cu
void run_passes(AranGpuSolver3d *s);
// kkylin.cu: stage 0 = M2M, 1 = M2L, 2 = L2L
void build_kkylin_tables(AranGpuSolver3d *s);
void kkylin_pass(AranGpuSolver3d *s, int stage);
// m2l.cu: M2L into the children of parents[first, first + count), in FP64
// (mult64/loc64) or FP32 (mult32/loc32)
void launch_m2l(AranGpuSolver3d *s, bool fp64, int first, int count, cudaStream_t st);
bool launch_m2l_lanes(AranGpuSolver3d *s, OpTables<float> &tb, const int *parents, int count,
                      const cplx<float> *mult, cplx<float> *loc, cudaStream_t st);
// m2m_lanes.cu: lane-parallel FP32 M2M (parents of depths dhi down to dlo)
// and L2L (children of depths dlo up to dhi, from depth 3) at the orders
// m2l_lane_order accepts; false leaves the pass to passes.cu's kernels
void build_oct_lane_tables(OpTables<float> &tb, cudaStream_t st);
bool launch_m2m_lanes(AranGpuSolver3d *s, OpTables<float> &tb, cplx<float> *mult, int dhi,
                      int dlo, cudaStream_t st);
bool launch_l2l_lanes(AranGpuSolver3d *s, OpTables<float> &tb, cplx<float> *loc, int dlo,
                      int dhi, cudaStream_t st);
// m2l_tc.cu: the FP32 M2L on the tensor cores (orders 8 and 12); false
// leaves it to the other kernels
bool launch_m2l_tc(AranGpuSolver3d *s, const int *parents, int count, const float *mult,
                   float *loc, cudaStream_t st);
// p2p.cu
constexpr int kBigRange = 2048;   // near ranges above this many particles are chunked
void build_p2p_work(AranGpuSolver3d *s);
void launch_p2p(AranGpuSolver3d *s, cudaStream_t st);
void compute_stats(AranGpuSolver3d *s);
// semifar.cu: P2L of coarse-leaf points into semifar nodes' locals (before
// L2L) and M2P of those nodes' multipoles to the points (after L2P)
void launch_semifar_p2l(AranGpuSolver3d *s, cudaStream_t st);
void launch_semifar_m2p(AranGpuSolver3d *s, cudaStream_t st);
void copy_expansions(AranGpuSolver3d *s, double *mult, double *local);

inline int ceil_div(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

// solver2d.cu: a 2D solve, or only its forest (tree_only, acc unused); and a
// host copy of the last forest (node arrays, permutation, per-node Laurent
// multipole/local coefficients of the last solve as interleaved complex FP64)
struct Forest2dHost {
  int p = 0, nnodes = 0;
  std::vector<int> begin, end, child, parent, sys, ij, perm;
  std::vector<uint8_t> depth;
  std::vector<double> center, sysbox, mult, loc;
};
int solve2d_impl(AranGpuSolver2d *s, int nsys, const int64_t *offs, const double *box,
                 const double *xy, const double *q, double *acc, int mem, bool tree_only);
int forest2d_to_host(AranGpuSolver2d *s, Forest2dHost &h, bool expansions);

// m2l.cu: the M2L kernel a solve of s uses (the solver's setting, else
// $ARAN_M2L_KERNEL, else ARAN_M2L_AUTO)
int m2l_kernel_choice(const AranGpuSolver3d *s);
// the sibling configurations (table slots, parents per CTA) that serve
// order p: count, and the k-th
int m2l_sibling_configs(int p, int *nst, int *g, int k);

// poll limit of the M2L consumers' waits for a table copy: 2^20, or the
// value of ARAN_DEBUG_WAIT_POLLS (a test sets it to 0 to make the wait give
// up; copies already issued are still waited for with the full limit)
int consumer_wait_polls();

// raises a kernel's dynamic shared-memory limit on the current device to at
// least `bytes` and never lowers it: solvers of different orders on other
// threads launch the same kernel with their own sizes at the same time
void smem_raise(const void *kernel, size_t bytes);
// lets a kernel use more than the default 48 KB of dynamic shared memory
template <typename K>
void smem_opt_in(K kernel, size_t bytes) {
  if (bytes > 48 * 1024) smem_raise(reinterpret_cast<const void *>(kernel), bytes);
}

}  // namespace aran
