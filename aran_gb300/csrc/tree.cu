// tree.cu -- device octree and interaction lists.
//
// Replaces libvsg's VsgPRTree3d insertion (vsg_prtree3d_insert_point, called
// from aran/aransolver3d.c:972-978) and its near/far traversal
// (vsg_prtree3d_near_far_traversal_full, aran/aransolver3d.c:1189-1190) by a
// Morton-sorted, level-synchronous build:
//   1. 63-bit keys from the 21-bit quantised coordinates, radix sort;
//   2. level by level, a node with more than maxbox points (and depth below
//      the limit) gets its 8 octants, whose point ranges are found by binary
//      search in the sorted keys;
//   3. colleagues (adjacent same-depth non-empty nodes, <= 27) level by level;
//   4. far lists: non-empty children of the parent's internal colleagues that
//      are not adjacent (the M2L sources of aran/aransolver3d.c:333-354);
//   5. near lists per non-empty leaf L, as ranges of leaf ordinals (leaves
//      are numbered in Morton order, so all leaves below a node are one
//      range): every colleague of L (a leaf, or an internal node standing for
//      all leaves below it), plus the leaf colleagues of every ancestor of L
//      (a coarser leaf adjacent to an ancestor is near everything below it).
// A solve of several independent systems builds a forest the same way: each
// system's particles are sorted within its own segment and in its own box,
// level 0 holds one root per system, and since a root's only colleague is
// itself no colleague, far or near list ever joins two systems.  Each
// level's kernels then run over the nodes of all systems at once.
#include <cub/cub.cuh>

#include "internal.cuh"

namespace aran {

namespace {

// Morton keys of the particles, each in its system's box (sys_box: lb[3],
// ub[3], scale[3] per system; particles of system k are sys_off[k] ..
// sys_off[k+1]-1); a non-finite coordinate or charge sets kErrNonFinite in
// the error word (the solve then stops before any output)
__global__ void k_keys(int64_t n, const double *__restrict__ xyz, const double *__restrict__ q,
                       int nsys, const int *__restrict__ sys_off,
                       const double *__restrict__ sys_box, uint64_t *__restrict__ keys,
                       int *__restrict__ idx, int *__restrict__ err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nsys;   // the last system k with sys_off[k] <= i, in [lo, hi)
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (sys_off[mid] <= i) lo = mid; else hi = mid;
  }
  const double *b = sys_box + 9 * lo;
  const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
  if (!(isfinite(x) && isfinite(y) && isfinite(z) && isfinite(q[i]))) atomicOr(err, kErrNonFinite);
  const int64_t ix = cell_index(cell_pos(x, b[0], b[6])), iy = cell_index(cell_pos(y, b[1], b[7])),
                iz = cell_index(cell_pos(z, b[2], b[8]));
  // outside the box: the key clamps it into a boundary cell, which the FP64
  // path evaluates like the oracle, but its distance from the cell
  // overflows the scaled FP32 expansions
  if (cell_outside(ix) || cell_outside(iy) || cell_outside(iz)) atomicOr(err, kErrOutside);
  uint64_t qx = (uint64_t)cell_clamp(ix);
  uint64_t qy = (uint64_t)cell_clamp(iy);
  uint64_t qz = (uint64_t)cell_clamp(iz);
  keys[i] = spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
  idx[i] = (int)i;
}

__global__ void k_gather(int64_t n, const int *__restrict__ perm, const double *__restrict__ xyz,
                         const double *__restrict__ q, double *__restrict__ sx,
                         double *__restrict__ sy, double *__restrict__ sz,
                         double *__restrict__ sq) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  sx[i] = xyz[3 * (int64_t)o];
  sy[i] = xyz[3 * (int64_t)o + 1];
  sz[i] = xyz[3 * (int64_t)o + 2];
  sq[i] = q[o];
}

struct NodeArrays {
  uint64_t *key;
  int *ijk;
  uint8_t *depth;
  int *begin, *end, *child, *parent, *sys;
  double *center;
};

// one root per system at depth 0 (roots have no colleagues but themselves,
// so no list of the forest joins two systems)
__global__ void k_roots(NodeArrays na, int nsys, const int *__restrict__ sys_off,
                        const double *__restrict__ sys_box) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nsys) return;
  const double *b = sys_box + 9 * r;
  na.key[r] = 0;
  na.ijk[3 * r] = na.ijk[3 * r + 1] = na.ijk[3 * r + 2] = 0;
  na.depth[r] = 0;
  na.begin[r] = sys_off[r];
  na.end[r] = sys_off[r + 1];
  na.child[r] = -1;
  na.parent[r] = -1;
  na.sys[r] = r;
  na.center[3 * r] = node_center_axis(b[0], b[3], 0, 0);
  na.center[3 * r + 1] = node_center_axis(b[1], b[4], 0, 0);
  na.center[3 * r + 2] = node_center_axis(b[2], b[5], 0, 0);
}

__global__ void k_flag_internal(int cnt, int off, const int *__restrict__ begin,
                                const int *__restrict__ end, int maxbox, int d, int maxd,
                                int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int c = end[off + i] - begin[off + i];
  flags[i] = (c > maxbox && d < maxd) ? 1 : 0;
}

__device__ __forceinline__ int digit_at(const uint64_t *k, int j, int shift) {
  return (int)((k[j] >> shift) & 7ull);
}

// eight threads per node of the level, thread c making child c: its range
// ends at the first key of the parent's range whose digit at this depth
// exceeds c (one binary search per thread), and begins where child c-1 ends
// (the neighbouring lane's result)
__global__ void k_make_children(int cnt, int off, int child_off, const int *__restrict__ flags,
                                const int *__restrict__ pos, const uint64_t *__restrict__ skeys,
                                int d, NodeArrays na, const double *__restrict__ sys_box) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int i = (int)(g >> 3), c = (int)(g & 7);
  const bool live = i < cnt;
  const int node = off + (live ? i : 0);
  const bool split = live && flags[i] != 0;
  int lo = 0, b = 0;
  if (split) {
    b = na.begin[node];
    const int e = na.end[node];
    const int shift = 3 * (kKeyBits - d - 1);
    lo = b;
    int hi = e;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (digit_at(skeys, mid, shift) <= c) lo = mid + 1; else hi = mid;
    }
  }
  // the eight threads of a node are eight consecutive lanes
  const int prev = __shfl_up_sync(0xffffffffu, lo, 1, 8);
  if (!live) return;
  if (!split) {
    if (c == 0) na.child[node] = -1;
    return;
  }
  const int base = child_off + 8 * pos[i];
  if (c == 0) na.child[node] = base;
  const uint64_t pk = na.key[node];
  const int pi = na.ijk[3 * node], pj = na.ijk[3 * node + 1], pk3 = na.ijk[3 * node + 2];
  const int cn = base + c;
  const int sy = na.sys[node];
  const double *bx = sys_box + 9 * sy;
  na.key[cn] = (pk << 3) | (uint64_t)c;
  const int ci = (pi << 1) | (c & 1), cj = (pj << 1) | ((c >> 1) & 1), ck = (pk3 << 1) | ((c >> 2) & 1);
  na.ijk[3 * cn] = ci;
  na.ijk[3 * cn + 1] = cj;
  na.ijk[3 * cn + 2] = ck;
  na.depth[cn] = (uint8_t)(d + 1);
  na.begin[cn] = c == 0 ? b : prev;
  na.end[cn] = lo;
  na.child[cn] = -1;
  na.parent[cn] = node;
  na.sys[cn] = sy;
  na.center[3 * cn] = node_center_axis(bx[0], bx[3], d + 1, ci);
  na.center[3 * cn + 1] = node_center_axis(bx[1], bx[4], d + 1, cj);
  na.center[3 * cn + 2] = node_center_axis(bx[2], bx[5], d + 1, ck);
}

__device__ __forceinline__ bool adjacent(const int *ijk, int a, int b) {
  int dx = ijk[3 * a] - ijk[3 * b], dy = ijk[3 * a + 1] - ijk[3 * b + 1],
      dz = ijk[3 * a + 2] - ijk[3 * b + 2];
  return dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1;
}

__device__ __forceinline__ int ncount(const int *begin, const int *end, int a) {
  return end[a] - begin[a];
}

// colleagues of the nodes of one level, the non-empty adjacent children of
// the parent's colleagues in (colleague, child) order.  Thread per node for
// wide levels:
__global__ void k_colleagues_thread(int cnt, int off, const int *__restrict__ begin,
                                    const int *__restrict__ end, const int *__restrict__ child,
                                    const int *__restrict__ parent, const int *__restrict__ ijk,
                                    int *__restrict__ col, int *__restrict__ ncol) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int c = off + i;
  int k = 0;
  if (ncount(begin, end, c) > 0) {
    int p = parent[c];
    if (p < 0) {
      col[27 * c] = c;
      k = 1;
    } else {
      int np = ncol[p];
      for (int j = 0; j < np; ++j) {
        int q = col[27 * p + j];
        int c0 = child[q];
        if (c0 < 0) continue;
        for (int o = 0; o < 8; ++o) {
          int s = c0 + o;
          if (ncount(begin, end, s) > 0 && adjacent(ijk, c, s) && k < 27) col[27 * c + k++] = s;
        }
      }
    }
  }
  ncol[c] = k;
}

// and one warp per node for narrow levels (shorter dependent chains): lane
// j < 27 takes colleague j of the parent and keeps those of its children
// that are non-empty and adjacent; a warp prefix sum places them in order
__global__ void k_colleagues(int cnt, int off, const int *__restrict__ begin,
                             const int *__restrict__ end, const int *__restrict__ child,
                             const int *__restrict__ parent, const int *__restrict__ ijk,
                             int *__restrict__ col, int *__restrict__ ncol) {
  const int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int i = (int)(g >> 5), lane = (int)(g & 31);
  if (i >= cnt) return;               // whole warps leave together
  const int c = off + i;
  if (ncount(begin, end, c) == 0) {
    if (lane == 0) ncol[c] = 0;
    return;
  }
  const int p = parent[c];
  if (p < 0) {
    if (lane == 0) {
      col[27 * c] = c;
      ncol[c] = 1;
    }
    return;
  }
  const int np = ncol[p];
  unsigned keep = 0;                  // bit o: child o of colleague `lane` is kept
  int c0 = -1;
  if (lane < np) {
    const int q = col[27 * p + lane];
    c0 = child[q];
    if (c0 >= 0)
      for (int o = 0; o < 8; ++o) {
        const int s = c0 + o;
        if (ncount(begin, end, s) > 0 && adjacent(ijk, c, s)) keep |= 1u << o;
      }
  }
  const int mine = __popc(keep);
  int before = mine;                  // inclusive prefix over lanes
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, before, d);
    if (lane >= d) before += v;
  }
  int k = before - mine;
  for (int o = 0; o < 8; ++o)
    if ((keep >> o) & 1u) {
      if (k < 27) col[27 * c + k] = c0 + o;
      ++k;
    }
  const int total = __shfl_sync(0xffffffffu, before, 31);
  if (lane == 0) ncol[c] = total < 27 ? total : 27;
}

// M2L sources of node t (same depth, not adjacent, children of the parent's
// internal colleagues).  mode 0 counts, mode 1 writes.
__global__ void k_far(int cnt, int off, const int *__restrict__ begin, const int *__restrict__ end,
                      const int *__restrict__ child, const int *__restrict__ parent,
                      const int *__restrict__ ijk, const int *__restrict__ col,
                      const int *__restrict__ ncol, int *__restrict__ far_cnt,
                      const int *__restrict__ far_off, int *__restrict__ far_src,
                      uint16_t *__restrict__ far_dir, int mode) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int t = off + i;
  int k = 0;
  int w = mode ? far_off[t] : 0;
  if (ncount(begin, end, t) > 0) {
    int p = parent[t];
    if (p >= 0) {
      int np = ncol[p];
      for (int j = 0; j < np; ++j) {
        int q = col[27 * p + j];
        int c0 = child[q];
        if (c0 < 0) continue;
        for (int o = 0; o < 8; ++o) {
          int s = c0 + o;
          if (ncount(begin, end, s) == 0 || adjacent(ijk, t, s)) continue;
          if (mode) {
            int dx = ijk[3 * t] - ijk[3 * s], dy = ijk[3 * t + 1] - ijk[3 * s + 1],
                dz = ijk[3 * t + 2] - ijk[3 * s + 2];
            far_src[w + k] = s;
            far_dir[w + k] = (uint16_t)((dx + 3) + 7 * (dy + 3) + 49 * (dz + 3));
          }
          ++k;
        }
      }
    }
  }
  if (!mode) far_cnt[t] = k;
}

__global__ void k_mark_leaf_starts(int nn, const int *__restrict__ begin, const int *__restrict__ end,
                                   const int *__restrict__ child, int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  if (child[i] < 0 && end[i] > begin[i]) flags[begin[i]] = 1;
}

// leaf ordinal of particle 32 w, the first of window w
__global__ void k_win_leaf(int64_t nw, const int *__restrict__ incl, int *__restrict__ win_leaf) {
  const int64_t w = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (w < nw) win_leaf[w] = incl[32 * w] - 1;
}

__global__ void k_leaf_ranges(int nn, const int *__restrict__ begin, const int *__restrict__ end,
                              const int *__restrict__ child, const int *__restrict__ incl,
                              int *__restrict__ lf_begin, int *__restrict__ lf_end,
                              int *__restrict__ leaf_node) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  int b = begin[i], e = end[i];
  if (e > b) {
    lf_begin[i] = incl[b] - 1;
    lf_end[i] = incl[e - 1];
    if (child[i] < 0) leaf_node[incl[b] - 1] = i;
  } else {
    lf_begin[i] = 0;
    lf_end[i] = 0;
  }
}

// box of node y (depth >= depth of a) touches the box of node a
__device__ __forceinline__ bool adjacent_ml(const int *ijk, const uint8_t *depth, int a, int y) {
  const int sh = depth[y] - depth[a];
  for (int k = 0; k < 3; ++k) {
    long long lo = ((long long)ijk[3 * a + k] << sh) - 1;
    long long hi = (long long)(ijk[3 * a + k] + 1) << sh;
    long long v = ijk[3 * y + k];
    if (v < lo || v > hi) return false;
  }
  return true;
}

// Near ranges (and semifar nodes) of leaf ordinal L; mode 0 counts, mode 1
// writes.  With a semifar threshold T > 0 an internal colleague's subtree is
// walked: descendants touching the leaf are walked further (near when they
// are leaves), a descendant that does not touch it is a semifar node of the
// leaf when it holds more than T points and a near range otherwise; a
// coarser leaf colleague of an ancestor is near unless the shallowest node
// between that ancestor and L that does not touch it holds more than T
// points (it then reaches L through its own semifar P2L/M2P).
__global__ void k_near(int nleaves, const int *__restrict__ leaf_node, const int *__restrict__ begin,
                       const int *__restrict__ end, const int *__restrict__ child,
                       const int *__restrict__ parent, const int *__restrict__ col,
                       const int *__restrict__ ncol, const int *__restrict__ lf_begin,
                       const int *__restrict__ lf_end, const int *__restrict__ ijk,
                       const uint8_t *__restrict__ depth, int T, int *__restrict__ near_cnt,
                       const int *__restrict__ near_off, int *__restrict__ near_rng,
                       int *__restrict__ semi_cnt, const int *__restrict__ semi_off,
                       int *__restrict__ semi_node, int *__restrict__ semi_leaf,
                       int *__restrict__ big, int mode) {
  int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nleaves) return;
  int node = leaf_node[L];
  int k = 0, ks = 0;
  int w = mode ? near_off[L] : 0;
  int ws = (mode && T > 0) ? semi_off[L] : 0;
  // a range is every leaf under node q, so it holds end[q] - begin[q]
  // points; ranges above kBigRange are listed for the chunked P2P pass:
  // big[0] = chunk total, big[1] = heavy ranges, then per heavy range its
  // index and the offset of its first chunk
  auto emit = [&](int q) {
    if (mode) {
      near_rng[2 * (w + k)] = lf_begin[q];
      near_rng[2 * (w + k) + 1] = lf_end[q];
      const int c = end[q] - begin[q];
      if (c > kBigRange) {
        const int coff = atomicAdd(&big[0], (c + kBigRange - 1) / kBigRange);
        const int h = atomicAdd(&big[1], 1);
        big[2 + 2 * h] = w + k;
        big[3 + 2 * h] = coff;
      }
    }
    ++k;
  };
  int nc = ncol[node];
  for (int j = 0; j < nc; ++j) {
    int q = col[27 * node + j];
    if (T <= 0 || child[q] < 0) {
      emit(q);
      continue;
    }
    // depth-first walk of q's subtree (at most 7 pending siblings per level)
    int stk[8 * 22];
    int sp = 0;
    for (int o = 7; o >= 0; --o) stk[sp++] = child[q] + o;
    while (sp > 0) {
      int d = stk[--sp];
      if (end[d] == begin[d]) continue;
      if (adjacent_ml(ijk, depth, node, d)) {
        if (child[d] < 0) emit(d);
        else
          for (int o = 7; o >= 0; --o) stk[sp++] = child[d] + o;
      } else if (end[d] - begin[d] > T) {
        if (mode) {
          semi_node[ws + ks] = d;
          semi_leaf[ws + ks] = L;
        }
        ++ks;
      } else {
        emit(d);
      }
    }
  }
  for (int a = parent[node]; a >= 0; a = parent[a]) {
    int na = ncol[a];
    for (int j = 0; j < na; ++j) {
      int q = col[27 * a + j];
      if (child[q] >= 0 || end[q] == begin[q]) continue;
      if (T > 0) {
        int x = -1;
        for (int y = node; y != a; y = parent[y])
          if (!adjacent_ml(ijk, depth, q, y)) x = y;
        if (x >= 0 && end[x] - begin[x] > T) continue;
      }
      emit(q);
    }
  }
  if (!mode) {
    near_cnt[L] = k;
    if (T > 0) semi_cnt[L] = ks;
  }
}

__global__ void k_parent_flags(int nn, const int *__restrict__ child, const uint8_t *__restrict__ depth,
                               int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  flags[i] = (child[i] >= 0 && depth[i] >= 1) ? 1 : 0;
}

__global__ void k_parent_scatter(int nn, const int *__restrict__ flags, const int *__restrict__ pos,
                                 int *__restrict__ parents) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  if (flags[i]) parents[pos[i]] = i;
}

// relative (leaf-centred) particle coordinates for the kernels
template <typename T>
__global__ void k_relative(int64_t n, const int *__restrict__ incl, const int *__restrict__ leaf_node,
                           const double *__restrict__ center, const double *__restrict__ sx,
                           const double *__restrict__ sy, const double *__restrict__ sz,
                           const double *__restrict__ sq, real4<T> *__restrict__ rel) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int node = leaf_node[incl[i] - 1];
  real4<T> r;
  r.x = (T)(sx[i] - center[3 * node]);
  r.y = (T)(sy[i] - center[3 * node + 1]);
  r.z = (T)(sz[i] - center[3 * node + 2]);
  r.q = (T)sq[i];
  rel[i] = r;
}

template <typename T>
void exclusive_scan(AranGpuSolver3d *s, const T *in, T *out, int n, cudaStream_t st) {
  size_t bytes = 0;
  ACHECK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st));
  s->cub_tmp.reserve(bytes);
  ACHECK(cub::DeviceScan::ExclusiveSum(s->cub_tmp.ptr, bytes, in, out, n, st));
  s->launches += 2;
}

template <typename T>
void inclusive_scan(AranGpuSolver3d *s, const T *in, T *out, int64_t n, cudaStream_t st) {
  size_t bytes = 0;
  ACHECK(cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out, n, st));
  s->cub_tmp.reserve(bytes);
  ACHECK(cub::DeviceScan::InclusiveSum(s->cub_tmp.ptr, bytes, in, out, n, st));
  s->launches += 2;
}

NodeArrays arrays(DevTree &t) {
  NodeArrays na;
  na.key = t.key.ptr;
  na.ijk = t.ijk.ptr;
  na.depth = t.depth.ptr;
  na.begin = t.begin.ptr;
  na.end = t.end.ptr;
  na.child = t.child.ptr;
  na.parent = t.parent.ptr;
  na.sys = t.sys.ptr;
  na.center = t.center.ptr;
  return na;
}

void grow_nodes(DevTree &t, size_t need, size_t keep, cudaStream_t st) {
  t.key.grow_keep(need, keep, st);
  t.ijk.grow_keep(3 * need, 3 * keep, st);
  t.depth.grow_keep(need, keep, st);
  t.begin.grow_keep(need, keep, st);
  t.end.grow_keep(need, keep, st);
  t.child.grow_keep(need, keep, st);
  t.parent.grow_keep(need, keep, st);
  t.sys.grow_keep(need, keep, st);
  t.center.grow_keep(3 * need, 3 * keep, st);
}

// the nodes of one level about to be split are shown to the host leaf
// predicate; those it keeps as leaves lose their flag
void apply_leaf_predicate(AranGpuSolver3d *s, int off, int cnt, int d, int *d_flags,
                          cudaStream_t st) {
  const DevTree &t = s->tree;
  std::vector<int> fl(cnt), b(cnt), e(cnt), ijk(3 * (size_t)cnt), sy(cnt);
  ACHECK(cudaMemcpyAsync(fl.data(), d_flags, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(sy.data(), t.sys.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(b.data(), t.begin.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(e.data(), t.end.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(ijk.data(), t.ijk.ptr + 3 * (size_t)off, 3 * cnt * sizeof(int),
                         cudaMemcpyDeviceToHost, st));
  ACHECK(cudaStreamSynchronize(st));
  bool changed = false;
  for (int i = 0; i < cnt; ++i) {
    if (!fl[i]) continue;
    AranGpuNodeView v;
    const double *box = s->h_sys_box.data() + 9 * (size_t)sy[i];
    for (int a = 0; a < 3; ++a) {
      // the cell by halving the system's box, as the node centres are made
      double lo = box[a], hi = box[3 + a];
      for (int bit = d - 1; bit >= 0; --bit) {
        const double mid = (lo + hi) * 0.5;
        if ((ijk[3 * (size_t)i + a] >> bit) & 1) lo = mid;
        else hi = mid;
      }
      v.lbound[a] = lo;
      v.ubound[a] = hi;
      v.center[a] = (lo + hi) * 0.5;
    }
    v.point_count = e[i] - b[i];
    v.depth = d;
    if (s->leaf_pred(&v, s->leaf_pred_data)) {
      fl[i] = 0;
      changed = true;
    }
  }
  if (changed)
    ACHECK(cudaMemcpyAsync(d_flags, fl.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, st));
  ACHECK(cudaStreamSynchronize(st));
}

}  // namespace

void build_tree(AranGpuSolver3d *s, int64_t n, const double *d_xyz, const double *d_q) {
  cudaStream_t st = s->s0;
  const AranGpuConfig3d &c = s->cfg;
  DevTree &t = s->tree;
  t.n = n;
  const int TB = 256;
  const int nsys = s->nsys;

  s->keys_in.reserve(n);
  s->keys_out.reserve(n);
  s->idx_in.reserve(n);
  s->perm.reserve(n);
  k_keys<<<ceil_div(n, TB), TB, 0, st>>>(n, d_xyz, d_q, nsys, s->sys_off.ptr, s->sys_box.ptr,
                                          s->keys_in.ptr, s->idx_in.ptr, s->err_dev.ptr);
  s->launches++;
  // the systems are contiguous in the input: each is sorted in place
  size_t bytes = 0;
  if (nsys == 1) {
    ACHECK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, s->keys_in.ptr, s->keys_out.ptr,
                                           s->idx_in.ptr, s->perm.ptr, (int)n, 0, 3 * kKeyBits, st));
    s->cub_tmp.reserve(bytes);
    ACHECK(cub::DeviceRadixSort::SortPairs(s->cub_tmp.ptr, bytes, s->keys_in.ptr, s->keys_out.ptr,
                                           s->idx_in.ptr, s->perm.ptr, (int)n, 0, 3 * kKeyBits, st));
  } else {
    const int *ob = s->sys_off.ptr, *oe = s->sys_off.ptr + 1;
    ACHECK(cub::DeviceSegmentedRadixSort::SortPairs(nullptr, bytes, s->keys_in.ptr, s->keys_out.ptr,
                                                    s->idx_in.ptr, s->perm.ptr, (int)n, nsys,
                                                    ob, oe, 0, 3 * kKeyBits, st));
    s->cub_tmp.reserve(bytes);
    ACHECK(cub::DeviceSegmentedRadixSort::SortPairs(s->cub_tmp.ptr, bytes, s->keys_in.ptr,
                                                    s->keys_out.ptr, s->idx_in.ptr, s->perm.ptr,
                                                    (int)n, nsys, ob, oe, 0, 3 * kKeyBits, st));
  }
  s->launches += 4;
  s->sx.reserve(n);
  s->sy.reserve(n);
  s->sz.reserve(n);
  s->sq.reserve(n);
  k_gather<<<ceil_div(n, TB), TB, 0, st>>>(n, s->perm.ptr, d_xyz, d_q, s->sx.ptr, s->sy.ptr,
                                            s->sz.ptr, s->sq.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SORT + 1], st));

  // level-synchronous subdivision
  int maxd = c.max_depth > 0 ? c.max_depth : kKeyBits;
  if (maxd > kKeyBits) maxd = kKeyBits;
  size_t est = (size_t)nsys + (size_t)(8 * (n / (c.maxbox + 1) + 1) * 2 + 64);
  grow_nodes(t, est, 0, st);
  t.level_off.assign(1, 0);
  t.level_internal.clear();
  NodeArrays na = arrays(t);
  k_roots<<<ceil_div(nsys, TB), TB, 0, st>>>(na, nsys, s->sys_off.ptr, s->sys_box.ptr);
  s->launches++;
  int off = 0, cnt = nsys;
  DBuf<int> &flags = s->scan_tmp;
  int d = 0;
  int *hostbuf = s->h_small;   // pinned: the level's readbacks go together
  hostbuf[2] = 0;
  while (cnt > 0) {
    t.level_off.push_back(off + cnt);
    flags.reserve(2 * (size_t)cnt + 2);
    int *pos = flags.ptr + cnt;
    k_flag_internal<<<ceil_div(cnt, TB), TB, 0, st>>>(cnt, off, t.begin.ptr, t.end.ptr, c.maxbox,
                                                       d, maxd, flags.ptr);
    s->launches++;
    if (s->leaf_pred) apply_leaf_predicate(s, off, cnt, d, flags.ptr, st);
    exclusive_scan(s, flags.ptr, pos, cnt, st);
    ACHECK(cudaMemcpyAsync(&hostbuf[0], pos + cnt - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    ACHECK(cudaMemcpyAsync(&hostbuf[1], flags.ptr + cnt - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (d == 0) ACHECK(cudaMemcpyAsync(&hostbuf[2], s->err_dev.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    ACHECK(cudaStreamSynchronize(st));
    if (hostbuf[2] & kErrNonFinite) throw InputError{"a particle coordinate or charge is NaN or infinite"};
    if ((hostbuf[2] & kErrOutside) && c.precision == ARAN_PRECISION_MIXED)
      throw InputError{"a particle lies outside the solver's box (mixed precision needs every point "
                       "inside [lbound, ubound])"};
    int ninternal = hostbuf[0] + hostbuf[1];
    t.level_internal.push_back(ninternal);
    int child_off = off + cnt;
    size_t need = (size_t)child_off + 8 * (size_t)ninternal;
    if (need > t.key.cap) {
      grow_nodes(t, need, child_off, st);
      na = arrays(t);
    }
    k_make_children<<<ceil_div(8 * (int64_t)cnt, TB), TB, 0, st>>>(cnt, off, child_off, flags.ptr, pos,
                                                       s->keys_out.ptr, d, na, s->sys_box.ptr);
    s->launches++;
    off = child_off;
    cnt = 8 * ninternal;
    ++d;
  }
  t.nnodes = off;
  t.nlevels = d;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::TREE + 1], st));
}

// M2L pair counts per target node, scanned into far_off (n_far = their
// sum, the M2L counter).  The rotation kernels do not need them, so they are
// made when the counter, the lists or the tree summary is asked for.
void count_far_lists(AranGpuSolver3d *s) {
  DevTree &t = s->tree;
  if (t.far_counted) return;
  cudaStream_t st = s->s0;
  const int TB = 256;
  const int nn = t.nnodes;
  t.far_off.reserve(nn + 1);
  DBuf<int> &cntbuf = s->scan_tmp;
  cntbuf.reserve((size_t)nn + 1);
  k_far<<<ceil_div(nn, TB), TB, 0, st>>>(nn, 0, t.begin.ptr, t.end.ptr, t.child.ptr, t.parent.ptr,
                                          t.ijk.ptr, t.col.ptr, t.ncol.ptr, cntbuf.ptr, nullptr,
                                          nullptr, nullptr, 0);
  ACHECK(cudaGetLastError());
  s->launches++;
  ACHECK(cudaMemsetAsync(cntbuf.ptr + nn, 0, sizeof(int), st));
  exclusive_scan(s, cntbuf.ptr, t.far_off.ptr, nn + 1, st);
  int nfar = 0;
  ACHECK(cudaMemcpyAsync(&nfar, t.far_off.ptr + nn, sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaStreamSynchronize(st));
  t.n_far = nfar;
  t.far_counted = true;
}

// M2L pair lists (source node and offset code per pair, CSR over the target
// nodes)
void build_far_lists(AranGpuSolver3d *s) {
  DevTree &t = s->tree;
  if (t.far_built) return;
  count_far_lists(s);
  cudaStream_t st = s->s0;
  const int TB = 256;
  const int nn = t.nnodes;
  t.far_src.reserve(t.n_far + 1);
  t.far_dir.reserve(t.n_far + 1);
  k_far<<<ceil_div(nn, TB), TB, 0, st>>>(nn, 0, t.begin.ptr, t.end.ptr, t.child.ptr, t.parent.ptr,
                                          t.ijk.ptr, t.col.ptr, t.ncol.ptr, nullptr, t.far_off.ptr,
                                          t.far_src.ptr, t.far_dir.ptr, 1);
  ACHECK(cudaGetLastError());
  s->launches++;
  t.far_built = true;
}

void build_lists(AranGpuSolver3d *s) {
  cudaStream_t st = s->s0;
  DevTree &t = s->tree;
  const int TB = 256;
  int nn = t.nnodes;
  int64_t n = t.n;
  t.col.reserve(27 * (size_t)nn);
  t.ncol.reserve(nn);
  for (int d = 0; d < t.nlevels; ++d) {
    int off = t.level_off[d], cnt = t.level_off[d + 1] - off;
    if (cnt >= 16384)
      k_colleagues_thread<<<ceil_div(cnt, TB), TB, 0, st>>>(cnt, off, t.begin.ptr, t.end.ptr,
                                                           t.child.ptr, t.parent.ptr, t.ijk.ptr,
                                                           t.col.ptr, t.ncol.ptr);
    else
      k_colleagues<<<ceil_div(32 * (int64_t)cnt, TB), TB, 0, st>>>(cnt, off, t.begin.ptr, t.end.ptr,
                                                                 t.child.ptr, t.parent.ptr, t.ijk.ptr,
                                                                 t.col.ptr, t.ncol.ptr);
    s->launches++;
  }
  DBuf<int> &cntbuf = s->scan_tmp;
  cntbuf.reserve((size_t)nn + 1 + (size_t)n + 1);
  // M2L pairs: the lists only feed the kkylin M2L (the rotation kernels
  // find their sources from the colleague grids); otherwise counts and
  // lists are made when asked for (count_far_lists, build_far_lists)
  t.far_counted = false;
  t.far_built = false;
  if (s->cfg.flavour == ARAN_FLAVOUR_KKYLIN) build_far_lists(s);

  // leaves in Morton order
  DBuf<int> &lflags = s->idx_in;  // reuse (n ints)
  int *incl = s->keys_in.ptr ? reinterpret_cast<int *>(s->keys_in.ptr) : nullptr;  // n ints fit in n u64
  ACHECK(cudaMemsetAsync(lflags.ptr, 0, n * sizeof(int), st));
  k_mark_leaf_starts<<<ceil_div(nn, TB), TB, 0, st>>>(nn, t.begin.ptr, t.end.ptr, t.child.ptr,
                                                       lflags.ptr);
  s->launches++;
  inclusive_scan(s, lflags.ptr, incl, n, st);
  ACHECK(cudaMemcpyAsync(s->h_small + 3, incl + n - 1, sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaStreamSynchronize(st));
  const int nleaves = s->h_small[3];
  t.nleaves = nleaves;
  t.lf_begin.reserve(nn);
  t.lf_end.reserve(nn);
  t.leaf_node.reserve(nleaves + 1);
  k_leaf_ranges<<<ceil_div(nn, TB), TB, 0, st>>>(nn, t.begin.ptr, t.end.ptr, t.child.ptr, incl,
                                                  t.lf_begin.ptr, t.lf_end.ptr, t.leaf_node.ptr);
  s->launches++;
  {
    const int64_t nw = (n + 31) / 32;
    t.win_leaf.reserve(nw + 1);
    if (nw > 0) {
      k_win_leaf<<<ceil_div(nw, TB), TB, 0, st>>>(nw, incl, t.win_leaf.ptr);
      s->launches++;
    }
  }
  // relative coordinates
  if (s->cfg.precision == ARAN_PRECISION_MIXED) {
    s->rel32.reserve(n);
    k_relative<float><<<ceil_div(n, TB), TB, 0, st>>>(n, incl, t.leaf_node.ptr, t.center.ptr,
                                                       s->sx.ptr, s->sy.ptr, s->sz.ptr, s->sq.ptr,
                                                       s->rel32.ptr);
  } else {
    s->rel64.reserve(n);
    k_relative<double><<<ceil_div(n, TB), TB, 0, st>>>(n, incl, t.leaf_node.ptr, t.center.ptr,
                                                        s->sx.ptr, s->sy.ptr, s->sz.ptr, s->sq.ptr,
                                                        s->rel64.ptr);
  }
  s->launches++;
  // near ranges (and semifar nodes) per leaf
  const int T = s->cfg.semifar_threshold;
  t.near_off.reserve(nleaves + 1);
  int *semi_cnt = nullptr;
  if (T > 0) {
    t.semi_off.reserve(nleaves + 1);
    cntbuf.reserve(2 * ((size_t)nleaves + 1) + (size_t)n + 1);
    semi_cnt = cntbuf.ptr + nleaves + 1;
  }
  k_near<<<ceil_div(nleaves, TB), TB, 0, st>>>(nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                                t.child.ptr, t.parent.ptr, t.col.ptr, t.ncol.ptr,
                                                t.lf_begin.ptr, t.lf_end.ptr, t.ijk.ptr, t.depth.ptr,
                                                T, cntbuf.ptr, nullptr, nullptr, semi_cnt, nullptr,
                                                nullptr, nullptr, nullptr, 0);
  s->launches++;
  ACHECK(cudaMemsetAsync(cntbuf.ptr + nleaves, 0, sizeof(int), st));
  exclusive_scan(s, cntbuf.ptr, t.near_off.ptr, nleaves + 1, st);
  s->h_small[5] = 0;
  ACHECK(cudaMemcpyAsync(s->h_small + 4, t.near_off.ptr + nleaves, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (T > 0) {
    ACHECK(cudaMemsetAsync(semi_cnt + nleaves, 0, sizeof(int), st));
    exclusive_scan(s, semi_cnt, t.semi_off.ptr, nleaves + 1, st);
    ACHECK(cudaMemcpyAsync(s->h_small + 5, t.semi_off.ptr + nleaves, sizeof(int), cudaMemcpyDeviceToHost, st));
  }
  ACHECK(cudaStreamSynchronize(st));
  const int nrng = s->h_small[4], nsemi = s->h_small[5];
  t.n_near_rng = nrng;
  t.n_semi = nsemi;
  t.near_rng.reserve(2 * (size_t)nrng + 2);
  if (T > 0) {
    t.semi_node.reserve(nsemi + 1);
    t.semi_leaf.reserve(nsemi + 1);
  }
  // heavy-range list (k_near's write pass fills it): at most one entry per range
  t.big_rng.reserve(2 * (size_t)nrng + 2);
  ACHECK(cudaMemsetAsync(t.big_rng.ptr, 0, 2 * sizeof(int), st));
  k_near<<<ceil_div(nleaves, TB), TB, 0, st>>>(nleaves, t.leaf_node.ptr, t.begin.ptr, t.end.ptr,
                                                t.child.ptr, t.parent.ptr, t.col.ptr, t.ncol.ptr,
                                                t.lf_begin.ptr, t.lf_end.ptr, t.ijk.ptr, t.depth.ptr,
                                                T, nullptr, t.near_off.ptr, t.near_rng.ptr, nullptr,
                                                t.semi_off.ptr, t.semi_node.ptr, t.semi_leaf.ptr,
                                                t.big_rng.ptr, 1);
  s->launches++;
  // internal nodes of depth >= 1: one M2L block each (their children)
  {
    DBuf<int> &fl = s->scan_tmp;
    fl.reserve(2 * (size_t)nn + 2);
    k_parent_flags<<<ceil_div(nn, TB), TB, 0, st>>>(nn, t.child.ptr, t.depth.ptr, fl.ptr);
    s->launches++;
    ACHECK(cudaMemsetAsync(fl.ptr + nn, 0, sizeof(int), st));
    exclusive_scan(s, fl.ptr, fl.ptr + nn + 1, nn + 1, st);
    ACHECK(cudaMemcpyAsync(s->h_small + 6, fl.ptr + nn + 1 + nn, sizeof(int), cudaMemcpyDeviceToHost, st));
    ACHECK(cudaStreamSynchronize(st));
    const int np = s->h_small[6];
    t.n_parents = np;
    t.parents.reserve(np + 1);
    k_parent_scatter<<<ceil_div(nn, TB), TB, 0, st>>>(nn, fl.ptr, fl.ptr + nn + 1, t.parents.ptr);
    s->launches++;
  }
  build_p2p_work(s);
  ACHECK(cudaEventRecord(s->ev[2 * Stage::LISTS + 1], st));
}

}  // namespace aran
