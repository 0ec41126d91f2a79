// solver2d.cu -- the 2D Cauchy-kernel FMM of LibAran on the GPU, for a
// batch of independent systems solved in one pass (a forest).
//
// Reference: aran_solver2d_solve (aran/aransolver2d.c:1137-1204) driving
// aran_development2d_{p2m,m2m,m2l,l2l,local_evaluate}
// (aran/arandevelopment2d.c:167-346) over libvsg's quadtree, with the P2P
// kernel of tests/dummypot.c:62-76 (acc_i += q_j / (z_i - z_j)).
//
// Layout.  Particles are sorted by a 64-bit key (system id << 42 | 2x21-bit
// Morton code of the coordinates quantised in the system's box), so every
// system is one contiguous range and every quadtree node one sub-range.
// Nodes are level-major over the whole forest: level 0 holds one root per
// system.  Expansions are FP64 complex, p + 1 terms per node:
//   multipole  mult[k] = coefficient of z^{-k} (k = 1..p; k = 0 is the
//              constant term the reference keeps and never fills),
//   local      loc[k]  = coefficient of z^k (k = 0..p).
// The operators restate the reference's loops (aranlaurentseriesd.c:47-73,
// 358-452): M2M and L2L are Horner sums with Pascal-triangle binomials, M2L
// is the Laurent -> Taylor re-expansion, with one warp per node and one lane
// per output term.  The tree contract is the 3D one with 4 children: a node
// with more than maxbox points below the depth limit gets all 4 quadrants;
// same-depth non-adjacent children of adjacent nodes are far; adjacent
// leaves, and a leaf against all leaves below an adjacent internal node,
// are near.
#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.cuh"

namespace aran {
namespace {

constexpr int kMaxOrder2d = 64;
constexpr int kSysShift = 42;   // 2 x 21 Morton bits below the system id

FMM_HD uint64_t spread2(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 16)) & 0x0000ffff0000ffffull;
  v = (v | (v << 8)) & 0x00ff00ff00ff00ffull;
  v = (v | (v << 4)) & 0x0f0f0f0f0f0f0f0full;
  v = (v | (v << 2)) & 0x3333333333333333ull;
  v = (v | (v << 1)) & 0x5555555555555555ull;
  return v;
}

typedef cplx<double> zd;

__device__ __forceinline__ zd zmul(zd a, zd b) { return cmul(a, b); }
__device__ __forceinline__ zd zscale(zd a, double s) { return cmake(a.re * s, a.im * s); }
__device__ __forceinline__ zd zinv(zd a) {
  double r2 = a.re * a.re + a.im * a.im;
  double w = 1.0 / r2;
  return cmake(a.re * w, -a.im * w);
}
// a^e by binary exponentiation
__device__ __forceinline__ zd zpow(zd a, int e) {
  zd r = cmake(1.0, 0.0);
  while (e) {
    if (e & 1) r = zmul(r, a);
    a = zmul(a, a);
    e >>= 1;
  }
  return r;
}

__device__ __forceinline__ double shfl_sum(double v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------- keys/sort
// per system: lbx, lby, ubx, uby, scale x, scale y
// a non-finite coordinate or charge sets kErrNonFinite in *err, a point
// outside its system's closed box kErrOutside (its key is clamped into a
// boundary cell)
__global__ void k2_keys(int64_t n, int nsys, const int64_t *__restrict__ offs,
                        const double *__restrict__ sysbox, const double *__restrict__ xy,
                        const double *__restrict__ q, uint64_t *__restrict__ keys,
                        int *__restrict__ idx, int *__restrict__ err) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  // last system s with offs[s] <= i
  int lo = 0, hi = nsys;  // answer in [lo, hi)
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (offs[mid] <= i) lo = mid; else hi = mid;
  }
  const double *b = sysbox + 6 * lo;
  const double x = xy[2 * i], y = xy[2 * i + 1];
  if (!(isfinite(x) && isfinite(y) && isfinite(q[i]))) atomicOr(err, kErrNonFinite);
  const int64_t ix = cell_index(cell_pos(x, b[0], b[4])), iy = cell_index(cell_pos(y, b[1], b[5]));
  if (cell_outside(ix) || cell_outside(iy)) atomicOr(err, kErrOutside);
  uint64_t qx = (uint64_t)cell_clamp(ix);
  uint64_t qy = (uint64_t)cell_clamp(iy);
  keys[i] = ((uint64_t)lo << kSysShift) | spread2(qx) | (spread2(qy) << 1);
  idx[i] = (int)i;
}

__global__ void k2_gather(int64_t n, const int *__restrict__ perm, const double *__restrict__ xy,
                          const double *__restrict__ q, double *__restrict__ sx,
                          double *__restrict__ sy, double *__restrict__ sq) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int o = perm[i];
  sx[i] = xy[2 * (int64_t)o];
  sy[i] = xy[2 * (int64_t)o + 1];
  sq[i] = q[o];
}

// ---------------------------------------------------------------- quadtree
struct Nodes2 {
  int *sys, *ij, *begin, *end, *child, *parent;
  uint8_t *depth;
  double *center;
};

__global__ void k2_roots(int nsys, const int64_t *__restrict__ offs, const double *__restrict__ sysbox,
                         Nodes2 na) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const double *b = sysbox + 6 * s;
  na.sys[s] = s;
  na.ij[2 * s] = na.ij[2 * s + 1] = 0;
  na.depth[s] = 0;
  na.begin[s] = (int)offs[s];
  na.end[s] = (int)offs[s + 1];
  na.child[s] = -1;
  na.parent[s] = -1;
  na.center[2 * s] = node_center_axis(b[0], b[2], 0, 0);
  na.center[2 * s + 1] = node_center_axis(b[1], b[3], 0, 0);
}

__global__ void k2_flag(int cnt, int off, const int *__restrict__ begin, const int *__restrict__ end,
                        int maxbox, int d, int maxd, int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int c = end[off + i] - begin[off + i];
  flags[i] = (c > maxbox && d < maxd) ? 1 : 0;
}

__global__ void k2_children(int cnt, int off, int child_off, const int *__restrict__ flags,
                            const int *__restrict__ pos, const uint64_t *__restrict__ skeys, int d,
                            Nodes2 na, const double *__restrict__ sysbox) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int node = off + i;
  if (!flags[i]) {
    na.child[node] = -1;
    return;
  }
  int base = child_off + 4 * pos[i];
  na.child[node] = base;
  int b = na.begin[node], e = na.end[node];
  int shift = 2 * (kKeyBits - d - 1);
  int s = na.sys[node];
  const double *bx = sysbox + 6 * s;
  int pi = na.ij[2 * node], pj = na.ij[2 * node + 1];
  int start = b;
  for (int c = 0; c < 4; ++c) {
    int lo = start, hi = e;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if ((int)((skeys[mid] >> shift) & 3ull) <= c) lo = mid + 1; else hi = mid;
    }
    int cn = base + c;
    int ci = (pi << 1) | (c & 1), cj = (pj << 1) | ((c >> 1) & 1);
    na.sys[cn] = s;
    na.ij[2 * cn] = ci;
    na.ij[2 * cn + 1] = cj;
    na.depth[cn] = (uint8_t)(d + 1);
    na.begin[cn] = start;
    na.end[cn] = lo;
    na.child[cn] = -1;
    na.parent[cn] = node;
    na.center[2 * cn] = node_center_axis(bx[0], bx[2], d + 1, ci);
    na.center[2 * cn + 1] = node_center_axis(bx[1], bx[3], d + 1, cj);
    start = lo;
  }
}

__device__ __forceinline__ bool adj2(const int *ij, int a, int b) {
  int dx = ij[2 * a] - ij[2 * b], dy = ij[2 * a + 1] - ij[2 * b + 1];
  return dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1;
}

__global__ void k2_colleagues(int cnt, int off, const int *__restrict__ begin,
                              const int *__restrict__ end, const int *__restrict__ child,
                              const int *__restrict__ parent, const int *__restrict__ ij,
                              int *__restrict__ col, int *__restrict__ ncol) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cnt) return;
  int c = off + i;
  int k = 0;
  if (end[c] > begin[c]) {
    int p = parent[c];
    if (p < 0) {
      col[9 * c] = c;
      k = 1;
    } else {
      for (int j = 0; j < ncol[p]; ++j) {
        int c0 = child[col[9 * p + j]];
        if (c0 < 0) continue;
        for (int o = 0; o < 4; ++o) {
          int s = c0 + o;
          if (end[s] > begin[s] && adj2(ij, c, s) && k < 9) col[9 * c + k++] = s;
        }
      }
    }
  }
  ncol[c] = k;
}

// far sources of node t; mode 0 counts, mode 1 writes
__global__ void k2_far(int nn, const int *__restrict__ begin, const int *__restrict__ end,
                       const int *__restrict__ child, const int *__restrict__ parent,
                       const int *__restrict__ ij, const int *__restrict__ col,
                       const int *__restrict__ ncol, int *__restrict__ far_cnt,
                       const int *__restrict__ far_off, int *__restrict__ far_src, int mode) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nn) return;
  int k = 0;
  int w = mode ? far_off[t] : 0;
  int p = parent[t];
  if (end[t] > begin[t] && p >= 0) {
    for (int j = 0; j < ncol[p]; ++j) {
      int c0 = child[col[9 * p + j]];
      if (c0 < 0) continue;
      for (int o = 0; o < 4; ++o) {
        int s = c0 + o;
        if (end[s] == begin[s] || adj2(ij, t, s)) continue;
        if (mode) far_src[w + k] = s;
        ++k;
      }
    }
  }
  if (!mode) far_cnt[t] = k;
}

__global__ void k2_leaf_starts(int nn, const int *__restrict__ begin, const int *__restrict__ end,
                               const int *__restrict__ child, int *__restrict__ flags) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  if (child[i] < 0 && end[i] > begin[i]) flags[begin[i]] = 1;
}

__global__ void k2_leaf_ranges(int nn, const int *__restrict__ begin, const int *__restrict__ end,
                               const int *__restrict__ child, const int *__restrict__ incl,
                               int *__restrict__ lf_begin, int *__restrict__ lf_end,
                               int *__restrict__ leaf_node, int *__restrict__ leaf_be) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nn) return;
  int b = begin[i], e = end[i];
  if (e > b) {
    lf_begin[i] = incl[b] - 1;
    lf_end[i] = incl[e - 1];
    if (child[i] < 0) {
      leaf_node[incl[b] - 1] = i;
      leaf_be[incl[b] - 1] = b;
    }
  } else {
    lf_begin[i] = lf_end[i] = 0;
  }
}

// near leaf-ordinal ranges of leaf L; mode 0 counts, mode 1 writes
__global__ void k2_near(int nleaves, const int *__restrict__ leaf_node, const int *__restrict__ begin,
                        const int *__restrict__ end, const int *__restrict__ child,
                        const int *__restrict__ parent, const int *__restrict__ col,
                        const int *__restrict__ ncol, const int *__restrict__ lf_begin,
                        const int *__restrict__ lf_end, int *__restrict__ near_cnt,
                        const int *__restrict__ near_off, int2 *__restrict__ near_rng, int mode) {
  int L = blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nleaves) return;
  int node = leaf_node[L];
  int k = 0;
  int w = mode ? near_off[L] : 0;
  for (int j = 0; j < ncol[node]; ++j) {
    int q = col[9 * node + j];
    if (mode) near_rng[w + k] = make_int2(lf_begin[q], lf_end[q]);
    ++k;
  }
  for (int a = parent[node]; a >= 0; a = parent[a]) {
    for (int j = 0; j < ncol[a]; ++j) {
      int q = col[9 * a + j];
      if (child[q] >= 0 || end[q] == begin[q]) continue;
      if (mode) near_rng[w + k] = make_int2(lf_begin[q], lf_end[q]);
      ++k;
    }
  }
  if (!mode) near_cnt[L] = k;
}

// ------------------------------------------------------------------ passes
// P2M: a_{-i} += q (z - zc)^{i-1}, i = 1..p-1 (arandevelopment2d.c:167-189);
// one warp per leaf, lanes over particles, warp sums per term.
__global__ void k2_p2m(int nleaves, int p, const int *__restrict__ leaf_node,
                       const int *__restrict__ begin, const int *__restrict__ end,
                       const double *__restrict__ center, const double *__restrict__ sx,
                       const double *__restrict__ sy, const double *__restrict__ sq,
                       zd *__restrict__ mult) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nleaves) return;
  int node = leaf_node[warp];
  int b = begin[node], e = end[node];
  double cx = center[2 * node], cy = center[2 * node + 1];
  zd acc[3];
  for (int k = 0; k < 3; ++k) acc[k] = cmake(0.0, 0.0);
  for (int base = b; base < e; base += 32) {
    int i = base + lane;
    zd d = cmake(0.0, 0.0), tmp = cmake(0.0, 0.0);
    if (i < e) {
      d = cmake(sx[i] - cx, sy[i] - cy);
      tmp = cmake(sq[i], 0.0);
    }
    for (int t = 1; t < p; ++t) {
      double re = shfl_sum(tmp.re), im = shfl_sum(tmp.im);
      if ((t & 31) == lane) {
        zd v = cmake(re, im);
        // constant register indices (no local-memory array)
        if (t < 32) acc[0] = cadd(acc[0], v);
        else if (t < 64) acc[1] = cadd(acc[1], v);
        else acc[2] = cadd(acc[2], v);
      }
      tmp = zmul(tmp, d);
    }
  }
  const int P1 = p + 1;
  for (int k = 0; k < 3; ++k) {
    int t = lane + 32 * k;
    if (t <= p) mult[(int64_t)node * P1 + t] = acc[k];
  }
}

// M2M, one level: warp per node of the level; the children's multipoles
// re-expanded at the node (aran_laurent_seriesd_translate, negative part:
// b_{-i} += sum_{j<i} C(i-1, j-1) a_{-j} (zs - zd)^{i-j} + a_{-i}).
__global__ void k2_m2m(int cnt, int off, int p, const int *__restrict__ child,
                       const int *__restrict__ begin, const int *__restrict__ end,
                       const double *__restrict__ center, const double *__restrict__ binom, int nb,
                       zd *__restrict__ mult) {
  __shared__ zd sm[4][kMaxOrder2d + 1];
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int k = blockIdx.x * (blockDim.x >> 5) + wl;
  int node = off + k;
  bool active = k < cnt && child[node] >= 0;
  const int P1 = p + 1;
  zd acc[3];
  for (int s = 0; s < 3; ++s) acc[s] = cmake(0.0, 0.0);
  if (active) {
    int c0 = child[node];
    double px = center[2 * node], py = center[2 * node + 1];
    for (int c = c0; c < c0 + 4; ++c) {
      if (end[c] == begin[c]) continue;
      __syncwarp();
      for (int t = lane; t <= p; t += 32) sm[wl][t] = mult[(int64_t)c * P1 + t];
      __syncwarp();
      zd z0 = cmake(center[2 * c] - px, center[2 * c + 1] - py);
      for (int s = 0; s < 3; ++s) {
        int i = lane + 32 * s;
        if (i > p) break;
        if (i == 0) {
          acc[s] = cadd(acc[s], sm[wl][0]);
          continue;
        }
        zd sum = cmake(0.0, 0.0);
        for (int j = 1; j < i; ++j) {
          double bc = binom[(i - 1) * nb + (j - 1)];
          sum = zmul(cadd(sum, zscale(sm[wl][j], bc)), z0);
        }
        acc[s] = cadd(acc[s], cadd(sum, sm[wl][i]));
      }
    }
    for (int s = 0; s < 3; ++s) {
      int i = lane + 32 * s;
      if (i <= p) mult[(int64_t)node * P1 + i] = acc[s];
    }
  }
}

// M2L: warp per target node, lanes per local term i:
// L_i += (-1/z)^i sum_{j=1}^{p-1} C(i+j-1, j-1) a_{-j} z^{-j}, z = zt - zs
// (aran_laurent_seriesd_to_taylor, aranlaurentseriesd.c:409-452).
__global__ void __launch_bounds__(128) k2_m2l(int nn, int p, const int *__restrict__ far_off,
                                              const int *__restrict__ far_src,
                                              const double *__restrict__ center,
                                              const double *__restrict__ binom, int nb,
                                              const zd *__restrict__ mult, zd *__restrict__ loc) {
  extern __shared__ double smem[];
  const int P1 = p + 1;
  const int SP = p | 1;                  // odd row stride: conflict-free lanes
  double *tab = smem;                    // tab[i * SP + j] = C(i+j-1, j-1)
  zd *src = reinterpret_cast<zd *>(smem + P1 * SP);
  for (int x = threadIdx.x; x < P1 * SP; x += blockDim.x) {
    int i = x / SP, j = x % SP;
    tab[x] = (j >= 1 && j < p) ? binom[(i + j - 1) * nb + (j - 1)] : 0.0;
  }
  __syncthreads();
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int t = blockIdx.x * (blockDim.x >> 5) + wl;
  if (t >= nn) return;
  int f0 = far_off[t], f1 = far_off[t + 1];
  if (f0 == f1) return;
  zd *ms = src + wl * P1;
  double tx = center[2 * t], ty = center[2 * t + 1];
  zd acc[3];
  for (int s = 0; s < 3; ++s) acc[s] = cmake(0.0, 0.0);
  for (int f = f0; f < f1; ++f) {
    int sn = far_src[f];
    __syncwarp();
    for (int k = lane; k <= p; k += 32) ms[k] = mult[(int64_t)sn * P1 + k];
    __syncwarp();
    zd inv = zinv(cmake(tx - center[2 * sn], ty - center[2 * sn + 1]));
    zd ninv = cmake(-inv.re, -inv.im);
    for (int s = 0; s < 3; ++s) {
      int i = lane + 32 * s;
      if (i > p) break;
      const double *row = tab + i * SP;
      zd sum = cmake(0.0, 0.0);
      for (int j = p - 1; j >= 1; --j) sum = zmul(cadd(sum, zscale(ms[j], row[j])), inv);
      acc[s] = cadd(acc[s], zmul(sum, zpow(ninv, i)));
    }
  }
  for (int s = 0; s < 3; ++s) {
    int i = lane + 32 * s;
    if (i <= p) {
      zd *o = loc + (int64_t)t * P1 + i;
      *o = cadd(*o, acc[s]);
    }
  }
}

// L2L, one level: warp per node of the level (depth >= 1); the parent local
// re-expanded at the node (aran_taylor_translate: b_i += sum_{j>=i}
// C(j, i) a_j z^{j-i}, Horner from a_p, z = zchild - zparent).
__global__ void k2_l2l(int cnt, int off, int p, const int *__restrict__ parent,
                       const int *__restrict__ begin, const int *__restrict__ end,
                       const double *__restrict__ center, const double *__restrict__ binom, int nb,
                       zd *__restrict__ loc) {
  __shared__ zd sm[4][kMaxOrder2d + 1];
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int k = blockIdx.x * (blockDim.x >> 5) + wl;
  if (k >= cnt) return;
  int node = off + k;
  int par = parent[node];
  if (par < 0 || end[node] == begin[node]) return;
  const int P1 = p + 1;
  for (int t = lane; t <= p; t += 32) sm[wl][t] = loc[(int64_t)par * P1 + t];
  __syncwarp();
  zd z = cmake(center[2 * node] - center[2 * par], center[2 * node + 1] - center[2 * par + 1]);
  for (int s = 0; s < 3; ++s) {
    int i = lane + 32 * s;
    if (i > p) break;
    zd sum = sm[wl][p];
    for (int j = p - 1; j >= i; --j) sum = cadd(zmul(sum, z), zscale(sm[wl][j], binom[j * nb + i]));
    zd *o = loc + (int64_t)node * P1 + i;
    *o = cadd(*o, sum);
  }
}

// P2P: warp per leaf, lanes over targets; every source of the near ranges
// (tests/dummypot.c:62-76, both directions covered by the symmetric lists).
__global__ void k2_p2p(int nleaves, const int *__restrict__ leaf_be, const int *__restrict__ near_off,
                       const int2 *__restrict__ near_rng, const double *__restrict__ sx,
                       const double *__restrict__ sy, const double *__restrict__ sq,
                       zd *__restrict__ near_acc) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nleaves) return;
  int b = leaf_be[warp], e = leaf_be[warp + 1];
  int r0 = near_off[warp], r1 = near_off[warp + 1];
  for (int base = b; base < e; base += 32) {
    int i = base + lane;
    bool on = i < e;
    double xi = on ? sx[i] : 0.0, yi = on ? sy[i] : 0.0;
    double re = 0.0, im = 0.0;
    for (int r = r0; r < r1; ++r) {
      int2 rg = near_rng[r];
      int j0 = leaf_be[rg.x], j1 = leaf_be[rg.y];
      for (int j = j0; j < j1; ++j) {
        double dx = xi - sx[j], dy = yi - sy[j];
        double r2 = dx * dx + dy * dy;
        if (!on || j == i) continue;
        double w = sq[j] * __drcp_rn(r2);
        re += dx * w;
        im -= dy * w;
      }
    }
    if (on) near_acc[i] = cmake(re, im);
  }
}

// L2P + near field + unsort: acc[perm[i]] = L(z_i - zc) + near_i
// (aran_laurent_seriesd_evaluate, aranlaurentseriesd.c:311-347, Horner)
__global__ void k2_l2p(int64_t n, int p, const int *__restrict__ incl, const int *__restrict__ leaf_node,
                       const double *__restrict__ center, const double *__restrict__ sx,
                       const double *__restrict__ sy, const zd *__restrict__ loc,
                       const zd *__restrict__ near_acc, const int *__restrict__ perm,
                       double *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int node = leaf_node[incl[i] - 1];
  const zd *a = loc + (int64_t)node * (p + 1);
  zd z = cmake(sx[i] - center[2 * node], sy[i] - center[2 * node + 1]);
  zd v = a[p];
  for (int k = p - 1; k >= 0; --k) v = cadd(zmul(v, z), a[k]);
  v = cadd(v, near_acc[i]);
  int o = perm[i];
  out[2 * (int64_t)o] = v.re;
  out[2 * (int64_t)o + 1] = v.im;
}

// ------------------------------------------------- mixed precision passes
// FP32 expansions scaled by the node size h (the larger side of the
// system's box / 2^depth): multipole ma_k = a_{-k} / h^{k-1}, local
// la_k = b_k h^k, so every operator works on O(1) numbers whatever the
// depth; centres, node sizes and the near-field differences stay FP64 and
// every particle's sum is FP64.  The operators are those of the FP64 kernels
// above with z/h in place of z (rho = h_child / h_parent = 1/2):
//   M2M  mb_i = sum_{j<i} C(i-1, j-1) rho^{j-1} ma_j u^{i-j} + rho^{i-1} ma_i,
//        u = (z_child - z_parent) / h_parent;
//   M2L  la_i = (1/h) (-w)^i sum_j C(i+j-1, j-1) ma_j w^j, w = h / (zt - zs);
//   L2L  lc_i = rho^i sum_{j>=i} C(j, i) lb_j u^{j-i};
//   L2P  sum_k la_k ((z - zc) / h)^k;  P2M  ma_k = sum q ((z - zc) / h)^{k-1}.
typedef cplx<float> zf;

__device__ __forceinline__ double node_size2(const double *__restrict__ sysbox, int sys, int depth) {
  const double *b = sysbox + 6 * sys;
  return fmax(b[2] - b[0], b[3] - b[1]) * ldexp(1.0, -depth);
}

__device__ __forceinline__ float shfl_sumf(float v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ zf zfmul(zf a, zf b) {
  return cmake(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}

__global__ void k2f_p2m(int nleaves, int p, const int *__restrict__ leaf_node,
                        const int *__restrict__ begin, const int *__restrict__ end,
                        const int *__restrict__ sysn, const uint8_t *__restrict__ depth,
                        const double *__restrict__ sysbox, const double *__restrict__ center,
                        const double *__restrict__ sx, const double *__restrict__ sy,
                        const double *__restrict__ sq, zf *__restrict__ mult) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nleaves) return;
  int node = leaf_node[warp];
  int b = begin[node], e = end[node];
  const double cx = center[2 * node], cy = center[2 * node + 1];
  const double ih = 1.0 / node_size2(sysbox, sysn[node], depth[node]);
  zf acc[3];
  for (int k = 0; k < 3; ++k) acc[k] = cmake(0.f, 0.f);
  for (int base = b; base < e; base += 32) {
    int i = base + lane;
    zf d = cmake(0.f, 0.f), tmp = cmake(0.f, 0.f);
    if (i < e) {
      d = cmake((float)((sx[i] - cx) * ih), (float)((sy[i] - cy) * ih));
      tmp = cmake((float)sq[i], 0.f);
    }
    for (int t = 1; t < p; ++t) {
      float re = shfl_sumf(tmp.re), im = shfl_sumf(tmp.im);
      if ((t & 31) == lane) {
        zf v = cmake(re, im);
        if (t < 32) acc[0] = cadd(acc[0], v);
        else if (t < 64) acc[1] = cadd(acc[1], v);
        else acc[2] = cadd(acc[2], v);
      }
      tmp = zfmul(tmp, d);
    }
  }
  const int P1 = p + 1;
  for (int k = 0; k < 3; ++k) {
    int t = lane + 32 * k;
    if (t <= p) mult[(int64_t)node * P1 + t] = acc[k];
  }
}

__global__ void k2f_m2m(int cnt, int off, int p, const int *__restrict__ child,
                        const int *__restrict__ begin, const int *__restrict__ end,
                        const int *__restrict__ sysn, const uint8_t *__restrict__ depth,
                        const double *__restrict__ sysbox, const double *__restrict__ center,
                        const float *__restrict__ binom, int nb, zf *__restrict__ mult) {
  __shared__ zf sm[4][kMaxOrder2d + 1];
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int k = blockIdx.x * (blockDim.x >> 5) + wl;
  int node = off + k;
  bool active = k < cnt && child[node] >= 0;
  const int P1 = p + 1;
  zf acc[3];
  for (int s = 0; s < 3; ++s) acc[s] = cmake(0.f, 0.f);
  if (active) {
    int c0 = child[node];
    const double px = center[2 * node], py = center[2 * node + 1];
    const double ih = 1.0 / node_size2(sysbox, sysn[node], depth[node]);
    for (int c = c0; c < c0 + 4; ++c) {
      if (end[c] == begin[c]) continue;
      __syncwarp();
      // rho^{t-1} ma_t, rho = 1/2
      for (int t = lane; t <= p; t += 32) {
        const zf v = mult[(int64_t)c * P1 + t];
        const float r = t >= 1 ? ldexpf(1.f, 1 - t) : 1.f;
        sm[wl][t] = cmake(v.re * r, v.im * r);
      }
      __syncwarp();
      const zf u = cmake((float)((center[2 * c] - px) * ih), (float)((center[2 * c + 1] - py) * ih));
      for (int s = 0; s < 3; ++s) {
        int i = lane + 32 * s;
        if (i > p) break;
        if (i == 0) {
          acc[s] = cadd(acc[s], sm[wl][0]);
          continue;
        }
        zf sum = cmake(0.f, 0.f);
        for (int j = 1; j < i; ++j) {
          const float bc = binom[(i - 1) * nb + (j - 1)];
          sum = zfmul(cadd(sum, cmake(sm[wl][j].re * bc, sm[wl][j].im * bc)), u);
        }
        acc[s] = cadd(acc[s], cadd(sum, sm[wl][i]));
      }
    }
    for (int s = 0; s < 3; ++s) {
      int i = lane + 32 * s;
      if (i <= p) mult[(int64_t)node * P1 + i] = acc[s];
    }
  }
}

// M2L, warp per target node, lane i <-> local term i.  Per source, lane j
// makes w^j (binary powers) and s_j = ma_j w^j; then
// la_i += (1/h) (-1)^i w^i sum_j C(i+j-1, j-1) s_j, with the s_j of the
// source read from shared memory (double-buffered, so one __syncwarp per
// source) and the next source's coefficients loaded while this one runs.
__global__ void __launch_bounds__(128) k2f_m2l(int nn, int p, const int *__restrict__ far_off,
                                               const int *__restrict__ far_src,
                                               const int *__restrict__ sysn,
                                               const uint8_t *__restrict__ depth,
                                               const double *__restrict__ sysbox,
                                               const double *__restrict__ center,
                                               const float *__restrict__ binom, int nb,
                                               const zf *__restrict__ mult, zf *__restrict__ loc) {
  extern __shared__ float smemf[];
  const int P1 = p + 1;
  const int SP = p | 1;
  float *tab = smemf;                    // tab[i * SP + j] = C(i+j-1, j-1)
  zf *sbuf = reinterpret_cast<zf *>(smemf + ((P1 * SP + 1) & ~1));
  for (int x = threadIdx.x; x < P1 * SP; x += blockDim.x) {
    int i = x / SP, j = x % SP;
    tab[x] = (j >= 1 && j < p) ? binom[(i + j - 1) * nb + (j - 1)] : 0.f;
  }
  __syncthreads();
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int t = blockIdx.x * (blockDim.x >> 5) + wl;
  if (t >= nn) return;
  int f0 = far_off[t], f1 = far_off[t + 1];
  if (f0 == f1) return;
  zf *sw = sbuf + wl * 2 * 32;           // two buffers of 32 per warp
  const double tx = center[2 * t], ty = center[2 * t + 1];
  const double h = node_size2(sysbox, sysn[t], depth[t]), ih = 1.0 / h;
  const float *row = tab + (lane <= p ? lane : 0) * SP;
  zf acc = cmake(0.f, 0.f);
  const bool mine = lane >= 1 && lane < p;   // lanes holding a source term
  int sn = far_src[f0];
  zf ma = mine ? mult[(int64_t)sn * P1 + lane] : cmake(0.f, 0.f);
  for (int f = f0; f < f1; ++f) {
    // w = h / (zt - zs): the centre offset in node sizes (small integers,
    // exact in FP32) from FP64, its inverse in FP32
    const float ux = (float)((tx - center[2 * sn]) * ih), uy = (float)((ty - center[2 * sn + 1]) * ih);
    const float iu2 = 1.f / (ux * ux + uy * uy);
    const zf w = cmake(ux * iu2, -uy * iu2);
    // prefetch the next source's term
    zf nma = cmake(0.f, 0.f);
    int nsn = sn;
    if (f + 1 < f1) {
      nsn = far_src[f + 1];
      if (mine) nma = mult[(int64_t)nsn * P1 + lane];
    }
    // w^lane by binary powers
    zf wp = cmake(1.f, 0.f), b = w;
    for (int e = lane; e; e >>= 1) {
      if (e & 1) wp = zfmul(wp, b);
      b = zfmul(b, b);
    }
    zf *buf = sw + 32 * (f & 1);
    buf[lane] = zfmul(ma, wp);
    __syncwarp();
    if (lane <= p) {
      zf sum = cmake(0.f, 0.f);
      for (int j = 1; j < p; ++j) {
        const zf sj = buf[j];
        sum.re = fmaf(row[j], sj.re, sum.re);
        sum.im = fmaf(row[j], sj.im, sum.im);
      }
      acc = cadd(acc, zfmul(sum, wp));
    }
    sn = nsn;
    ma = nma;
  }
  // (-1)^i of every term, applied once
  const float ihf = (float)(1.0 / h);
  if (lane <= p) {
    const zf a = (lane & 1) ? cmake(-acc.re, -acc.im) : acc;
    zf *o = loc + (int64_t)t * P1 + lane;
    *o = cadd(*o, cmake(a.re * ihf, a.im * ihf));
  }
}

__global__ void k2f_l2l(int cnt, int off, int p, const int *__restrict__ parent,
                        const int *__restrict__ begin, const int *__restrict__ end,
                        const int *__restrict__ sysn, const uint8_t *__restrict__ depth,
                        const double *__restrict__ sysbox, const double *__restrict__ center,
                        const float *__restrict__ binom, int nb, zf *__restrict__ loc) {
  __shared__ zf sm[4][kMaxOrder2d + 1];
  int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int k = blockIdx.x * (blockDim.x >> 5) + wl;
  if (k >= cnt) return;
  int node = off + k;
  int par = parent[node];
  if (par < 0 || end[node] == begin[node]) return;
  const int P1 = p + 1;
  for (int t = lane; t <= p; t += 32) sm[wl][t] = loc[(int64_t)par * P1 + t];
  __syncwarp();
  const double ihp = 1.0 / node_size2(sysbox, sysn[par], depth[par]);
  const zf u = cmake((float)((center[2 * node] - center[2 * par]) * ihp),
                     (float)((center[2 * node + 1] - center[2 * par + 1]) * ihp));
  for (int s = 0; s < 3; ++s) {
    int i = lane + 32 * s;
    if (i > p) break;
    zf sum = sm[wl][p];
    for (int j = p - 1; j >= i; --j) {
      const float bc = binom[j * nb + i];
      sum = cadd(zfmul(sum, u), cmake(sm[wl][j].re * bc, sm[wl][j].im * bc));
    }
    const float r = ldexpf(1.f, -i);
    zf *o = loc + (int64_t)node * P1 + i;
    *o = cadd(*o, cmake(sum.re * r, sum.im * r));
  }
}

// near field, warp per target leaf: each near range is staged 32 sources at
// a time in shared memory as FP32 positions relative to the target leaf's
// centre (the FP64 difference rounded once), and lanes sum their targets
// against them in FP32; a pair closer than h/8 (h the target leaf's size),
// where that rounding would show, is recomputed from the FP64 positions.
// FP32 partial sums per range, FP64 sums per target.
__global__ void __launch_bounds__(128) k2f_p2p(int nleaves, const int *__restrict__ leaf_be,
                        const int *__restrict__ near_off, const int2 *__restrict__ near_rng,
                        const int *__restrict__ leaf_node, const int *__restrict__ sysn,
                        const uint8_t *__restrict__ depth, const double *__restrict__ sysbox,
                        const double *__restrict__ center, const double *__restrict__ sx,
                        const double *__restrict__ sy, const double *__restrict__ sq,
                        zd *__restrict__ near_acc) {
  __shared__ float4 stg[4][32];
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int warp = blockIdx.x * 4 + wl;
  if (warp >= nleaves) return;
  const int b = leaf_be[warp], e = leaf_be[warp + 1];
  const int r0 = near_off[warp], r1 = near_off[warp + 1];
  const int node = leaf_node[warp];
  const double cx = center[2 * node], cy = center[2 * node + 1];
  const double hh = node_size2(sysbox, sysn[node], depth[node]);
  const float thr2 = (float)(hh * hh / 64.0);
  float4 *buf = stg[wl];
  for (int base = b; base < e; base += 32) {
    const int i = base + lane;
    const bool on = i < e;
    const double xi = on ? sx[i] : cx, yi = on ? sy[i] : cy;
    const float xr = (float)(xi - cx), yr = (float)(yi - cy);
    double re = 0.0, im = 0.0;
    for (int r = r0; r < r1; ++r) {
      const int2 rg = near_rng[r];
      const int j0 = leaf_be[rg.x], j1 = leaf_be[rg.y];
      float fr = 0.f, fi = 0.f;
      for (int c0 = j0; c0 < j1; c0 += 32) {
        const int cnt = min(32, j1 - c0);
        __syncwarp();
        if (lane < cnt) {
          const int j = c0 + lane;
          buf[lane] = make_float4((float)(sx[j] - cx), (float)(sy[j] - cy), (float)sq[j],
                                  __int_as_float(j));
        }
        __syncwarp();
        for (int k = 0; k < cnt; ++k) {
          const float4 sv = buf[k];
          float dx = xr - sv.x, dy = yr - sv.y;
          float r2 = dx * dx + dy * dy;
          if (r2 < thr2) {
            const int j = __float_as_int(sv.w);
            if (j == i || !on) continue;
            dx = (float)(xi - sx[j]);
            dy = (float)(yi - sy[j]);
            r2 = dx * dx + dy * dy;
            if (!(r2 > 0.f)) continue;
          }
          const float wgt = sv.z * __frcp_rn(r2);
          fr = fmaf(dx, wgt, fr);
          fi = fmaf(-dy, wgt, fi);
        }
      }
      re += fr;
      im += fi;
    }
    if (on) near_acc[i] = cmake(re, im);
  }
}

__global__ void k2f_l2p(int64_t n, int p, const int *__restrict__ incl, const int *__restrict__ leaf_node,
                        const int *__restrict__ sysn, const uint8_t *__restrict__ depth,
                        const double *__restrict__ sysbox, const double *__restrict__ center,
                        const double *__restrict__ sx, const double *__restrict__ sy,
                        const zf *__restrict__ loc, const zd *__restrict__ near_acc,
                        const int *__restrict__ perm, double *__restrict__ out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  int node = leaf_node[incl[i] - 1];
  const zf *a = loc + (int64_t)node * (p + 1);
  const double ih = 1.0 / node_size2(sysbox, sysn[node], depth[node]);
  const zf z = cmake((float)((sx[i] - center[2 * node]) * ih), (float)((sy[i] - center[2 * node + 1]) * ih));
  zf v = a[p];
  for (int k = p - 1; k >= 0; --k) v = cadd(zfmul(v, z), a[k]);
  const zd nr = near_acc[i];
  int o = perm[i];
  out[2 * (int64_t)o] = (double)v.re + nr.re;
  out[2 * (int64_t)o + 1] = (double)v.im + nr.im;
}

// counters: [0] sum cnt_L * sum_r cnt(r), [1] sum cnt_L^2, [2] sum cnt_L (cnt_L + 1) / 2,
// [3] non-empty nodes with a parent
__global__ void k2_stats(int nleaves, int nn, const int *__restrict__ leaf_be,
                         const int *__restrict__ near_off, const int2 *__restrict__ near_rng,
                         const int *__restrict__ begin, const int *__restrict__ end,
                         const int *__restrict__ parent, unsigned long long *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long a = 0, b = 0, c = 0, d = 0;
  if (i < nleaves) {
    long long cl = leaf_be[i + 1] - leaf_be[i];
    long long s = 0;
    for (int r = near_off[i]; r < near_off[i + 1]; ++r) {
      int2 rg = near_rng[r];
      s += leaf_be[rg.y] - leaf_be[rg.x];
    }
    a = (unsigned long long)(cl * s);
    b = (unsigned long long)(cl * cl);
    c = (unsigned long long)(cl * (cl + 1) / 2);
  }
  if (i < nn && parent[i] >= 0 && end[i] > begin[i]) d = 1;
  for (int o = 16; o; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
    d += __shfl_xor_sync(0xffffffffu, d, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(out, a);
    atomicAdd(out + 1, b);
    atomicAdd(out + 2, c);
    atomicAdd(out + 3, d);
  }
}

}  // namespace
}  // namespace aran

struct AranGpuSolver2d {
  AranGpuConfig2d cfg;
  int device = 0;
  cudaStream_t s0 = nullptr, s1 = nullptr;
  cudaEvent_t ev[2 * aran::Stage::NSTAGE] = {};
  cudaEvent_t ev_lists = nullptr, ev_p2p = nullptr;
  aran::DBuf<double> binom;   // (2p+1)^2 Pascal triangle
  int nb = 0;
  // particles
  aran::DBuf<int64_t> offs;
  aran::DBuf<double> sysbox;
  aran::DBuf<uint64_t> keys_in, keys_out;
  aran::DBuf<int> idx_in, perm, incl, flags;
  aran::DBuf<int> err2;   // input checks of the key pass
  aran::DBuf<uint8_t> cub_tmp;
  aran::DBuf<double> sx, sy, sq, io_xy, io_q, io_acc;
  // forest
  aran::DBuf<int> nsys_, ij, begin, end, child, parent, col, ncol, far_off, far_src;
  aran::DBuf<int> lf_begin, lf_end, leaf_node, leaf_be, near_off;
  aran::DBuf<int2> near_rng;
  aran::DBuf<uint8_t> depth;
  aran::DBuf<double> center;
  aran::DBuf<aran::cplx<double>> mult, loc, near_acc;
  aran::DBuf<aran::cplx<float>> mult32, loc32;   // mixed precision: scaled FP32 expansions
  aran::DBuf<float> binom32;
  aran::DBuf<unsigned long long> stats_dev;
  std::vector<int> level_off;
  int nnodes = 0, nlevels = 0, nleaves = 0, nrng = 0, empty_roots = 0;
  int64_t n = 0, nfar = 0;
  int64_t stats[11] = {};
  double ms[16] = {};
  int64_t launches = 0;
  // host predicate keeping nodes about to be split as leaves (virtual leaves)
  AranGpuLeafPredicate leaf_pred = nullptr;
  void *leaf_pred_data = nullptr;
  std::vector<double> h_sysbox;   // per system: lbx, lby, ubx, uby, scale x, scale y
};

namespace aran {
namespace {

template <typename T>
void ex_scan(AranGpuSolver2d *s, const T *in, T *out, int n, cudaStream_t st) {
  size_t bytes = 0;
  ACHECK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st));
  s->cub_tmp.reserve(bytes);
  ACHECK(cub::DeviceScan::ExclusiveSum(s->cub_tmp.ptr, bytes, in, out, n, st));
  s->launches += 2;
}

Nodes2 nodes(AranGpuSolver2d *s) {
  Nodes2 na;
  na.sys = s->nsys_.ptr;
  na.ij = s->ij.ptr;
  na.begin = s->begin.ptr;
  na.end = s->end.ptr;
  na.child = s->child.ptr;
  na.parent = s->parent.ptr;
  na.depth = s->depth.ptr;
  na.center = s->center.ptr;
  return na;
}

void grow(AranGpuSolver2d *s, size_t need, size_t keep, cudaStream_t st) {
  s->nsys_.grow_keep(need, keep, st);
  s->ij.grow_keep(2 * need, 2 * keep, st);
  s->begin.grow_keep(need, keep, st);
  s->end.grow_keep(need, keep, st);
  s->child.grow_keep(need, keep, st);
  s->parent.grow_keep(need, keep, st);
  s->depth.grow_keep(need, keep, st);
  s->center.grow_keep(2 * need, 2 * keep, st);
}

int read_int(const int *d, cudaStream_t st) {
  int h = 0;
  ACHECK(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaStreamSynchronize(st));
  return h;
}

// the nodes of one level about to be split are shown to the host leaf
// predicate (z components 0); those it keeps as leaves lose their flag
void leaf_predicate2(AranGpuSolver2d *s, int off, int cnt, int d, cudaStream_t st) {
  std::vector<int> fl(cnt), b(cnt), e(cnt), ij(2 * (size_t)cnt), sys(cnt);
  ACHECK(cudaMemcpyAsync(fl.data(), s->flags.ptr, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(b.data(), s->begin.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(e.data(), s->end.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(ij.data(), s->ij.ptr + 2 * (size_t)off, 2 * cnt * sizeof(int),
                         cudaMemcpyDeviceToHost, st));
  ACHECK(cudaMemcpyAsync(sys.data(), s->nsys_.ptr + off, cnt * sizeof(int), cudaMemcpyDeviceToHost, st));
  ACHECK(cudaStreamSynchronize(st));
  bool changed = false;
  for (int i = 0; i < cnt; ++i) {
    if (!fl[i]) continue;
    AranGpuNodeView v;
    std::memset(&v, 0, sizeof(v));
    const double *bx = s->h_sysbox.data() + 6 * (size_t)sys[i];
    for (int a = 0; a < 2; ++a) {
      double lo = bx[a], hi = bx[2 + a];
      for (int bit = d - 1; bit >= 0; --bit) {
        const double mid = (lo + hi) * 0.5;
        if ((ij[2 * (size_t)i + a] >> bit) & 1) lo = mid;
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
    ACHECK(cudaMemcpyAsync(s->flags.ptr, fl.data(), cnt * sizeof(int), cudaMemcpyHostToDevice, st));
  ACHECK(cudaStreamSynchronize(st));
}

void build_forest(AranGpuSolver2d *s, int nsys, const double *dxy, const double *dq) {
  cudaStream_t st = s->s0;
  const int TB = 256;
  const int64_t n = s->n;
  s->keys_in.reserve(n);
  s->keys_out.reserve(n);
  s->idx_in.reserve(n);
  s->perm.reserve(n);
  s->err2.reserve(1);
  ACHECK(cudaMemsetAsync(s->err2.ptr, 0, sizeof(int), st));
  k2_keys<<<ceil_div(n, TB), TB, 0, st>>>(n, nsys, s->offs.ptr, s->sysbox.ptr, dxy, dq,
                                           s->keys_in.ptr, s->idx_in.ptr, s->err2.ptr);
  s->launches++;
  {
    const int e = read_int(s->err2.ptr, st);
    if (e & kErrNonFinite) throw InputError{"a particle coordinate or charge is NaN or infinite"};
    if ((e & kErrOutside) && s->cfg.precision == ARAN_PRECISION_MIXED)
      throw InputError{"a particle lies outside its system's box (mixed precision needs every "
                       "point inside it)"};
  }
  int sysbits = 1;
  while ((1ll << sysbits) < nsys) ++sysbits;
  size_t bytes = 0;
  ACHECK(cub::DeviceRadixSort::SortPairs(nullptr, bytes, s->keys_in.ptr, s->keys_out.ptr,
                                         s->idx_in.ptr, s->perm.ptr, (int)n, 0,
                                         kSysShift + sysbits, st));
  s->cub_tmp.reserve(bytes);
  ACHECK(cub::DeviceRadixSort::SortPairs(s->cub_tmp.ptr, bytes, s->keys_in.ptr, s->keys_out.ptr,
                                         s->idx_in.ptr, s->perm.ptr, (int)n, 0,
                                         kSysShift + sysbits, st));
  s->launches += 4;
  s->sx.reserve(n);
  s->sy.reserve(n);
  s->sq.reserve(n);
  k2_gather<<<ceil_div(n, TB), TB, 0, st>>>(n, s->perm.ptr, dxy, dq, s->sx.ptr, s->sy.ptr, s->sq.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::SORT + 1], st));

  int maxd = s->cfg.max_depth > 0 ? s->cfg.max_depth : kKeyBits;
  grow(s, (size_t)nsys + 4 * (n / (s->cfg.maxbox + 1) + 1) * 2 + 64, 0, st);
  k2_roots<<<ceil_div(nsys, TB), TB, 0, st>>>(nsys, s->offs.ptr, s->sysbox.ptr, nodes(s));
  s->launches++;
  s->level_off.assign(1, 0);
  int off = 0, cnt = nsys, d = 0;
  while (cnt > 0) {
    s->level_off.push_back(off + cnt);
    s->flags.reserve(2 * (size_t)cnt + 2);
    int *pos = s->flags.ptr + cnt + 1;
    k2_flag<<<ceil_div(cnt, TB), TB, 0, st>>>(cnt, off, s->begin.ptr, s->end.ptr, s->cfg.maxbox, d,
                                               maxd, s->flags.ptr);
    s->launches++;
    if (s->leaf_pred) leaf_predicate2(s, off, cnt, d, st);
    ACHECK(cudaMemsetAsync(s->flags.ptr + cnt, 0, sizeof(int), st));
    ex_scan(s, s->flags.ptr, pos, cnt + 1, st);
    int ninternal = read_int(pos + cnt, st);
    int child_off = off + cnt;
    size_t need = (size_t)child_off + 4 * (size_t)ninternal;
    if (need > s->begin.cap) grow(s, need, child_off, st);
    k2_children<<<ceil_div(cnt, TB), TB, 0, st>>>(cnt, off, child_off, s->flags.ptr, pos,
                                                   s->keys_out.ptr, d, nodes(s), s->sysbox.ptr);
    s->launches++;
    off = child_off;
    cnt = 4 * ninternal;
    ++d;
  }
  s->nnodes = off;
  s->nlevels = d;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::TREE + 1], st));
}

void build_lists2(AranGpuSolver2d *s) {
  cudaStream_t st = s->s0;
  const int TB = 256;
  const int nn = s->nnodes;
  const int64_t n = s->n;
  s->col.reserve(9 * (size_t)nn);
  s->ncol.reserve(nn);
  for (int d = 0; d < s->nlevels; ++d) {
    int off = s->level_off[d], cnt = s->level_off[d + 1] - off;
    k2_colleagues<<<ceil_div(cnt, TB), TB, 0, st>>>(cnt, off, s->begin.ptr, s->end.ptr, s->child.ptr,
                                                     s->parent.ptr, s->ij.ptr, s->col.ptr, s->ncol.ptr);
    s->launches++;
  }
  s->flags.reserve((size_t)std::max<int64_t>(nn, n) + 2);
  s->far_off.reserve(nn + 1);
  k2_far<<<ceil_div(nn, TB), TB, 0, st>>>(nn, s->begin.ptr, s->end.ptr, s->child.ptr, s->parent.ptr,
                                           s->ij.ptr, s->col.ptr, s->ncol.ptr, s->flags.ptr, nullptr,
                                           nullptr, 0);
  s->launches++;
  ACHECK(cudaMemsetAsync(s->flags.ptr + nn, 0, sizeof(int), st));
  ex_scan(s, s->flags.ptr, s->far_off.ptr, nn + 1, st);
  s->nfar = read_int(s->far_off.ptr + nn, st);
  s->far_src.reserve(s->nfar + 1);
  k2_far<<<ceil_div(nn, TB), TB, 0, st>>>(nn, s->begin.ptr, s->end.ptr, s->child.ptr, s->parent.ptr,
                                           s->ij.ptr, s->col.ptr, s->ncol.ptr, nullptr, s->far_off.ptr,
                                           s->far_src.ptr, 1);
  s->launches++;
  // leaves in key order
  s->incl.reserve(n);
  ACHECK(cudaMemsetAsync(s->flags.ptr, 0, n * sizeof(int), st));
  k2_leaf_starts<<<ceil_div(nn, TB), TB, 0, st>>>(nn, s->begin.ptr, s->end.ptr, s->child.ptr,
                                                   s->flags.ptr);
  s->launches++;
  {
    size_t bytes = 0;
    ACHECK(cub::DeviceScan::InclusiveSum(nullptr, bytes, s->flags.ptr, s->incl.ptr, (int)n, st));
    s->cub_tmp.reserve(bytes);
    ACHECK(cub::DeviceScan::InclusiveSum(s->cub_tmp.ptr, bytes, s->flags.ptr, s->incl.ptr, (int)n, st));
    s->launches += 2;
  }
  s->nleaves = read_int(s->incl.ptr + n - 1, st);
  const int nl = s->nleaves;
  s->lf_begin.reserve(nn);
  s->lf_end.reserve(nn);
  s->leaf_node.reserve(nl + 1);
  s->leaf_be.reserve(nl + 1);
  k2_leaf_ranges<<<ceil_div(nn, TB), TB, 0, st>>>(nn, s->begin.ptr, s->end.ptr, s->child.ptr,
                                                   s->incl.ptr, s->lf_begin.ptr, s->lf_end.ptr,
                                                   s->leaf_node.ptr, s->leaf_be.ptr);
  s->launches++;
  int nint = (int)n;
  ACHECK(cudaMemcpyAsync(s->leaf_be.ptr + nl, &nint, sizeof(int), cudaMemcpyHostToDevice, st));
  s->near_off.reserve(nl + 1);
  k2_near<<<ceil_div(nl, TB), TB, 0, st>>>(nl, s->leaf_node.ptr, s->begin.ptr, s->end.ptr,
                                            s->child.ptr, s->parent.ptr, s->col.ptr, s->ncol.ptr,
                                            s->lf_begin.ptr, s->lf_end.ptr, s->flags.ptr, nullptr,
                                            nullptr, 0);
  s->launches++;
  ACHECK(cudaMemsetAsync(s->flags.ptr + nl, 0, sizeof(int), st));
  ex_scan(s, s->flags.ptr, s->near_off.ptr, nl + 1, st);
  s->nrng = read_int(s->near_off.ptr + nl, st);
  s->near_rng.reserve(s->nrng + 1);
  k2_near<<<ceil_div(nl, TB), TB, 0, st>>>(nl, s->leaf_node.ptr, s->begin.ptr, s->end.ptr,
                                            s->child.ptr, s->parent.ptr, s->col.ptr, s->ncol.ptr,
                                            s->lf_begin.ptr, s->lf_end.ptr, nullptr, s->near_off.ptr,
                                            s->near_rng.ptr, 1);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::LISTS + 1], st));
}

void run_passes2_mixed(AranGpuSolver2d *s, double *dacc) {
  cudaStream_t st = s->s0, s1 = s->s1;
  const int p = s->cfg.order, P1 = p + 1;
  const int nn = s->nnodes, nl = s->nleaves;
  const int64_t n = s->n;
  typedef cplx<float> zf;
  s->mult32.reserve((size_t)nn * P1);
  s->loc32.reserve((size_t)nn * P1);
  s->near_acc.reserve(n);
  ACHECK(cudaEventRecord(s->ev_lists, st));
  ACHECK(cudaStreamWaitEvent(s1, s->ev_lists, 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P], s1));
  k2f_p2p<<<ceil_div(nl, 4), 128, 0, s1>>>(nl, s->leaf_be.ptr, s->near_off.ptr, s->near_rng.ptr,
                                            s->leaf_node.ptr, s->nsys_.ptr, s->depth.ptr,
                                            s->sysbox.ptr, s->center.ptr, s->sx.ptr, s->sy.ptr,
                                            s->sq.ptr, s->near_acc.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P + 1], s1));
  ACHECK(cudaEventRecord(s->ev_p2p, s1));

  ACHECK(cudaMemsetAsync(s->mult32.ptr, 0, (size_t)nn * P1 * sizeof(zf), st));
  ACHECK(cudaMemsetAsync(s->loc32.ptr, 0, (size_t)nn * P1 * sizeof(zf), st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M], st));
  k2f_p2m<<<ceil_div((int64_t)nl * 32, 128), 128, 0, st>>>(
      nl, p, s->leaf_node.ptr, s->begin.ptr, s->end.ptr, s->nsys_.ptr, s->depth.ptr, s->sysbox.ptr,
      s->center.ptr, s->sx.ptr, s->sy.ptr, s->sq.ptr, s->mult32.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M], st));
  for (int d = s->nlevels - 2; d >= 0; --d) {
    int off = s->level_off[d], cnt = s->level_off[d + 1] - off;
    k2f_m2m<<<ceil_div(cnt, 4), 128, 0, st>>>(cnt, off, p, s->child.ptr, s->begin.ptr, s->end.ptr,
                                              s->nsys_.ptr, s->depth.ptr, s->sysbox.ptr,
                                              s->center.ptr, s->binom32.ptr, s->nb, s->mult32.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L], st));
  {
    size_t smem = (size_t)(((P1 * (p | 1)) + 1) & ~1) * sizeof(float) + 4 * 2 * 32 * sizeof(zf);
    k2f_m2l<<<ceil_div(nn, 4), 128, smem, st>>>(nn, p, s->far_off.ptr, s->far_src.ptr, s->nsys_.ptr,
                                                 s->depth.ptr, s->sysbox.ptr, s->center.ptr,
                                                 s->binom32.ptr, s->nb, s->mult32.ptr, s->loc32.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L], st));
  for (int d = 2; d < s->nlevels; ++d) {
    int off = s->level_off[d], cnt = s->level_off[d + 1] - off;
    k2f_l2l<<<ceil_div(cnt, 4), 128, 0, st>>>(cnt, off, p, s->parent.ptr, s->begin.ptr, s->end.ptr,
                                              s->nsys_.ptr, s->depth.ptr, s->sysbox.ptr,
                                              s->center.ptr, s->binom32.ptr, s->nb, s->loc32.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L + 1], st));
  ACHECK(cudaStreamWaitEvent(st, s->ev_p2p, 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P], st));
  k2f_l2p<<<ceil_div(n, 256), 256, 0, st>>>(n, p, s->incl.ptr, s->leaf_node.ptr, s->nsys_.ptr,
                                            s->depth.ptr, s->sysbox.ptr, s->center.ptr, s->sx.ptr,
                                            s->sy.ptr, s->loc32.ptr, s->near_acc.ptr, s->perm.ptr,
                                            dacc);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P + 1], st));
}

void run_passes2(AranGpuSolver2d *s, double *dacc) {
  cudaStream_t st = s->s0, s1 = s->s1;
  const int p = s->cfg.order, P1 = p + 1;
  const int nn = s->nnodes, nl = s->nleaves;
  const int64_t n = s->n;
  if (s->cfg.precision == ARAN_PRECISION_MIXED) {
    run_passes2_mixed(s, dacc);
  } else {
  s->mult.reserve((size_t)nn * P1);
  s->loc.reserve((size_t)nn * P1);
  s->near_acc.reserve(n);
  // near field on its own stream
  ACHECK(cudaEventRecord(s->ev_lists, st));
  ACHECK(cudaStreamWaitEvent(s1, s->ev_lists, 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P], s1));
  k2_p2p<<<ceil_div((int64_t)nl * 32, 128), 128, 0, s1>>>(nl, s->leaf_be.ptr, s->near_off.ptr,
                                                          s->near_rng.ptr, s->sx.ptr, s->sy.ptr,
                                                          s->sq.ptr, s->near_acc.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2P + 1], s1));
  ACHECK(cudaEventRecord(s->ev_p2p, s1));

  ACHECK(cudaMemsetAsync(s->mult.ptr, 0, (size_t)nn * P1 * sizeof(zd), st));
  ACHECK(cudaMemsetAsync(s->loc.ptr, 0, (size_t)nn * P1 * sizeof(zd), st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M], st));
  k2_p2m<<<ceil_div((int64_t)nl * 32, 128), 128, 0, st>>>(nl, p, s->leaf_node.ptr, s->begin.ptr,
                                                          s->end.ptr, s->center.ptr, s->sx.ptr,
                                                          s->sy.ptr, s->sq.ptr, s->mult.ptr);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::P2M + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M], st));
  for (int d = s->nlevels - 2; d >= 0; --d) {
    int off = s->level_off[d], cnt = s->level_off[d + 1] - off;
    k2_m2m<<<ceil_div(cnt, 4), 128, 0, st>>>(cnt, off, p, s->child.ptr, s->begin.ptr, s->end.ptr,
                                             s->center.ptr, s->binom.ptr, s->nb, s->mult.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2M + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L], st));
  {
    size_t smem = (size_t)P1 * (p | 1) * sizeof(double) + 4 * (size_t)P1 * sizeof(zd);
    k2_m2l<<<ceil_div(nn, 4), 128, smem, st>>>(nn, p, s->far_off.ptr, s->far_src.ptr, s->center.ptr,
                                                s->binom.ptr, s->nb, s->mult.ptr, s->loc.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::M2L + 1], st));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L], st));
  for (int d = 2; d < s->nlevels; ++d) {
    int off = s->level_off[d], cnt = s->level_off[d + 1] - off;
    k2_l2l<<<ceil_div(cnt, 4), 128, 0, st>>>(cnt, off, p, s->parent.ptr, s->begin.ptr, s->end.ptr,
                                             s->center.ptr, s->binom.ptr, s->nb, s->loc.ptr);
    s->launches++;
  }
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2L + 1], st));
  ACHECK(cudaStreamWaitEvent(st, s->ev_p2p, 0));
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P], st));
  k2_l2p<<<ceil_div(n, 256), 256, 0, st>>>(n, p, s->incl.ptr, s->leaf_node.ptr, s->center.ptr,
                                           s->sx.ptr, s->sy.ptr, s->loc.ptr, s->near_acc.ptr,
                                           s->perm.ptr, dacc);
  s->launches++;
  ACHECK(cudaEventRecord(s->ev[2 * Stage::L2P + 1], st));
  }
  // counters
  s->stats_dev.reserve(4);
  ACHECK(cudaMemsetAsync(s->stats_dev.ptr, 0, 4 * sizeof(unsigned long long), st));
  int m = std::max(nl, nn);
  k2_stats<<<ceil_div(m, 256), 256, 0, st>>>(nl, nn, s->leaf_be.ptr, s->near_off.ptr, s->near_rng.ptr,
                                             s->begin.ptr, s->end.ptr, s->parent.ptr, s->stats_dev.ptr);
  s->launches++;
}

int check2(const AranGpuConfig2d *c) {
  if (!c) return fail(ARAN_ERR_INVALID, "config is NULL");
  if (c->maxbox < 1) return fail(ARAN_ERR_INVALID, "maxbox must be >= 1");
  if (c->order < 1 || c->order > kMaxOrder2d)
    return fail(ARAN_ERR_INVALID, "order must be in [1, " + std::to_string(kMaxOrder2d) + "]");
  if (c->max_depth < 0 || c->max_depth > kKeyBits)
    return fail(ARAN_ERR_INVALID, "max_depth must be in [0, 21]");
  if (c->precision != ARAN_PRECISION_FP64 && c->precision != ARAN_PRECISION_MIXED)
    return fail(ARAN_ERR_INVALID, "unknown precision");
  if (c->precision == ARAN_PRECISION_MIXED && c->order > 31)
    return fail(ARAN_ERR_INVALID, "mixed precision 2D solves take orders up to 31");
  return ARAN_OK;
}

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" {

int aran_gpu_solver2d_create(const AranGpuConfig2d *cfg, AranGpuSolver2d **out) {
  if (!out) return fail(ARAN_ERR_INVALID, "out is NULL");
  *out = nullptr;
  int rc = check2(cfg);
  if (rc != ARAN_OK) return rc;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return fail(ARAN_ERR_NO_DEVICE, std::string("no CUDA device available: ") + cudaGetErrorString(e));
  AranGpuSolver2d *s = new AranGpuSolver2d();
  s->cfg = *cfg;
  try {
    ACHECK(cudaGetDevice(&s->device));
    ACHECK(cudaStreamCreateWithFlags(&s->s0, cudaStreamNonBlocking));
    ACHECK(cudaStreamCreateWithFlags(&s->s1, cudaStreamNonBlocking));
    for (auto &ev : s->ev) ACHECK(cudaEventCreate(&ev));
    ACHECK(cudaEventCreateWithFlags(&s->ev_lists, cudaEventDisableTiming));
    ACHECK(cudaEventCreateWithFlags(&s->ev_p2p, cudaEventDisableTiming));
    // Pascal triangle in doubles (aran/aranbinomial.c:44-51)
    const int p = cfg->order;
    s->nb = 2 * p + 2;
    std::vector<double> b((size_t)s->nb * s->nb, 0.0);
    for (int i = 0; i < s->nb; ++i)
      for (int j = 0; j <= i; ++j)
        b[(size_t)i * s->nb + j] =
            (j == 0 || j == i) ? 1.0 : b[(size_t)(i - 1) * s->nb + j] + b[(size_t)(i - 1) * s->nb + j - 1];
    s->binom.reserve(b.size());
    ACHECK(cudaMemcpyAsync(s->binom.ptr, b.data(), b.size() * sizeof(double), cudaMemcpyHostToDevice,
                           s->s0));
    std::vector<float> bf(b.begin(), b.end());
    s->binom32.reserve(bf.size());
    ACHECK(cudaMemcpyAsync(s->binom32.ptr, bf.data(), bf.size() * sizeof(float),
                           cudaMemcpyHostToDevice, s->s0));
    ACHECK(cudaStreamSynchronize(s->s0));
  } catch (const CudaError &ce) {
    int r = from_cuda(ce);
    aran_gpu_solver2d_destroy(s);
    return r;
  }
  *out = s;
  return ARAN_OK;
}

void aran_gpu_solver2d_destroy(AranGpuSolver2d *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->s0) cudaStreamSynchronize(s->s0);
  if (s->s1) cudaStreamSynchronize(s->s1);
  s->binom.release();
  s->offs.release();
  s->sysbox.release();
  s->keys_in.release();
  s->keys_out.release();
  s->idx_in.release();
  s->err2.release();
  s->perm.release();
  s->incl.release();
  s->flags.release();
  s->cub_tmp.release();
  s->sx.release();
  s->sy.release();
  s->sq.release();
  s->io_xy.release();
  s->io_q.release();
  s->io_acc.release();
  s->nsys_.release();
  s->ij.release();
  s->begin.release();
  s->end.release();
  s->child.release();
  s->parent.release();
  s->col.release();
  s->ncol.release();
  s->far_off.release();
  s->far_src.release();
  s->lf_begin.release();
  s->lf_end.release();
  s->leaf_node.release();
  s->leaf_be.release();
  s->near_off.release();
  s->near_rng.release();
  s->depth.release();
  s->center.release();
  s->mult.release();
  s->loc.release();
  s->near_acc.release();
  s->mult32.release();
  s->loc32.release();
  s->binom32.release();
  s->stats_dev.release();
  for (auto &ev : s->ev)
    if (ev) cudaEventDestroy(ev);
  if (s->ev_lists) cudaEventDestroy(s->ev_lists);
  if (s->ev_p2p) cudaEventDestroy(s->ev_p2p);
  if (s->s0) cudaStreamDestroy(s->s0);
  if (s->s1) cudaStreamDestroy(s->s1);
  delete s;
}

int aran_gpu_solver2d_solve(AranGpuSolver2d *s, int nsys, const int64_t *offs, const double *box,
                            const double *xy, const double *q, double *acc, int mem) {
  if (!acc) return fail(ARAN_ERR_INVALID, "NULL argument");
  return aran::solve2d_impl(s, nsys, offs, box, xy, q, acc, mem, false);
}

int aran_gpu_solver2d_set_leaf_predicate(AranGpuSolver2d *s, AranGpuLeafPredicate pred,
                                         void *user_data) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  s->leaf_pred = pred;
  s->leaf_pred_data = pred ? user_data : nullptr;
  return ARAN_OK;
}

}  // extern "C"

namespace aran {

int solve2d_impl(AranGpuSolver2d *s, int nsys, const int64_t *offs, const double *box,
                 const double *xy, const double *q, double *acc, int mem, bool tree_only) {
  if (!s) return fail(ARAN_ERR_INVALID, "solver is NULL");
  if (nsys < 1 || nsys > (1 << 21)) return fail(ARAN_ERR_INVALID, "nsys must be in [1, 2^21]");
  if (!offs || !box || !xy || !q) return fail(ARAN_ERR_INVALID, "NULL argument");
  if (mem != ARAN_MEM_HOST && mem != ARAN_MEM_DEVICE) return fail(ARAN_ERR_INVALID, "bad mem kind");
  if (offs[0] != 0) return fail(ARAN_ERR_INVALID, "offs[0] must be 0");
  int empty = 0;
  std::vector<double> sb(6 * (size_t)nsys);
  for (int i = 0; i < nsys; ++i) {
    if (offs[i + 1] < offs[i]) return fail(ARAN_ERR_INVALID, "offs must be non-decreasing");
    empty += offs[i + 1] == offs[i];
    for (int a = 0; a < 2; ++a) {
      double lo = box[4 * i + a], hi = box[4 * i + 2 + a];
      if (!(hi > lo) || !std::isfinite(lo) || !std::isfinite(hi))
        return fail(ARAN_ERR_INVALID, "box of system " + std::to_string(i) + " must satisfy lb < ub");
      sb[6 * i + a] = lo;
      sb[6 * i + 2 + a] = hi;
      sb[6 * i + 4 + a] = (double)(1 << kKeyBits) / (hi - lo);
    }
  }
  const int64_t n = offs[nsys];
  if (n < 1) return fail(ARAN_ERR_INVALID, "no particles");
  if (n > (int64_t)1 << 30) return fail(ARAN_ERR_INVALID, "more than 2^30 particles");
  try {
    ACHECK(cudaSetDevice(s->device));
    s->launches = 0;
    s->n = n;
    s->empty_roots = empty;
    cudaStream_t st = s->s0;
    ACHECK(cudaEventRecord(s->ev[2 * Stage::TOTAL], st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::H2D], st));
    s->offs.reserve(nsys + 1);
    s->sysbox.reserve(sb.size());
    ACHECK(cudaMemcpyAsync(s->offs.ptr, offs, (nsys + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st));
    ACHECK(cudaMemcpyAsync(s->sysbox.ptr, sb.data(), sb.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    const double *dxy = xy, *dq = q;
    double *dacc = acc;
    if (mem == ARAN_MEM_HOST) {
      s->io_xy.reserve(2 * n);
      s->io_q.reserve(n);
      s->io_acc.reserve(2 * n);
      ACHECK(cudaMemcpyAsync(s->io_xy.ptr, xy, 2 * n * sizeof(double), cudaMemcpyHostToDevice, st));
      ACHECK(cudaMemcpyAsync(s->io_q.ptr, q, n * sizeof(double), cudaMemcpyHostToDevice, st));
      dxy = s->io_xy.ptr;
      dq = s->io_q.ptr;
      dacc = s->io_acc.ptr;
    }
    ACHECK(cudaEventRecord(s->ev[2 * Stage::H2D + 1], st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::SORT], st));
    s->h_sysbox = sb;
    build_forest(s, nsys, dxy, dq);
    if (tree_only) {
      ACHECK(cudaStreamSynchronize(st));
      return ARAN_OK;
    }
    build_lists2(s);
    run_passes2(s, dacc);
    ACHECK(cudaEventRecord(s->ev[2 * Stage::D2H], st));
    if (mem == ARAN_MEM_HOST)
      ACHECK(cudaMemcpyAsync(acc, dacc, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, st));
    unsigned long long cnt[4];
    ACHECK(cudaMemcpyAsync(cnt, s->stats_dev.ptr, sizeof(cnt), cudaMemcpyDeviceToHost, st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::D2H + 1], st));
    ACHECK(cudaEventRecord(s->ev[2 * Stage::TOTAL + 1], st));
    ACHECK(cudaStreamSynchronize(st));
    ACHECK(cudaStreamSynchronize(s->s1));
    ACHECK(cudaGetLastError());
    std::memset(s->stats, 0, sizeof(s->stats));
    s->stats[0] = s->nnodes - s->empty_roots;
    s->stats[1] = (int64_t)((cnt[0] - cnt[1]) / 2 + cnt[2]);
    s->stats[2] = n;
    s->stats[3] = (int64_t)cnt[3];
    s->stats[4] = s->nfar;
    s->stats[5] = (int64_t)cnt[3];
    s->stats[6] = n;
    auto el = [&](int a, int b) {
      float m = 0.f;
      cudaEventElapsedTime(&m, s->ev[a], s->ev[b]);
      return (double)m;
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
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  } catch (const InputError &ie) {
    // stopped after the key pass: nothing was written
    cudaStreamSynchronize(s->s0);
    cudaStreamSynchronize(s->s1);
    return fail(ARAN_ERR_INVALID, ie.msg);
  }
  return ARAN_OK;
}

int forest2d_to_host(AranGpuSolver2d *s, Forest2dHost &h, bool expansions) {
  try {
    ACHECK(cudaSetDevice(s->device));
    const int nn = s->nnodes;
    h.p = s->cfg.order;
    h.nnodes = nn;
    h.begin.resize(nn);
    h.end.resize(nn);
    h.child.resize(nn);
    h.parent.resize(nn);
    h.sys.resize(nn);
    h.ij.resize(2 * (size_t)nn);
    h.depth.resize(nn);
    h.center.resize(2 * (size_t)nn);
    h.perm.resize(s->n);
    h.sysbox = s->h_sysbox;
    ACHECK(cudaMemcpy(h.begin.data(), s->begin.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.end.data(), s->end.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.child.data(), s->child.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.parent.data(), s->parent.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.sys.data(), s->nsys_.ptr, nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.ij.data(), s->ij.ptr, 2 * (size_t)nn * sizeof(int), cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.depth.data(), s->depth.ptr, nn, cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.center.data(), s->center.ptr, 2 * (size_t)nn * sizeof(double),
                      cudaMemcpyDeviceToHost));
    ACHECK(cudaMemcpy(h.perm.data(), s->perm.ptr, s->n * sizeof(int), cudaMemcpyDeviceToHost));
    h.mult.clear();
    h.loc.clear();
    if (expansions) {
      const size_t len = (size_t)nn * (h.p + 1) * 2;
      h.mult.resize(len);
      h.loc.resize(len);
      if (s->cfg.precision == ARAN_PRECISION_MIXED) {
        // back from the scaled FP32 storage: a_{-k} = ma_k h^{k-1}, b_k = la_k h^-k
        std::vector<float> m32(len), l32(len);
        ACHECK(cudaMemcpy(m32.data(), s->mult32.ptr, len * sizeof(float), cudaMemcpyDeviceToHost));
        ACHECK(cudaMemcpy(l32.data(), s->loc32.ptr, len * sizeof(float), cudaMemcpyDeviceToHost));
        for (int i = 0; i < nn; ++i) {
          const double *b = s->h_sysbox.data() + 6 * (size_t)h.sys[i];
          const double hs = std::max(b[2] - b[0], b[3] - b[1]) * std::ldexp(1.0, -(int)h.depth[i]);
          for (int k = 0; k <= h.p; ++k) {
            const size_t o = 2 * ((size_t)i * (h.p + 1) + k);
            const double fm = k >= 1 ? std::pow(hs, k - 1) : 1.0, fl = std::pow(hs, -k);
            h.mult[o] = m32[o] * fm;
            h.mult[o + 1] = m32[o + 1] * fm;
            h.loc[o] = l32[o] * fl;
            h.loc[o + 1] = l32[o + 1] * fl;
          }
        }
      } else {
        ACHECK(cudaMemcpy(h.mult.data(), s->mult.ptr, len * sizeof(double), cudaMemcpyDeviceToHost));
        ACHECK(cudaMemcpy(h.loc.data(), s->loc.ptr, len * sizeof(double), cudaMemcpyDeviceToHost));
      }
    }
  } catch (const CudaError &ce) {
    return from_cuda(ce);
  }
  return ARAN_OK;
}

}  // namespace aran

extern "C" {

int aran_gpu_solver2d_get_stats(AranGpuSolver2d *s, int64_t stats[11]) {
  if (!s || !stats) return fail(ARAN_ERR_INVALID, "NULL argument");
  std::memcpy(stats, s->stats, sizeof(s->stats));
  return ARAN_OK;
}

int aran_gpu_solver2d_timings(AranGpuSolver2d *s, double ms[16]) {
  if (!s || !ms) return fail(ARAN_ERR_INVALID, "NULL argument");
  std::memcpy(ms, s->ms, sizeof(s->ms));
  return ARAN_OK;
}

int aran_gpu_solver2d_tree_info(AranGpuSolver2d *s, int64_t info[5]) {
  if (!s || !info) return fail(ARAN_ERR_INVALID, "NULL argument");
  info[0] = s->nnodes;
  info[1] = s->nfar;
  info[2] = s->nrng;
  info[3] = s->nleaves;
  info[4] = s->nlevels > 0 ? s->nlevels - 1 : 0;
  return ARAN_OK;
}

int64_t aran_gpu_solver2d_launches(AranGpuSolver2d *s) { return s ? s->launches : -1; }

}  // extern "C"
