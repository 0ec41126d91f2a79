// m2l.cu -- multipole-to-local translations (far_func of
// aran/aransolver3d.c:333-354) with the "point and shoot" operator of
// aran_spherical_seriesd_to_local_rotate (aran/aransphericalseriesd-rotate.c:
// 165-207): rotate the source multipole so the translation runs along z,
// translate along z (aran/aransphericalseriesd-translate.c:609-676), rotate
// back and accumulate.
//
// Same-depth M2L sources of a node are non-adjacent children of its
// parent's colleagues, so the 8 children of a parent draw their sources from
// one 6x6x6 block of cells and every translation is one of the 316 offsets
// (dx,dy,dz) in [-3,3]^3 minus [-1,1]^3.  One CTA takes the 8 siblings (warp
// w <-> child w; its local stays in registers) and walks the offsets in
// lockstep: each offset's rotation/translation table (even/odd Wigner
// blocks for theta and -theta, z-phases, radial powers) is brought into
// shared memory once by a TMA bulk copy and used by every sibling that has a
// source at that offset.  The copies are double-buffered (mbarrier
// completion), so the next offset's table streams in while the current one
// is applied.  Every mbarrier wait is bounded; a wait that gives up sets
// the error word and the CTA stops issuing copies.  At orders whose tables
// do not fit in shared memory (NST = 0) the warps read the offset tables
// and vertical factors straight from global memory (L2-resident).
#include <cstring>

#include "internal.cuh"
#include "async.cuh"

namespace aran {


namespace {

__constant__ uint16_t c_dir_codes[316];
__constant__ int8_t c_dir_vec[316 * 3];

// asynchronous copy of one complex coefficient (8 bytes FP32, 16 bytes FP64)
template <typename T>
__device__ __forceinline__ void cp_async_cplx(cplx<T> *dst, const cplx<T> *src) {
  if (sizeof(cplx<T>) == 8) cp_async8(dst, src);
  else cp_async16(dst, src);
}

struct M2LOffsets {
  int ef, ei, ph, rp, vv, stride;  // in T units; ef/ei: (E, O) pairs in source-order planes
};

constexpr int kSibWarps = 8;   // consumers: one per child of the parent
constexpr int kMaxRounds = ((kMaxOrder + 1) * (kMaxOrder + 2) / 2 + 31) / 32;

template <typename T, int NST, int R, int G>
__global__ void __launch_bounds__(32 * (kSibWarps + 1), sizeof(T) == 4 ? 3 : 2)
    k_m2l_sibling(int nparents, const int *__restrict__ parents, const int *__restrict__ child,
                  const int *__restrict__ begin, const int *__restrict__ end,
                  const int *__restrict__ col, const int *__restrict__ ncol,
                  const int *__restrict__ ijk, const uint8_t *__restrict__ depth, int p,
                  const T *__restrict__ dirs, M2LOffsets D,
                  const uint8_t *__restrict__ lm_g, double scale_e,
                  const cplx<T> *__restrict__ mult, cplx<T> *__restrict__ loc,
                  int *__restrict__ err, int polls) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int nm = tri(p), nl = tri(p + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // shared layout: NST tables | full[NST] | empty[NST] | per-warp buffers
  // (G columns) | G 6x6x6 source grids | offset mask | active list (NST = 0:
  // no tables or barriers in shared memory)
  size_t off = 0;
  T *tab = reinterpret_cast<T *>(smem_raw);
  off += (size_t)NST * D.stride * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw + off);
  uint64_t *empty = full + NST;
  off += 2 * NST * sizeof(uint64_t);
  off = (off + 15) & ~(size_t)15;
  cplx<T> *wbuf = reinterpret_cast<cplx<T> *>(smem_raw + off);
  off += (size_t)kSibWarps * G * (nm + nl) * sizeof(cplx<T>);
  int *grid = reinterpret_cast<int *>(smem_raw + off);
  off += (size_t)G * 216 * sizeof(int);
  unsigned *mask = reinterpret_cast<unsigned *>(smem_raw + off);
  off += 10 * sizeof(unsigned);
  uint16_t *active = reinterpret_cast<uint16_t *>(smem_raw + off);
  off += 320 * sizeof(uint16_t);
  uint8_t *lm = smem_raw + off;           // (l, m) of coefficient c (tri order)
  off += 2 * nl;
  uint8_t *vmap = smem_raw + off;         // (l, m) of m-major slot k
  __shared__ int s_nact;

  for (int i = threadIdx.x; i < G * 216; i += blockDim.x) grid[i] = -1;
  if (threadIdx.x < 10) mask[threadIdx.x] = 0u;
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    int l, m;
    mmajor_lm(k, p, l, m);
    vmap[2 * k] = (uint8_t)l;
    vmap[2 * k + 1] = (uint8_t)m;
    lm[2 * k] = lm_g[2 * k];
    lm[2 * k + 1] = lm_g[2 * k + 1];
  }
  if (NST > 0 && threadIdx.x == 0) {
    for (int b = 0; b < NST; ++b) {
      mbar_init(&full[b], 1);
      mbar_init(&empty[b], kSibWarps);
    }
    fence_mbar_init();
  }
  __syncthreads();
  // the G parents of this CTA: their colleagues' children fill the grids
  for (int g = 0; g < G; ++g) {
    const int pidx = blockIdx.x * G + g;
    if (pidx >= nparents) break;
    const int P = parents[pidx];
    const int pi = ijk[3 * P], pj = ijk[3 * P + 1], pk = ijk[3 * P + 2];
    const int nc = ncol[P];
    for (int e = threadIdx.x; e < nc * 8; e += blockDim.x) {
      int q = col[27 * P + e / 8];
      int qc = child[q];
      if (qc < 0) continue;
      int o = e & 7;
      int s = qc + o;
      if (end[s] == begin[s]) continue;
      int gx = 2 * (ijk[3 * q] - pi + 1) + (o & 1);
      int gy = 2 * (ijk[3 * q + 1] - pj + 1) + ((o >> 1) & 1);
      int gz = 2 * (ijk[3 * q + 2] - pk + 1) + ((o >> 2) & 1);
      grid[g * 216 + gx + 6 * (gy + 6 * gz)] = s;
    }
  }
  __syncthreads();
  // consumer warp w <-> child w of each of the G parents (column g)
  int tg[G];
  bool tvalid[G];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const int pidx = blockIdx.x * G + g;
    tvalid[g] = false;
    tg[g] = 0;
    if (w < kSibWarps && pidx < nparents) {
      tg[g] = child[parents[pidx]] + w;
      tvalid[g] = end[tg[g]] > begin[tg[g]];
    }
  }
  const int tx = 2 + (w & 1), ty = 2 + ((w >> 1) & 1), tz = 2 + ((w >> 2) & 1);
  auto source_of = [&](int g, int di) -> int {
    if (!tvalid[g]) return -1;
    int cx = tx - c_dir_vec[3 * di], cy = ty - c_dir_vec[3 * di + 1], cz = tz - c_dir_vec[3 * di + 2];
    if (cx < 0 || cx > 5 || cy < 0 || cy > 5 || cz < 0 || cz > 5) return -1;
    return grid[g * 216 + cx + 6 * (cy + 6 * cz)];
  };
#pragma unroll
  for (int g = 0; g < G; ++g)
    if (tvalid[g])
      for (int di = lane; di < 316; di += 32)
        if (source_of(g, di) >= 0) atomicOr(&mask[di >> 5], 1u << (di & 31));
  __syncthreads();
  for (int di = threadIdx.x; di < 316; di += blockDim.x) {
    unsigned m = mask[di >> 5];
    if ((m >> (di & 31)) & 1u) {
      int pos = __popc(m & ((1u << (di & 31)) - 1u));
      for (int k = 0; k < (di >> 5); ++k) pos += __popc(mask[k]);
      active[pos] = (uint16_t)di;
    }
  }
  if (threadIdx.x == 0) {
    int tot = 0;
    for (int k = 0; k < 10; ++k) tot += __popc(mask[k]);
    s_nact = tot;
  }
  __syncthreads();
  const int nact = s_nact;
  const uint32_t tbytes = (uint32_t)(D.stride * sizeof(T));

  if (w == kSibWarps) {
    // producer warp: stream the offset tables through the NST-slot ring
    if (NST > 0 && lane == 0) {
      int issued = 0;
      for (int i = 0; i < nact; ++i) {
        const int b = i % (NST > 0 ? NST : 1);
        if (i >= NST && !mbar_wait_or_flag(&empty[b], ((i / (NST > 0 ? NST : 1)) - 1) & 1, err)) {
          atomicOr(err, kErrTimeout);
          break;
        }
        mbar_expect_tx(&full[b], tbytes);
        bulk_g2s(tab + (size_t)b * D.stride, dirs + (size_t)c_dir_codes[active[i]] * D.stride,
                 tbytes, &full[b]);
        ++issued;
      }
      // the last copy of every slot has landed before the CTA can leave
      // (earlier ones were waited for by the consumers before the slot was
      // refilled), also when the consumers stopped early
      for (int i = issued > NST ? issued - NST : 0; i < issued; ++i)
        mbar_wait(&full[i % (NST > 0 ? NST : 1)], (i / (NST > 0 ? NST : 1)) & 1);
    }
    return;
  }

  // accumulated locals of the G targets live in registers
  cplx<T> acc[G][R];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int r = 0; r < R; ++r) acc[g][r] = cmake<T>(0, 0);
  // column g: src (phased multipole) and tr (translated, m-major slots)
  // share region A, rot follows; between the vertical stage and the next
  // direction's phase stage the rot region holds the next source multipoles,
  // copied in asynchronously (cp.async) while the rotation back runs
  cplx<T> *cbuf = wbuf + (size_t)w * G * (nm + nl);
  int next_i = 0, next_s[G];
  auto find_next = [&](int from) {
    for (next_i = from; next_i < nact; ++next_i) {
      bool any = false;
#pragma unroll
      for (int g = 0; g < G; ++g) {
        next_s[g] = source_of(g, active[next_i]);
        any |= next_s[g] >= 0;
      }
      if (any) break;
    }
  };
  auto prefetch = [&]() {
#pragma unroll
    for (int g = 0; g < G; ++g)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int c = lane + 32 * r;
        if (c >= nm) continue;
        cplx<T> *dst = cbuf + g * (nm + nl) + nl + c;
        if (next_i < nact && next_s[g] >= 0)
          cp_async_cplx(dst, mult + (size_t)next_s[g] * nm + c);
        else
          *dst = cmake<T>(0, 0);
      }
    cp_async_commit();
  };
  find_next(0);
  prefetch();

  for (int i = 0; i < nact; ++i) {
    const int b = i % (NST > 0 ? NST : 1);
    if (NST > 0 && !mbar_wait_or_flag(&full[b], (i / (NST > 0 ? NST : 1)) & 1, err, polls)) {
      atomicOr(err, kErrTimeout);
      break;
    }
    if (i == next_i) {
      const T *tb = NST > 0 ? tab + (size_t)b * D.stride
                            : dirs + (size_t)c_dir_codes[active[i]] * D.stride;
      const T *ph = tb + D.ph;
      const T *EOf = tb + D.ef;
      const T *EOi = tb + D.ei;
      cp_async_wait_all();
      __syncwarp();
      // z-phase of the source multipoles: e^{i m phi}
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int c = lane + 32 * r;
        if (c < nm) {
          const int m = lm[2 * c + 1];
          T cr = ph[2 * m], ci = ph[2 * m + 1];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            cplx<T> v = cbuf[g * (nm + nl) + nl + c];
            cbuf[g * (nm + nl) + c] = cmake<T>(v.re * cr - v.im * ci, v.re * ci + v.im * cr);
          }
        }
      }
      find_next(i + 1);
      __syncwarp();
      // rotation to the z axis (degrees < p)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int c = lane + 32 * r;
        if (c < nm) {
          const int l = lm[2 * c];
          const T *e = EOf + 2 * c;        // plane 0; plane m+1 is nm - tri(m+1) further
          int step = 2 * (nm - 1);
          const int so = tri(l);
          T re[G], im[G];
#pragma unroll
          for (int g = 0; g < G; ++g) re[g] = im[g] = 0;
#pragma unroll 2
          for (int m = 0; m <= l; ++m, e += step, step -= 2 * (m + 1)) {
            const T ee = e[0], eo = e[1];
#pragma unroll
            for (int g = 0; g < G; ++g) {
              cplx<T> x = cbuf[g * (nm + nl) + so + m];
              re[g] += ee * x.re;
              im[g] += eo * x.im;
            }
          }
#pragma unroll
          for (int g = 0; g < G; ++g) cbuf[g * (nm + nl) + nl + c] = cmake<T>(re[g], im[g]);
        }
      }
      __syncwarp();
      // translation along z (m-major lanes)
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int k = lane + 32 * r;
        if (k < nl) {
          const int m = vmap[2 * k + 1];
          // vertical factor times radial power for source degree n: row n of vv
          const T *vcol = tb + D.vv + m2l_vrow_off(p, m) + k;
          int vstep = m2l_vrow_len(p, m);
          T re[G], im[G];
#pragma unroll
          for (int g = 0; g < G; ++g) re[g] = im[g] = 0;
#pragma unroll 2
          for (int n = m; n < p; ++n, vcol += vstep, vstep += p + 1 - n) {
            const T f = vcol[0];
            const int sidx = nl + tri(n, m);
#pragma unroll
            for (int g = 0; g < G; ++g) {
              cplx<T> a = cbuf[g * (nm + nl) + sidx];
              re[g] += f * a.re;
              im[g] += f * a.im;
            }
          }
#pragma unroll
          for (int g = 0; g < G; ++g) cbuf[g * (nm + nl) + k] = cmake<T>(re[g], im[g]);
        }
      }
      __syncwarp();
      prefetch();   // rot region is free until the next phase stage
      // rotation back (degrees <= p), conjugate z-phase, accumulate
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int c = lane + 32 * r;
        if (c < nl) {
          const int l = lm[2 * c], mp = lm[2 * c + 1];
          const T *e = EOi + 2 * c;        // plane 0; plane m+1 is nl - tri(m+1) further
          int step = 2 * (nl - 1);
          T re[G], im[G];
#pragma unroll
          for (int g = 0; g < G; ++g) re[g] = im[g] = 0;
          // slot of (l, m) in m-major order: m(p+1) - m(m-1)/2 + (l - m)
          int slot = l;
#pragma unroll 2
          for (int m = 0; m <= l; ++m, e += step, step -= 2 * (m + 1)) {
            const T ee = e[0], eo = e[1];
#pragma unroll
            for (int g = 0; g < G; ++g) {
              cplx<T> x = cbuf[g * (nm + nl) + slot];
              re[g] += ee * x.re;
              im[g] += eo * x.im;
            }
            slot += p - m;                   // (l, m+1)
          }
          T cr = ph[2 * mp], ci = -ph[2 * mp + 1];
#pragma unroll
          for (int g = 0; g < G; ++g) {
            acc[g][r].re += re[g] * cr - im[g] * ci;
            acc[g][r].im += re[g] * ci + im[g] * cr;
          }
        }
      }
    }
    __syncwarp();
    if (NST > 0 && lane == 0) mbar_arrive(&empty[b]);
  }
  cp_async_wait_all();   // source copies still in flight after an early stop
  if (nact > 0) {
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (!tvalid[g]) continue;
      const T ih = (T)(ldexp(1.0, depth[tg[g]]) / scale_e);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        int c = lane + 32 * r;
        if (c < nl) loc[(size_t)tg[g] * nl + c] = cmake<T>(acc[g][r].re * ih, acc[g][r].im * ih);
      }
    }
  }
}

bool g_codes_ready[64] = {};

void upload_codes(int device) {
  if (device >= 0 && device < 64 && g_codes_ready[device]) return;
  uint16_t codes[316];
  int8_t vec[316 * 3];
  int k = 0;
  for (int dz = -3; dz <= 3; ++dz)
    for (int dy = -3; dy <= 3; ++dy)
      for (int dx = -3; dx <= 3; ++dx) {
        if (dx >= -1 && dx <= 1 && dy >= -1 && dy <= 1 && dz >= -1 && dz <= 1) continue;
        codes[k] = (uint16_t)((dx + 3) + 7 * (dy + 3) + 49 * (dz + 3));
        vec[3 * k] = (int8_t)dx;
        vec[3 * k + 1] = (int8_t)dy;
        vec[3 * k + 2] = (int8_t)dz;
        ++k;
      }
  ACHECK(cudaMemcpyToSymbol(c_dir_codes, codes, sizeof(codes)));
  ACHECK(cudaMemcpyToSymbol(c_dir_vec, vec, sizeof(vec)));
  if (device >= 0 && device < 64) g_codes_ready[device] = true;
}

template <typename T, int NST, int G>
size_t m2l_smem(int p, int stride) {
  int nm = tri(p), nl = tri(p + 1);
  size_t off = (size_t)NST * stride * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  off += 2 * NST * sizeof(uint64_t);
  off = (off + 15) & ~(size_t)15;
  off += (size_t)kSibWarps * G * (nm + nl) * sizeof(cplx<T>);
  off += (size_t)G * 216 * sizeof(int) + 10 * sizeof(unsigned) + 320 * sizeof(uint16_t) + 4 * nl;
  return off + 64;
}

template <typename T, int NST, int R, int G>
bool try_launch(AranGpuSolver3d *s, OpTables<T> &tb, const M2LOffsets &D, const int *parents,
                int count, const cplx<T> *mult, cplx<T> *loc, cudaStream_t st, int dev_smem) {
  DevTree &t = s->tree;
  const int p = s->cfg.order;
  size_t sm = m2l_smem<T, NST, G>(p, D.stride);
  if ((int)sm > dev_smem) return false;
  smem_opt_in(k_m2l_sibling<T, NST, R, G>, sm);
  k_m2l_sibling<T, NST, R, G><<<ceil_div(count, G), 32 * (kSibWarps + 1), sm, st>>>(
      count, parents, t.child.ptr, t.begin.ptr, t.end.ptr, t.col.ptr, t.ncol.ptr,
      t.ijk.ptr, t.depth.ptr, p, tb.dir_m2l.ptr, D, tb.lm.ptr, s->scale_e, mult, loc,
      s->err_dev.ptr, consumer_wait_polls());
  ACHECK(cudaGetLastError());
  s->launches++;
  return true;
}

template <typename T>
void launch_t(AranGpuSolver3d *s, OpTables<T> &tb, const int *parents, int count,
              const cplx<T> *mult, cplx<T> *loc, cudaStream_t st) {
  if (count <= 0) return;
  const int kern = m2l_kernel_choice(s);
  if constexpr (sizeof(T) == 4) {
    if (kern == ARAN_M2L_TENSOR &&
        launch_m2l_tc(s, parents, count, reinterpret_cast<const float *>(mult),
                      reinterpret_cast<float *>(loc), st))
      return;
    if (kern != ARAN_M2L_SIBLING && launch_m2l_lanes(s, tb, parents, count, mult, loc, st)) return;
  }
  upload_codes(s->device);
  const int p = s->cfg.order;
  M2LOffsets D;
  D.ef = dir_offset(p, 0, 0);
  D.ei = dir_offset(p, 0, 2);
  D.ph = dir_offset(p, 0, 4);
  D.rp = dir_offset(p, 0, 5);
  D.vv = dir_offset(p, 0, 7);
  D.stride = dir_offset(p, 0, 6);
  int dev_smem = 0;
  ACHECK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  // R = rounds of 32 lanes over the tri(p+1) local coefficients; G parents
  // per CTA (each warp takes child w of every one of them)
  const int nl = tri(p + 1);
  // a sibling configuration set on the solver (FP32 part), when it serves nl
  if (sizeof(T) == 4 && s->m2l_nst > 0 && s->m2l_g > 0) {
    const int nst = s->m2l_nst, g = s->m2l_g;
    bool ok = false;
#define ARAN_TRY(NST_, R_, G_)                                                               \
  if (!ok && nst == NST_ && g == G_)                                                         \
    ok = try_launch<T, NST_, R_, G_>(s, tb, D, parents, count, mult, loc, st, dev_smem);
    if (nl <= 96) {
      ARAN_TRY(1, 3, 1) ARAN_TRY(2, 3, 1) ARAN_TRY(3, 3, 1)
      ARAN_TRY(1, 3, 2) ARAN_TRY(2, 3, 2) ARAN_TRY(3, 3, 2)
    } else if (nl <= 160) {
      ARAN_TRY(1, 5, 1) ARAN_TRY(2, 5, 1) ARAN_TRY(3, 5, 1)
      ARAN_TRY(1, 5, 2) ARAN_TRY(2, 5, 2)
    }
#undef ARAN_TRY
    if (ok) return;
  }
  // (two table slots keep a p <= 12 FP32 CTA under a third of the shared
  // memory, so three CTAs share an SM)
  if (nl <= 96) {
    if (sizeof(T) == 8 && try_launch<T, 3, 3, 2>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 2, 3, 2>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 1, 3, 2>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 1, 3, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
  } else if (nl <= 160) {
    if (try_launch<T, 1, 5, 2>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 1, 5, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
  } else if (nl <= 256) {
    if (try_launch<T, 3, 8, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 1, 8, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 0, 8, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
  } else {
    if (try_launch<T, 1, kMaxRounds, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
    if (try_launch<T, 0, kMaxRounds, 1>(s, tb, D, parents, count, mult, loc, st, dev_smem)) return;
  }
  throw CudaError{cudaErrorInvalidConfiguration, "M2L shared memory exceeds the device limit"};
}

}  // namespace

int m2l_kernel_choice(const AranGpuSolver3d *s) {
  if (s->m2l_kernel != ARAN_M2L_AUTO) return s->m2l_kernel;
  const char *pick = getenv("ARAN_M2L_KERNEL");
  if (pick && strcmp(pick, "sibling") == 0) return ARAN_M2L_SIBLING;
  if (pick && strcmp(pick, "lanes") == 0) return ARAN_M2L_LANES;
  if (pick && strcmp(pick, "tc") == 0) return ARAN_M2L_TENSOR;
  return ARAN_M2L_AUTO;
}

int m2l_sibling_configs(int p, int *nst, int *g, int k) {
  static const int small[6][2] = {{1, 1}, {2, 1}, {3, 1}, {1, 2}, {2, 2}, {3, 2}};
  static const int mid[5][2] = {{1, 1}, {2, 1}, {3, 1}, {1, 2}, {2, 2}};
  const int nl = tri(p + 1);
  const int (*tab)[2] = nl <= 96 ? small : (nl <= 160 ? mid : nullptr);
  const int count = nl <= 96 ? 6 : (nl <= 160 ? 5 : 0);
  if (tab && k >= 0 && k < count) {
    *nst = tab[k][0];
    *g = tab[k][1];
  }
  return count;
}

void launch_m2l(AranGpuSolver3d *s, bool fp64, int first, int count, cudaStream_t st) {
  const int *parents = s->tree.parents.ptr + first;
  if (!fp64)
    launch_t<float>(s, s->t32, parents, count,
                    reinterpret_cast<const cplx<float> *>(s->mult32.ptr),
                    reinterpret_cast<cplx<float> *>(s->loc32.ptr), st);
  else
    launch_t<double>(s, s->t64, parents, count,
                     reinterpret_cast<const cplx<double> *>(s->mult64.ptr),
                     reinterpret_cast<cplx<double> *>(s->loc64.ptr), st);
}

}  // namespace aran
