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
// the error word and the CTA stops issuing copies.
#include "internal.cuh"

namespace aran {

int dir_offset(int p, int kind, int what);

namespace {

__constant__ uint16_t c_dir_codes[316];
__constant__ int8_t c_dir_vec[316 * 3];

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mb)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mb, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mb)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *mb) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mb))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *mb, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: gives up after ~1M polls (each poll may itself suspend)
__device__ __forceinline__ bool mbar_wait(uint64_t *mb, uint32_t parity) {
  for (int i = 0; i < (1 << 20); ++i)
    if (mbar_try_wait(mb, parity)) return true;
  return false;
}

struct M2LOffsets {
  int ef, ei, ph, rp, stride;  // in T units; ef/ei interleaved (E, O) pairs
};

template <typename T, int NBUF>
__global__ void __launch_bounds__(256) k_m2l_sibling(
    int nparents, const int *__restrict__ parents, const int *__restrict__ child,
    const int *__restrict__ begin, const int *__restrict__ end, const int *__restrict__ col,
    const int *__restrict__ ncol, const int *__restrict__ ijk, const uint8_t *__restrict__ depth,
    int p, const T *__restrict__ dirs, M2LOffsets D, const T *__restrict__ vt_g,
    const uint8_t *__restrict__ lm_g, double scale_e, const cplx<T> *__restrict__ mult,
    cplx<T> *__restrict__ loc, int *__restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int nm = tri(p), nl = tri(p + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // shared layout: tables | mbarriers | vt | warp buffers | grid | mask | active | lm
  size_t off = 0;
  T *tab = reinterpret_cast<T *>(smem_raw);
  off += (size_t)NBUF * D.stride * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(smem_raw + off);
  off += 2 * sizeof(uint64_t);
  T *vt = reinterpret_cast<T *>(smem_raw + off);
  off += (size_t)nl * p * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  cplx<T> *wbuf = reinterpret_cast<cplx<T> *>(smem_raw + off);
  off += (size_t)8 * (2 * nm + nl) * sizeof(cplx<T>);
  int *grid = reinterpret_cast<int *>(smem_raw + off);
  off += 216 * sizeof(int);
  unsigned *mask = reinterpret_cast<unsigned *>(smem_raw + off);
  off += 10 * sizeof(unsigned);
  uint16_t *active = reinterpret_cast<uint16_t *>(smem_raw + off);
  off += 320 * sizeof(uint16_t);
  __shared__ int s_nact;

  const int P = parents[blockIdx.x];
  const int c0 = child[P];
  // source grid: children of P's internal colleagues, 6x6x6 cells
  for (int i = threadIdx.x; i < 216; i += blockDim.x) grid[i] = -1;
  if (threadIdx.x < 10) mask[threadIdx.x] = 0u;
  for (int i = threadIdx.x; i < nl * p; i += blockDim.x) vt[i] = vt_g[i];
  if (threadIdx.x == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
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
    grid[gx + 6 * (gy + 6 * gz)] = s;
  }
  __syncthreads();
  // my target (warp-uniform)
  const int t = c0 + w;
  const bool tvalid = end[t] > begin[t];
  const int tx = 2 + (w & 1), ty = 2 + ((w >> 1) & 1), tz = 2 + ((w >> 2) & 1);
  auto source_of = [&](int di) -> int {
    int cx = tx - c_dir_vec[3 * di], cy = ty - c_dir_vec[3 * di + 1], cz = tz - c_dir_vec[3 * di + 2];
    if (cx < 0 || cx > 5 || cy < 0 || cy > 5 || cz < 0 || cz > 5) return -1;
    return grid[cx + 6 * (cy + 6 * cz)];
  };
  if (tvalid)
    for (int di = lane; di < 316; di += 32)
      if (source_of(di) >= 0) atomicOr(&mask[di >> 5], 1u << (di & 31));
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

  // per-lane output coefficients
  constexpr int KMAX = ((kMaxOrder + 1) * (kMaxOrder + 2) / 2 + 31) / 32;
  cplx<T> acc[KMAX];
#pragma unroll
  for (int k = 0; k < KMAX; ++k) acc[k] = cmake<T>(0, 0);
  cplx<T> *src = wbuf + (size_t)w * (2 * nm + nl);
  cplx<T> *rot = src + nm;
  cplx<T> *tr = rot + nm;

  bool ok = true;
  if (threadIdx.x == 0 && nact > 0) {
    mbar_expect_tx(&mbar[0], tbytes);
    bulk_g2s(tab, dirs + (size_t)c_dir_codes[active[0]] * D.stride, tbytes, &mbar[0]);
  }
  for (int i = 0; i < nact; ++i) {
    const int b = NBUF == 2 ? (i & 1) : 0;
    const uint32_t parity = NBUF == 2 ? ((i >> 1) & 1) : (i & 1);
    if (NBUF == 2 && threadIdx.x == 0 && i + 1 < nact) {
      mbar_expect_tx(&mbar[b ^ 1], tbytes);
      bulk_g2s(tab + (size_t)(b ^ 1) * D.stride,
               dirs + (size_t)c_dir_codes[active[i + 1]] * D.stride, tbytes, &mbar[b ^ 1]);
    }
    if (!mbar_wait(&mbar[b], parity)) {
      ok = false;
      atomicExch(err, 1);
    }
    if (__syncthreads_or(!ok)) {
      // a table never arrived: wait (bounded) for the other copy in flight, then stop
      if (NBUF == 2 && threadIdx.x == 0 && i + 1 < nact) mbar_wait(&mbar[b ^ 1], ((i + 1) >> 1) & 1);
      __syncthreads();
      return;
    }
    const T *tb = tab + (size_t)b * D.stride;
    const int s = tvalid ? source_of(active[i]) : -1;
    if (s >= 0) {
      const T *ph = tb + D.ph;
      const T *EOf = tb + D.ef;
      const T *EOi = tb + D.ei;
      const T *rp = tb + D.rp;
      for (int c = lane; c < nm; c += 32) {
        cplx<T> v = mult[(size_t)s * nm + c];
        int m = lm_g[2 * c + 1];
        T cr = ph[2 * m], ci = ph[2 * m + 1];
        src[c] = cmake<T>(v.re * cr - v.im * ci, v.re * ci + v.im * cr);
      }
      __syncwarp();
      for (int c = lane; c < nm; c += 32) {
        int l = lm_g[2 * c], mp = lm_g[2 * c + 1];
        const T *row = EOf + 2 * (sq_off(l) + mp * (l + 1));
        const cplx<T> *sv = src + tri(l);
        T re = 0, im = 0;
        for (int m = 0; m <= l; ++m) {
          cplx<T> x = sv[m];
          re += row[2 * m] * x.re;
          im += row[2 * m + 1] * x.im;
        }
        rot[c] = cmake<T>(re, im);
      }
      __syncwarp();
      for (int c = lane; c < nl; c += 32) {
        int l = lm_g[2 * c], m = lm_g[2 * c + 1];
        const T *vrow = vt + c * p;
        T re = 0, im = 0;
        for (int n = m; n < p; ++n) {
          T f = vrow[n] * rp[l + n + 1];
          cplx<T> r = rot[tri(n, m)];
          re += f * r.re;
          im += f * r.im;
        }
        tr[c] = cmake<T>(re, im);
      }
      __syncwarp();
#pragma unroll
      for (int k = 0; k < KMAX; ++k) {
        int c = lane + 32 * k;
        if (c < nl) {
          int l = lm_g[2 * c], mp = lm_g[2 * c + 1];
          const T *row = EOi + 2 * (sq_off(l) + mp * (l + 1));
          const cplx<T> *sv = tr + tri(l);
          T re = 0, im = 0;
          for (int m = 0; m <= l; ++m) {
            cplx<T> x = sv[m];
            re += row[2 * m] * x.re;
            im += row[2 * m + 1] * x.im;
          }
          T cr = ph[2 * mp], ci = -ph[2 * mp + 1];
          acc[k].re += re * cr - im * ci;
          acc[k].im += re * ci + im * cr;
        }
      }
      __syncwarp();
    }
    __syncthreads();  // everyone is done with buffer b before it is refilled
    if (NBUF == 1 && threadIdx.x == 0 && i + 1 < nact) {
      mbar_expect_tx(&mbar[0], tbytes);
      bulk_g2s(tab, dirs + (size_t)c_dir_codes[active[i + 1]] * D.stride, tbytes, &mbar[0]);
    }
  }
  if (tvalid && nact > 0) {
    const T ih = (T)(ldexp(1.0, depth[t]) / scale_e);
#pragma unroll
    for (int k = 0; k < KMAX; ++k) {
      int c = lane + 32 * k;
      if (c < nl) loc[(size_t)t * nl + c] = cmake<T>(acc[k].re * ih, acc[k].im * ih);
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

template <typename T, int NBUF>
size_t m2l_smem(int p, int stride) {
  int nm = tri(p), nl = tri(p + 1);
  size_t off = (size_t)NBUF * stride * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  off += 2 * sizeof(uint64_t);
  off += (size_t)nl * p * sizeof(T);
  off = (off + 15) & ~(size_t)15;
  off += (size_t)8 * (2 * nm + nl) * sizeof(cplx<T>);
  off += 216 * sizeof(int) + 10 * sizeof(unsigned) + 320 * sizeof(uint16_t);
  return off + 64;
}

template <typename T>
void launch_t(AranGpuSolver3d *s, OpTables<T> &tb, const cplx<T> *mult, cplx<T> *loc,
              cudaStream_t st) {
  DevTree &t = s->tree;
  if (t.n_parents == 0) return;
  upload_codes(s->device);
  const int p = s->cfg.order;
  M2LOffsets D;
  D.ef = dir_offset(p, 0, 0);
  D.ei = dir_offset(p, 0, 2);
  D.ph = dir_offset(p, 0, 4);
  D.rp = dir_offset(p, 0, 5);
  D.stride = dir_offset(p, 0, 6);
  int dev_smem = 0;
  ACHECK(cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device));
  size_t sm2 = m2l_smem<T, 2>(p, D.stride);
  size_t sm1 = m2l_smem<T, 1>(p, D.stride);
  ACHECK(cudaMemsetAsync(s->err_dev.ptr, 0, sizeof(int), st));
  if ((int)sm2 <= dev_smem) {
    ACHECK(cudaFuncSetAttribute(k_m2l_sibling<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm2));
    k_m2l_sibling<T, 2><<<t.n_parents, 256, sm2, st>>>(
        t.n_parents, t.parents.ptr, t.child.ptr, t.begin.ptr, t.end.ptr, t.col.ptr, t.ncol.ptr,
        t.ijk.ptr, t.depth.ptr, p, tb.dir_m2l.ptr, D, tb.vt.ptr, tb.lm.ptr, s->scale_e, mult, loc,
        s->err_dev.ptr);
  } else {
    if ((int)sm1 > dev_smem) throw CudaError{cudaErrorInvalidConfiguration, "M2L shared memory exceeds the device limit"};
    ACHECK(cudaFuncSetAttribute(k_m2l_sibling<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm1));
    k_m2l_sibling<T, 1><<<t.n_parents, 256, sm1, st>>>(
        t.n_parents, t.parents.ptr, t.child.ptr, t.begin.ptr, t.end.ptr, t.col.ptr, t.ncol.ptr,
        t.ijk.ptr, t.depth.ptr, p, tb.dir_m2l.ptr, D, tb.vt.ptr, tb.lm.ptr, s->scale_e, mult, loc,
        s->err_dev.ptr);
  }
  ACHECK(cudaGetLastError());
  s->launches++;
}

}  // namespace

void launch_m2l(AranGpuSolver3d *s, cudaStream_t st) {
  if (s->cfg.precision == ARAN_PRECISION_MIXED)
    launch_t<float>(s, s->t32, reinterpret_cast<const cplx<float> *>(s->mult32.ptr),
                    reinterpret_cast<cplx<float> *>(s->loc32.ptr), st);
  else
    launch_t<double>(s, s->t64, reinterpret_cast<const cplx<double> *>(s->mult64.ptr),
                     reinterpret_cast<cplx<double> *>(s->loc64.ptr), st);
}

}  // namespace aran
