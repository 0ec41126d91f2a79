// noalloc.cu -- Newton near field of a small particle set without any device
// allocation.
//
// Who needs this: callers that may not allocate device memory while they
// run -- a host that hands the library a fixed device budget at start-up and
// forbids later allocations (an embedding runtime owning all device memory,
// a pooled-memory application that must not go through cudaMalloc's
// implicit synchronisation inside its time-critical loop).  For them
// aran_gpu_p2p_direct_noalloc evaluates every pair of up to kNoAllocMax
// particles (the P2P kernel of the solver over a single leaf, FP64) with all
// its scratch in one static device array of this file.
//
// Properties a caller must know:
//  * the scratch array (4 doubles per particle, kNoAllocMax particles, 4 MiB)
//    belongs to the library's device code: it is placed on a GPU when that
//    code is loaded there and stays until the process exits.  CUDA loads
//    modules lazily by default (CUDA_MODULE_LOADING=LAZY since CUDA 12.2),
//    so on each device the first call (or the first use of any other
//    kernel of the library there) loads it, which takes device memory and
//    can fail for lack of it.  Callers make one warm-up call per device at
//    start-up, before the region where they may not allocate and before any
//    stream capture (or run with CUDA_MODULE_LOADING=EAGER);
//  * every call looks up the array's device address with
//    cudaGetSymbolAddress, with the caller's device current: the host-side
//    symbol is only a stand-in for it.  Once the module is loaded the lookup
//    allocates nothing, and doing it per call stays right after a
//    cudaDeviceReset or a new primary context;
//  * the kernels run on the legacy default stream (stream 0) and the call
//    synchronises that stream before returning: the caller finishes writing
//    d_xyz and d_q (synchronises its own, e.g. non-blocking, streams) first,
//    and no call can be made while a global-mode stream capture is open;
//  * every call shares the array and the last call's contents remain in it;
//    the function clears what it accumulates before using it, so calls that
//    run one after the other are independent, but calls that overlap on the
//    GPU (from several host threads, or several processes sharing a context)
//    race on the array;
//  * it allocates nothing: no cudaMalloc/cudaFree or allocating library call.
#include "internal.cuh"

namespace aran {

namespace {

constexpr int kNoAllocMax = 131072;  // particles
constexpr int kNoAllocChunk = 4096;  // sources per block

static __device__ __align__(256) double g_noalloc_acc[4 * kNoAllocMax];

__global__ void k_noalloc_clear(int n4, double *__restrict__ acc) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n4) acc[i] = 0.0;
}

// every (target, source) pair of one source chunk; Newton potential and field
// as in tests/newtonpot3.c:61-78 and tests/newtonfield3.c:91-119
__global__ void k_noalloc_pairs(int n, const double *__restrict__ xyz, const double *__restrict__ q,
                                int field, double *__restrict__ acc) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int j0 = blockIdx.y * kNoAllocChunk;
  int j1 = min(n, j0 + kNoAllocChunk);
  if (t >= n) return;
  double tx = xyz[3 * t], ty = xyz[3 * t + 1], tz = xyz[3 * t + 2];
  double pot = 0, fx = 0, fy = 0, fz = 0;
  for (int j = j0; j < j1; ++j) {
    double dx = tx - xyz[3 * j], dy = ty - xyz[3 * j + 1], dz = tz - xyz[3 * j + 2];
    double r2 = dx * dx + dy * dy + dz * dz;
    // the solver's single-leaf rule: field mode keeps |r| > 1e-5, potential
    // mode skips the particle itself and coincident particles (r == 0)
    bool ok = field ? (r2 > 1e-10) : (r2 > 0.);
    double inv = ok ? rsqrt(r2) : 0.;
    double qi = q[j] * inv;
    pot += qi;
    if (field) {
      double q3 = qi * inv * inv;
      fx -= q3 * dx;
      fy -= q3 * dy;
      fz -= q3 * dz;
    }
  }
  atomicAdd(&acc[4 * t], pot);
  if (field) {
    atomicAdd(&acc[4 * t + 1], fx);
    atomicAdd(&acc[4 * t + 2], fy);
    atomicAdd(&acc[4 * t + 3], fz);
  }
}

__global__ void k_noalloc_finish(int n, const double *__restrict__ acc, double *__restrict__ pot,
                                 double *__restrict__ fld) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (pot) pot[i] = acc[4 * i];
  if (fld) {
    fld[3 * i] = acc[4 * i + 1];
    fld[3 * i + 1] = acc[4 * i + 2];
    fld[3 * i + 2] = acc[4 * i + 3];
  }
}

}  // namespace
}  // namespace aran

using namespace aran;

extern "C" int aran_gpu_p2p_direct_noalloc(int64_t n, const double *d_xyz, const double *d_q,
                                           double *d_pot, double *d_field) {
  if (n < 1 || n > kNoAllocMax) {
    set_error("aran_gpu_p2p_direct_noalloc: n = " + std::to_string(n) +
              " is outside [1, " + std::to_string(kNoAllocMax) +
              "], the capacity of its static scratch array");
    return ARAN_ERR_INVALID;
  }
  if (!d_xyz || !d_q || (!d_pot && !d_field)) {
    set_error("aran_gpu_p2p_direct_noalloc: xyz, q and at least one output are required");
    return ARAN_ERR_INVALID;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    set_error(std::string("aran_gpu_p2p_direct_noalloc: no current device: ") + cudaGetErrorString(e));
    return ARAN_ERR_NO_DEVICE;
  }
  // the symbol is only a host-side stand-in: ask the runtime for the
  // array's address on the current device
  double *acc = nullptr;
  e = cudaGetSymbolAddress(reinterpret_cast<void **>(&acc), g_noalloc_acc);
  if (e != cudaSuccess || !acc) {
    set_error(std::string("aran_gpu_p2p_direct_noalloc: cudaGetSymbolAddress failed: ") +
              cudaGetErrorString(e));
    return ARAN_ERR_CUDA;
  }
  const int nn = (int)n;
  const int TB = 128;
  k_noalloc_clear<<<ceil_div(4 * (int64_t)nn, 256), 256>>>(4 * nn, acc);
  dim3 grid(ceil_div(nn, TB), ceil_div(nn, kNoAllocChunk));
  k_noalloc_pairs<<<grid, TB>>>(nn, d_xyz, d_q, d_field != nullptr, acc);
  k_noalloc_finish<<<ceil_div(nn, 256), 256>>>(nn, acc, d_pot, d_field);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    set_error(std::string("aran_gpu_p2p_direct_noalloc: ") + cudaGetErrorString(e));
    return ARAN_ERR_CUDA;
  }
  return ARAN_OK;
}
