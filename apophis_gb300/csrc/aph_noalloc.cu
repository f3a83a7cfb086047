// aph_noalloc.cu -- EstimateTimestep for one meshblock that allocates nothing.
//
// Some callers cannot allocate device memory at the moment they need a timestep: a host
// code that hands all of its device memory to its own pool allocator up front (a Kokkos
// or Parthenon application sized to the GPU) has none left for cudaMalloc, and a call of
// cudaMalloc or cudaFree in the middle of its step would also synchronise the device.  This
// entry point keeps its scratch -- one partial minimum per CTA -- in a file-scope device
// array, so that neither it nor anything it calls allocates.  The array lives as long as
// the library is loaded, on every GPU that loads it.
#include <cuda.h>

#include <cfloat>
#include <mutex>

#include "../../include/aph_hydro.h"
#include "aph_capi_internal.h"
#include "aph_math.cuh"

using namespace aph;

namespace {

constexpr int kThreads = 256;
constexpr int kMaxCtas = APH_NOALLOC_MAX_CELLS / kThreads;
constexpr int kMaxDevices = 64;

// Shared by every call on a device; each call overwrites the first nctas entries.
static __device__ __align__(256) unsigned long long g_dt_partials[kMaxCtas];

// The driver's context queries, taken through the runtime (no link against libcuda).
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

struct DeviceScratch {
  std::mutex mu;
  CtxGetCurrentFn ctx_current = nullptr;
  CtxGetIdFn ctx_id = nullptr;
  bool looked_up = false;
  unsigned long long *ptr[kMaxDevices] = {};
  unsigned long long ctx[kMaxDevices] = {};  // the context the address belongs to
};
DeviceScratch g_scratch;

// Identity of the calling thread's current context (0 if none or unknown).
unsigned long long current_context_id() {
  if (!g_scratch.looked_up) {
    g_scratch.looked_up = true;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_scratch.ctx_current = (CtxGetCurrentFn)fn;
    fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &fn, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      g_scratch.ctx_id = (CtxGetIdFn)fn;
  }
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!g_scratch.ctx_current || !g_scratch.ctx_id || g_scratch.ctx_current(&c) != CUDA_SUCCESS || !c)
    return 0;
  if (g_scratch.ctx_id(c, &id) != CUDA_SUCCESS) return 0;
  return id;
}

// Device address of g_dt_partials on the current device.  It is looked up on the first call
// there, and again whenever the device's context is no longer the one it was looked up in
// (after cudaDeviceReset the library's module is loaded anew, at a new address).
aph_status scratch_for_current_device(unsigned long long **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "estimate_timestep_noalloc");
  if (dev < 0 || dev >= kMaxDevices) return fail(APH_ERR_UNSUPPORTED, "device ordinal %d too large", dev);
  std::lock_guard<std::mutex> lock(g_scratch.mu);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch.ptr[dev] || ctx == 0 || ctx != g_scratch.ctx[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_dt_partials);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_dt_partials)");
    g_scratch.ptr[dev] = (unsigned long long *)p;
    g_scratch.ctx[dev] = current_context_id();  // the lookup made the context current
  }
  *out = g_scratch.ptr[dev];
  return APH_OK;
}

struct OneBlock {
  const double *prim, *cons;
  int nx[3], ni, nj, ng, ndim;
  long long ncell;
  double dx[3], gm1;
};

// Per CTA: the minimum candidate's bit pattern (all ones when the CTA has no cell).
__global__ void __launch_bounds__(kThreads) k_dt_partials(OneBlock b, unsigned long long *partials) {
  __shared__ unsigned long long red[kThreads / 32];
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v = ~0ULL;
  if (idx < b.nx[0] * b.nx[1] * b.nx[2]) {
    const int i = idx % b.nx[0], j = (idx / b.nx[0]) % b.nx[1], k = idx / (b.nx[0] * b.nx[1]);
    const int sj = b.ndim >= 2 ? b.ng : 0, sk = b.ndim >= 3 ? b.ng : 0;
    const long long c = ((long long)(k + sk) * b.nj + (j + sj)) * b.ni + (i + b.ng);
    double w[NHYDRO];
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) w[n] = b.prim[n * b.ncell + c];
    const double m = dt_candidate(w, b.cons[IEN * b.ncell + c], b.dx, b.ndim, b.gm1);
    v = is_neg(m) ? ~0ULL : (unsigned long long)__double_as_longlong(m);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < kThreads / 32 ? red[threadIdx.x] : ~0ULL;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
      v = x < v ? x : v;
    }
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
  }
}

__global__ void __launch_bounds__(kThreads) k_dt_reduce(const unsigned long long *partials, int n,
                                                        double cfl, double *dt_out) {
  __shared__ unsigned long long red[kThreads / 32];
  unsigned long long v = ~0ULL;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = partials[i] < v ? partials[i] : v;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kThreads / 32; ++w) v = red[w] < v ? red[w] : v;
    v = red[0] < v ? red[0] : v;
    const double m = (v == ~0ULL) ? DBL_MAX : __longlong_as_double((long long)v);
    dt_out[0] = cfl * m;
  }
}

}  // namespace

extern "C" aph_status aph_hydro_estimate_timestep_noalloc(const double *prim, const double *cons,
                                                          const int nx[3], int nghost, int ndim,
                                                          const double dx[3], double gm1,
                                                          double cfl, double *dt_dev,
                                                          void *stream) {
  clear_error();
  if (!prim || !cons || !nx || !dx || !dt_dev) return fail(APH_ERR_INVALID, "NULL argument");
  if (ndim < 1 || ndim > 3) return fail(APH_ERR_INVALID, "ndim %d not in 1..3", ndim);
  if (nghost < 1) return fail(APH_ERR_INVALID, "nghost must be >= 1");
  long long cells = 1;
  for (int d = 0; d < 3; ++d) {
    if (d < ndim ? nx[d] < 1 : nx[d] != 1) return fail(APH_ERR_INVALID, "nx%d = %d invalid", d + 1, nx[d]);
    if (!(dx[d] > 0.0)) return fail(APH_ERR_INVALID, "dx%d must be positive", d + 1);
    cells *= nx[d];  // at most 2^20 * 2^31 after a passed check: no overflow
    if (cells > APH_NOALLOC_MAX_CELLS)
      return fail(APH_ERR_INVALID,
                  "meshblock of %d x %d x %d interior cells; the allocation-free estimate takes at "
                  "most %d", nx[0], nx[1], nx[2], APH_NOALLOC_MAX_CELLS);
  }
  if (!(gm1 > 0.0) || !(cfl > 0.0)) return fail(APH_ERR_INVALID, "gm1 and cfl must be positive");
  unsigned long long *partials = nullptr;
  if (aph_status st = scratch_for_current_device(&partials)) return st;
  OneBlock b;
  b.prim = prim;
  b.cons = cons;
  for (int d = 0; d < 3; ++d) {
    b.nx[d] = nx[d];
    b.dx[d] = dx[d];
  }
  b.ng = nghost;
  b.ndim = ndim;
  b.ni = nx[0] + 2 * nghost;
  b.nj = ndim >= 2 ? nx[1] + 2 * nghost : 1;
  const long long nk = ndim >= 3 ? nx[2] + 2 * nghost : 1;
  b.ncell = (long long)b.ni * b.nj * nk;
  b.gm1 = gm1;
  const int nctas = (int)((cells + kThreads - 1) / kThreads);
  cudaStream_t s = (cudaStream_t)stream;
  k_dt_partials<<<nctas, kThreads, 0, s>>>(b, partials);
  k_dt_reduce<<<1, kThreads, 0, s>>>(partials, nctas, cfl, dt_dev);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "estimate_timestep_noalloc");
}
