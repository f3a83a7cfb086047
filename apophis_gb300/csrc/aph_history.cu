// aph_history.cu -- history sums of the hydro package: total mass and total energy,
// sum over interior cells of U * CellVolume (GlobalQuantHst<Sum, IDN / IEN>,
// src/hydro/hydro.cpp:336-346, 754-771).  Deterministic: every CTA reduces its cells in a
// fixed tree order into one partial, and one CTA sums the partials in a fixed order.
#include "aph_capi_internal.h"

namespace aph {
namespace {

constexpr int kHistThreads = 256;

struct ConsOf {
  __device__ const double *operator()(const BlockDev &B) const { return B.cons; }
};
struct U0Of {
  __device__ const double *operator()(const StepBlock &B) const { return B.u0; }
};

template <class BLK, class Q>
__global__ void __launch_bounds__(kHistThreads) k_history(const BLK *blocks, int block0, int ng, int ndim,
                                                          Q q, double *partials) {
  __shared__ double sm[2][kHistThreads];
  const BLK &B = blocks[block0 + blockIdx.y];
  const int nint = B.nx[0] * B.nx[1] * B.nx[2];
  const int idx = blockIdx.x * kHistThreads + threadIdx.x;
  double m = 0.0, e = 0.0;
  if (idx < nint) {
    const int i = idx % B.nx[0], j = (idx / B.nx[0]) % B.nx[1], k = idx / (B.nx[0] * B.nx[1]);
    const int sj = ndim >= 2 ? ng : 0, sk = ndim >= 3 ? ng : 0;
    const long long c = ((long long)(k + sk) * B.nj + (j + sj)) * B.ni + (i + ng);
    const double vol = B.dx[0] * B.dx[1] * B.dx[2];
    const double *u = q(B);
    m = u[c] * vol;                      // IDN
    e = u[4 * B.ncell + c] * vol;        // IEN
  }
  sm[0][threadIdx.x] = m;
  sm[1][threadIdx.x] = e;
  __syncthreads();
  for (int s = kHistThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
      sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const size_t o = 2 * ((size_t)blockIdx.y * gridDim.x + blockIdx.x);
    partials[o] = sm[0][0];
    partials[o + 1] = sm[1][0];
  }
}

__global__ void __launch_bounds__(kHistThreads) k_history_finish(const double *partials, long long n,
                                                                 double *out) {
  __shared__ double sm[2][kHistThreads];
  double m = 0.0, e = 0.0;
  for (long long i = threadIdx.x; i < n; i += kHistThreads) {
    m += partials[2 * i];
    e += partials[2 * i + 1];
  }
  sm[0][threadIdx.x] = m;
  sm[1][threadIdx.x] = e;
  __syncthreads();
  for (int s = kHistThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      sm[0][threadIdx.x] += sm[0][threadIdx.x + s];
      sm[1][threadIdx.x] += sm[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = sm[0][0];
    out[1] = sm[1][0];
  }
}

template <class BLK, class Q>
cudaError_t launch_history_t(const BLK *blocks, int block0, int nblocks, int ng, int ndim,
                             int max_interior, Q q, double *scratch, size_t scratch_len,
                             double *out_dev, cudaStream_t s) {
  const unsigned gx = (unsigned)((max_interior + kHistThreads - 1) / kHistThreads);
  const long long nparts = (long long)gx * nblocks;
  if ((size_t)(2 * nparts) > scratch_len) return cudaErrorInvalidValue;
  k_history<<<dim3(gx, nblocks), kHistThreads, 0, s>>>(blocks, block0, ng, ndim, q, scratch);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  k_history_finish<<<1, kHistThreads, 0, s>>>(scratch, nparts, out_dev);
  return cudaGetLastError();
}

}  // namespace

size_t history_scratch_doubles(int max_interior, int nblocks) {
  return 2 * (size_t)((max_interior + kHistThreads - 1) / kHistThreads) * nblocks + 2;
}

cudaError_t launch_history(const PackDev &p, const BlockDev *blocks, int max_interior, double *scratch,
                           size_t scratch_len, double *out_dev, cudaStream_t s) {
  return launch_history_t(blocks, p.block0, p.nblocks, p.ng, p.ndim, max_interior, ConsOf{}, scratch,
                          scratch_len, out_dev, s);
}

cudaError_t launch_history_steps(const PackDev &p, const StepBlock *blocks, int max_interior,
                                 double *scratch, size_t scratch_len, double *out_dev, cudaStream_t s) {
  return launch_history_t(blocks, 0, p.nblocks, p.ng, p.ndim, max_interior, U0Of{}, scratch,
                          scratch_len, out_dev, s);
}

}  // namespace aph
