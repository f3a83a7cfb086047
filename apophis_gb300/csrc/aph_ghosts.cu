// aph_ghosts.cu -- ghost-zone fill on a uniform block grid: same-level exchange and the
// periodic / outflow / reflecting physical boundaries in one pass.  Integer work only.
#include "aph_amr.cuh"
#include "aph_capi_internal.h"

namespace aph {

// Map a global cell index along one dimension through the boundary of that dimension.
__device__ __forceinline__ int map_index(int g, int n, int lo, int hi, bool &flip) {
  if (g < 0) {
    if (lo == APH_BC_PERIODIC) return g + n;
    if (lo == APH_BC_OUTFLOW) return 0;
    flip = !flip;  // reflect: mirror about the face (apophis_boundaries.cpp:210-218)
    return -1 - g;
  }
  if (g >= n) {
    if (hi == APH_BC_PERIODIC) return g - n;
    if (hi == APH_BC_OUTFLOW) return n - 1;
    flip = !flip;
    return 2 * n - 1 - g;
  }
  return g;
}

__global__ void __launch_bounds__(256) k_fill_ghosts(PackDev p, const BlockDev *blocks, int field) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.ncell) return;
  const int idx[3] = {(int)(c % B.ni), (int)((c / B.ni) % B.nj), (int)(c / ((long long)B.ni * B.nj))};
  bool ghost = false;
  for (int d = 0; d < p.ndim; ++d) ghost |= (idx[d] < p.ng || idx[d] >= p.ng + B.nx[d]);
  if (!ghost) return;
  bool flip[3] = {false, false, false};
  int src_loc[3], src_idx[3];
  for (int d = 0; d < 3; ++d) {
    if (d < p.ndim) {
      const int g = map_index(B.loc[d] * B.nx[d] + idx[d] - p.ng, p.mesh_nx[d], p.bc[d][0],
                              p.bc[d][1], flip[d]);
      src_loc[d] = g / B.nx[d];
      src_idx[d] = g - src_loc[d] * B.nx[d] + p.ng;
    } else {
      src_loc[d] = 0;
      src_idx[d] = 0;
    }
  }
  const int sb = (src_loc[2] * p.nb[1] + src_loc[1]) * p.nb[0] + src_loc[0];
  const BlockDev &S = blocks[sb];
  const long long sc = ((long long)src_idx[2] * S.nj + src_idx[1]) * S.ni + src_idx[0];
  double *dst = field == 0 ? B.cons : B.u1;
  const double *src = field == 0 ? S.cons : S.u1;
  for (int n = 0; n < p.nvar; ++n) {
    double v = src[n * S.ncell + sc];
    if ((n == 1 && flip[0]) || (n == 2 && flip[1]) || (n == 3 && flip[2])) v = -v;
    dst[n * B.ncell + c] = v;
  }
}

__global__ void __launch_bounds__(256) k_fill_ghosts_amr(PackDev p, const BlockDev *blocks) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.ncell) return;
  amr_fill_cell(
      blocks, B, [](const BlockDev &X, int v, long long i) { return X.cons[v * X.ncell + i]; }, B.cons,
      p.nvar, p.bc, p.ng, c);
}

cudaError_t launch_fill_ghosts(const PackDev &p, const BlockDev *blocks, int max_ncell, int field,
                               cudaStream_t s) {
  dim3 grid((unsigned)((max_ncell + 255) / 256), p.nblocks);
  if (p.amr)
    k_fill_ghosts_amr<<<grid, 256, 0, s>>>(p, blocks);
  else
    k_fill_ghosts<<<grid, 256, 0, s>>>(p, blocks, field);
  return cudaGetLastError();
}

}  // namespace aph
