// aph_internal.h -- host/device shared structures and launcher prototypes.
// Included by the CUDA translation units (built once per arithmetic mode, in the
// namespaces aph_fast and aph_exact) and by the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace aph {

// Device copy of one meshblock's descriptor.
struct BlockDev {
  double *cons, *prim, *gamma, *u1;
  double *flux[3];
  int nx[3];          // interior cells
  int ni, nj, nk;     // entire extents (ghosts included)
  int loc[3];         // logical block position in the block grid
  double dx[3];
  long long ncell;    // ni * nj * nk
};

// Per-pack constants.
struct PackDev {
  int nblocks, ndim, ng, nvar;
  int max_nx[3];
  double gm1, dfloor, pfloor, cfl;
  // derived (fast mode)
  double igm1, gamma, c2g, one_igm1, hlle_k, hllc_k;
  int nb[3];          // blocks per dimension (uniform grids; 0 when unknown)
  int bc[3][2];       // physical boundary per face
  int mesh_nx[3];
};

// Work item of the fused stage kernel: one tile of one block.
struct TileItem {
  int block;
  int t0[3];          // first interior cell of the tile
  int tn[3];          // tile extent
};

}  // namespace aph

#define APH_DECLARE_LAUNCHERS(NS)                                                            \
  namespace NS {                                                                             \
  cudaError_t launch_cons_to_prim(const aph::PackDev &p, const aph::BlockDev *blocks,        \
                                  int max_ncell, int *floor_flag, cudaStream_t s);           \
  cudaError_t launch_fluxes(const aph::PackDev &p, const aph::BlockDev *blocks, int dir,     \
                            int recon, int rsolver, cudaStream_t s);                         \
  cudaError_t launch_update(const aph::PackDev &p, const aph::BlockDev *blocks, double gam0, \
                            double gam1, double beta, double beta_dt_host,                   \
                            const double *dt_dev, int max_interior, cudaStream_t s);         \
  cudaError_t launch_estimate_dt(const aph::PackDev &p, const aph::BlockDev *blocks,         \
                                 int max_interior, unsigned long long *min_bits,             \
                                 cudaStream_t s);                                            \
  cudaError_t launch_apply_gravity(const aph::PackDev &p, const aph::BlockDev *blocks,       \
                                   double g0, double g1, double g2, double beta,             \
                                   double beta_dt_host, const double *dt_dev,                \
                                   int max_interior, cudaStream_t s);                        \
  }
APH_DECLARE_LAUNCHERS(aph_fast)
APH_DECLARE_LAUNCHERS(aph_exact)
