// aph_internal.h -- host/device shared structures and launcher prototypes.
// Included by the CUDA translation units (built once per arithmetic mode, in the
// namespaces aph_fast and aph_exact) and by the C-ABI layer.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace aph {

// Neighbours of a meshblock on a statically refined 2D mesh (face order x-, x+, y-, y+).
constexpr int FACE_SAME = 0, FACE_COARSER = 1, FACE_FINER = 2, FACE_BOUNDARY = 3;
struct AmrFaces {
  int level;
  int origin[2];      // global index of the first interior cell, in cells of its level
  int kind[4];
  int cnt[4];
  int nbr[4][4];
};

// Host-side check of a refined mesh's face table against the blocks' sizes, before any
// kernel reads through it: every index the ghost fill and the flux correction form must land
// in the named block's interior.  Returns nullptr, or a message (written to msg).
const char *amr_check(int nblocks, const AmrFaces *faces, const int (*nx)[2], int ng, char *msg,
                      size_t len);

// Device copy of one meshblock's descriptor.
struct BlockDev {
  double *cons, *prim, *gamma, *u1;
  double *flux[3];
  long long fs[3][3];   // strides of flux[d] over (n, k, j); i contiguous
  double *eos_lambda;   // optional (3 components, the shape of cons)
  int nx[3];          // interior cells
  int ni, nj, nk;     // entire extents (ghosts included)
  int loc[3];         // logical block position in the block grid
  double dx[3];
  long long ncell;    // ni * nj * nk
  AmrFaces amr;
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
  int amr;            // 1: blocks carry AmrFaces (statically refined 2D mesh)
  int block0;         // first block of this launch (a partition of the pack)
};

// ---- batched stepper -----------------------------------------------------------
// One meshblock as the stepper sees it: the state u0 (caller-owned, ghosts included),
// the stage-start copy u1, and stepper-owned scratch: prim and gamma of the stage input
// (entire domain) and the accumulated flux difference du (interior only).
struct StepBlock {
  double *u0, *u1, *prim, *gamma, *du;
  // total energy of each cell before and after the floors of the last step's end (efl: the
  // all-ones NaN where no floor changed it), so that the next ConsToPrim floors once
  double *eraw, *efl;
  double *bflux;      // refined meshes: fluxes of the 4 boundary faces, [face][t][nvar]
  int member;         // ensembles: the member (independent problem) the block belongs to
  int nx[3];
  int ni, nj, nk;
  int loc[3];
  long long ncell, nint;
  long long ipre;     // interior cells of the blocks before this one (packed interiors)
  double dx[3];
  AmrFaces amr;
};

// Device-resident control block of a stepper (dt and time live on the device so that a
// captured step replays without host round trips).
struct StepCtl {
  double dt;                    // dt of the next step
  double time;
  double tlim;                  // dt is clipped so that time never passes tlim
  double dt_fixed;              // > 0: every step uses this dt
  unsigned long long min_bits;  // dt reduction (bit pattern of the positive minimum)
  int ncycle;
  int error;                    // aph_status of a device-side failure (barrier timeout)
  int nonfinite;                // set when an update produced a NaN or an infinity
  unsigned int bar_count, bar_gen;
  unsigned int work[8];         // dynamic work counters, one per phase
};

// One member of an ensemble (independent problems batched in one pack): its gas constants
// (as PackDev's), its clock and its dt reduction.  active: time < tlim at the start of the
// step; inactive members' blocks are skipped.
struct MemberCtl {
  double gm1, igm1, gamma, c2g, one_igm1, hlle_k, hllc_k;
  double dt, time, tlim;
  unsigned long long min_bits;
  int ncycle, active;
};

// A pass item's lines: its first line and its line count share one int (count below
// 2^kItemLineBits, first line below 2^(31 - kItemLineBits)).
constexpr int kItemLineBits = 10;

// Arguments of one stage launch.
struct StageArgs {
  PackDev p;
  const StepBlock *blocks;
  StepCtl *ctl;
  // per block b: [2b] the number of the last launch whose ConsToPrim applied a floor in b,
  // [2b+1] of the last launch that deferred a floored interior write-back of b; then at
  // [2 nblocks] the number of the last stage launch (numbers only grow, so a flag is current
  // when it equals the launch's own number and nothing has to clear the flags)
  unsigned long long *block_flags;
  const int2 *cell_items;       // (block, first cell) chunks of blockDim.x entire-domain cells
  int ncell_items;
  const int2 *line_items[3];    // per direction: (block, first line << kItemLineBits | lines)
  int nline_items[3];
  const int *fix_items;         // refined meshes: blocks with a finer neighbour
  int nfix_items;
  int bflux_stride;             // doubles per face of bflux (max transverse cells * nvar)
  int cf;                       // refined meshes with coarse-fine faces: the coarse-fine phase
  MemberCtl *members;           // ensembles (NULL: one problem, clock in ctl)
  const void *tmaps;            // TMA: three tensor maps (x, y, z windows) over prim, or NULL
  int ext[3];                   // TMA: entire extents ni, nj, nk of every block
  int T[3];
  int order[3];                 // sweep order (1-based directions)
  double gam0, gam1, beta;
  double grav[3];
  int gravity;
  int copy_u1;                  // stage 1: u1 <- u0 (interior, after the floors)
  int last;                     // last stage: dt candidates of the new state
  int init;                     // dt estimate only
  int ghosts_given;             // the caller filled every ghost cell of u0: no ghost phase
  int full_domain;              // ConsToPrim of every ghost cell, also those no pass reads
  int schedule;                 // 0 strided, 1 contiguous, 2 dynamic
  unsigned long long timeout_ns;
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

#define APH_DECLARE_STAGE(NS)                                                                  \
  namespace NS {                                                                               \
  size_t stage_smem_bytes(int recon, int n, int T, int nvar);                                  \
  size_t stage_smem_bytes_tma(int recon, int n, int T, int L, int nvar);                       \
  const void *stage_kernel(int recon, int rsolver);                                            \
  cudaError_t launch_stage(const aph::StageArgs &a, int recon, int rsolver, int grid,          \
                           int threads, size_t smem, bool cooperative, int reg_cap,            \
                           cudaStream_t s);                                                    \
  cudaError_t stage_occupancy(int recon, int rsolver, int threads, size_t smem, int reg_cap,   \
                              int *blocks);                                                    \
  cudaError_t launch_barrier_probe(aph::StepCtl *ctl, unsigned long long timeout_ns,          \
                                   cudaStream_t s);                                            \
  }
APH_DECLARE_STAGE(aph_fast)
APH_DECLARE_STAGE(aph_exact)
