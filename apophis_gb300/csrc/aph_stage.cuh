// aph_stage.cuh -- the batched RK stage: one persistent launch per stage over every
// meshblock of a pack, uneven block sizes included.
//
// Phases, separated by a grid-wide barrier whose waits are bounded in time:
//   1  per cell of the entire domain: a ghost cell's values from the neighbours' interiors
//      and the physical boundaries, then ConsToPrim (floors applied to u0, prim and gamma
//      to scratch); at stage 1 the floored interior is copied to u1
//   2+ one pass per direction: stage prim lines in shared memory, PPM with each face
//      value computed once and shared by its two cells (or PLM / donor cell), Riemann
//      solve, flux difference; the directions' differences accumulate in du in the
//      reference's x, y, z order, and the last pass applies the RK update,
//      the constant-g source and, at the last stage, the dt candidate of the new state
//   +  refined meshes only: the coarse cells at coarse-fine faces, corrected and updated
//      once every block's face fluxes are kept
// Face states live in shared memory only.  On GB300 the FP64 pipe, not HBM, bounds this
// kernel, so the design aims at the least FP64 work per zone: no reconstruction of
// ghost rows, one evaluation per face value, constant adiabatic indices when no floor
// fired, predicates on the integer pipe.
#pragma once
#include "aph_amr.cuh"
#include "aph_internal.h"
#include "aph_math.cuh"

#ifndef APH_NS
#error "APH_NS must name the namespace of this translation unit"
#endif

namespace APH_NS {

using namespace aph;

constexpr int kStageThreads = 256;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Grid-wide barrier.  Every CTA of the launch is resident (the grid is sized from the
// occupancy calculator, and launched cooperatively when possible); a wait that outlasts
// timeout_ns records APH_ERR_TIMEOUT and the CTA leaves, so the launch always ends.
__device__ __noinline__ bool grid_barrier(StepCtl *ctl, unsigned long long timeout_ns,
                                          unsigned int expected) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    volatile unsigned int *vgen = &ctl->bar_gen;
    volatile int *verr = &ctl->error;
    const unsigned int gen = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&ctl->bar_count, 1u) + 1u;
    if (arrived == expected) {
      atomicExch(&ctl->bar_count, 0u);
      __threadfence();
      atomicAdd(&ctl->bar_gen, 1u);
    } else {
      const unsigned long long t0 = global_ns();
      while (*vgen == gen) {
        if (*verr) { ok = 0; break; }
        __nanosleep(128);
        if (global_ns() - t0 > timeout_ns) {
          atomicCAS(&ctl->error, 0, 4 /* APH_ERR_TIMEOUT */);
          ok = 0;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ---- TMA staging of a pass item's window ----------------------------------------------------
// With a.tmaps set, the prim window of a constant-gamma item comes in as one 5D tensor copy
// (cp.async.bulk.tensor) of the whole line extent of its T lines, all five variables, from
// the pack's prim viewed as [block][var][k][j][i]; an mbarrier with its transaction count
// signals completion and every thread waits on it with a time bound.
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned phase) {
  unsigned done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(bar), "r"(phase)
      : "memory");
  return done != 0;
}

// Wait for the copy of this phase; after timeout_ns the wait records APH_ERR_TIMEOUT and
// keeps waiting for the copy in flight for up to another timeout_ns before giving up.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned phase, StepCtl *ctl,
                                                  unsigned long long timeout_ns) {
  if (mbar_try_wait(bar, phase)) return true;
  const unsigned long long t0 = global_ns();
  bool late = false;
  while (!mbar_try_wait(bar, phase)) {
    const unsigned long long dt = global_ns() - t0;
    if (!late && dt > timeout_ns) {
      atomicCAS(&ctl->error, 0, 4 /* APH_ERR_TIMEOUT */);
      late = true;
    }
    if (dt > 2 * timeout_ns) return false;
  }
  return !late;
}

__device__ __forceinline__ void tma_load_5d(unsigned dst, const void *tmap, unsigned bar, int c0,
                                            int c1, int c2, int c3, int c4) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5, %6}], [%7];" ::"r"(dst),
      "l"((unsigned long long)tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}

// Work distribution of a phase with n items.
struct Sched {
  int mode;
  __device__ __forceinline__ int first(unsigned int *ctr, int n) const {
    if (mode == 1) {  // this CTA's contiguous range, possibly empty
      const int s = (int)(((long long)blockIdx.x * n) / gridDim.x);
      const int e = (int)(((long long)(blockIdx.x + 1) * n) / gridDim.x);
      return s < e ? s : n;
    }
    if (mode == 2) return next(ctr, n, -1);
    return blockIdx.x;
  }
  __device__ __forceinline__ int next(unsigned int *ctr, int n, int cur) const {
    if (mode == 1) {
      const int end = (int)(((long long)(blockIdx.x + 1) * n) / gridDim.x);
      return cur + 1 < end ? cur + 1 : n;
    }
    if (mode == 2) {
      __shared__ int s_next;
      __syncthreads();
      if (threadIdx.x == 0) s_next = (int)atomicAdd(ctr, 1u);
      __syncthreads();
      return s_next < n ? s_next : n;
    }
    return cur + gridDim.x;
  }
};

// ---- ghost values on a uniform block grid ---------------------------------------------
__device__ __forceinline__ int map_index(int g, int n, int lo, int hi, bool &flip) {
  if (g < 0) {
    if (lo == 0) return g + n;      // periodic
    if (lo == 1) return 0;          // outflow
    flip = !flip;                   // reflecting
    return -1 - g;
  }
  if (g >= n) {
    if (hi == 0) return g - n;
    if (hi == 1) return n - 1;
    flip = !flip;
    return 2 * n - 1 - g;
  }
  return g;
}

// ---- floors at step boundaries ----------------------------------------------------------
// The reference applies the floors of ConsToPrim once to every new state, at the end of the
// stage that made it (FillDerived), and its pressure floor is not idempotent: it rebuilds E
// from the pressure before the floor (hydro.cpp:517-521).  Here a stage floors its input at
// its start, and the last stage of a step also stores its output floored (what a caller then
// reads is the reference's state) while keeping, per floored cell, the energy before the
// floor (eraw) and after it (efl).  The first stage of the next step reads the energy before
// the floor wherever the stored energy is still the floored one, so the floor is applied once.
constexpr unsigned long long kNoFloorTag = ~0ULL;  // a NaN that arithmetic never produces
// Marks (in a cell's du slot of the first momentum) a floored density and energy waiting in
// its du slots of those components; another NaN that arithmetic never produces.
constexpr unsigned long long kDeferTag = ~1ULL;

__device__ __forceinline__ double energy_in(const StepBlock &X, long long c, bool step_start) {
  const double e = X.u0[IEN * X.ncell + c];
  if (!step_start) return e;
  return __double_as_longlong(e) == __double_as_longlong(X.efl[c]) ? X.eraw[c] : e;
}

__device__ __forceinline__ void store_floored_energy(const StepBlock &X, long long c, double e_raw,
                                                     double e_floored) {
  const bool changed = __double_as_longlong(e_raw) != __double_as_longlong(e_floored);
  X.efl[c] = changed ? e_floored : __longlong_as_double((long long)kNoFloorTag);
  if (changed) X.eraw[c] = e_raw;
}

__device__ void ghost_cell(const StageArgs &a, const StepBlock &B, long long c) {
  const PackDev &p = a.p;
  const int idx[3] = {(int)(c % B.ni), (int)((c / B.ni) % B.nj), (int)(c / ((long long)B.ni * B.nj))};
  bool ghost = false;
  for (int d = 0; d < p.ndim; ++d) ghost |= (idx[d] < p.ng || idx[d] >= p.ng + B.nx[d]);
  if (!ghost) return;
  bool flip[3] = {false, false, false};
  int sl[3], si[3];
  for (int d = 0; d < 3; ++d) {
    if (d < p.ndim) {
      const int g = map_index(B.loc[d] * B.nx[d] + idx[d] - p.ng, p.mesh_nx[d], p.bc[d][0],
                              p.bc[d][1], flip[d]);
      sl[d] = g / B.nx[d];
      si[d] = g - sl[d] * B.nx[d] + p.ng;
    } else {
      sl[d] = 0;
      si[d] = 0;
    }
  }
  const StepBlock &S = a.blocks[(sl[2] * p.nb[1] + sl[1]) * p.nb[0] + sl[0]];
  const long long sc = ((long long)si[2] * S.nj + si[1]) * S.ni + si[0];
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) {
    double v = n == IEN ? energy_in(S, sc, a.copy_u1) : S.u0[n * S.ncell + sc];
    if ((n == IM1 && flip[0]) || (n == IM2 && flip[1]) || (n == IM3 && flip[2])) v = -v;
    B.u0[n * B.ncell + c] = v;
  }
  for (int n = NHYDRO; n < p.nvar; ++n) B.u0[n * B.ncell + c] = S.u0[n * S.ncell + sc];
}

__device__ __forceinline__ bool is_interior(const PackDev &p, const StepBlock &B, long long c,
                                            int &i, int &j, int &k) {
  i = (int)(c % B.ni);
  j = (int)((c / B.ni) % B.nj);
  k = (int)(c / ((long long)B.ni * B.nj));
  bool in = i >= p.ng && i < p.ng + B.nx[0];
  if (p.ndim >= 2) in = in && j >= p.ng && j < p.ng + B.nx[1];
  if (p.ndim >= 3) in = in && k >= p.ng && k < p.ng + B.nx[2];
  return in;
}

// Whether a pass reads ghost cell (i, j, k) of B: outside the interior along exactly one
// direction, by at most G cells.
__device__ __forceinline__ bool pass_reads(const PackDev &p, const StepBlock &B, int i, int j, int k,
                                           int G) {
  const int e[3] = {i, j, k};
  int out = 0, depth = 0;
  for (int d = 0; d < p.ndim; ++d) {
    const int x = e[d] - p.ng;
    const int o = x < 0 ? -x : (x >= B.nx[d] ? x - B.nx[d] + 1 : 0);
    if (o > 0) {
      ++out;
      depth = o;
    }
  }
  return out == 1 && depth <= G;
}

// Whether the face ghost cell (i, j, k) of B holds a copy of an interior cell: a same-level
// neighbour's (on a uniform block grid always, periodic wraps included), or B's own at an
// outflow or reflecting boundary -- rather than values formed by restriction or prolongation
// at a coarse-fine face.  ConsToPrim of a copy equals the source cell's primitives (with the
// normal velocity negated at a reflecting boundary: IEEE products are sign-symmetric), so the
// passes read those at the source (ghost_copy_src) and phase 1 leaves such ghosts alone.
__device__ __forceinline__ bool ghost_is_copy(const PackDev &p, const StepBlock &B, int i, int j, int k) {
  if (!p.amr) return true;
  const int e[3] = {i, j, k};
  int face = 0;
  for (int d = 0; d < p.ndim; ++d) {
    const int x = e[d] - p.ng;
    if (x < 0) face = 2 * d;
    else if (x >= B.nx[d]) face = 2 * d + 1;
  }
  return B.amr.kind[face] == FACE_SAME || B.amr.kind[face] == FACE_BOUNDARY;
}

// The source of the copied ghost cell at position c (c < 0 or c >= n) along DIR of line l of
// B (base, stride: the line's first interior cell and its step): the block S, its cell sc and
// the velocity component to negate (flipv, -1: none).  Leaves them untouched and returns
// false for a ghost formed at a coarse-fine face.
template <int DIR>
__device__ __forceinline__ bool ghost_copy_src(const StageArgs &a, const StepBlock &B, int l, int c,
                                               long long base, long long stride, const StepBlock *&S,
                                               long long &sc, int &flipv) {
  const PackDev &p = a.p;
  constexpr int d = DIR - 1;
  const int n = B.nx[d];
  if (!p.amr) {  // the uniform block grid's map (ghost_cell)
    bool flip = false;
    const int g = map_index(B.loc[d] * n + c, p.mesh_nx[d], p.bc[d][0], p.bc[d][1], flip);
    const int sl = g / n;
    int loc[3] = {B.loc[0], B.loc[1], B.loc[2]};
    loc[d] = sl;
    S = &a.blocks[(loc[2] * p.nb[1] + loc[1]) * p.nb[0] + loc[0]];
    sc = base + (long long)(g - sl * n) * stride;
    flipv = flip ? IV1 + d : -1;
    return true;
  }
  if (d > 1) return false;  // face tables are 2D
  const int side = c < 0 ? 0 : 1, depth = c < 0 ? -c - 1 : c - n;
  const int face = 2 * d + side, td = 1 - d;
  const int kind = B.amr.kind[face];
  if (kind == FACE_SAME) {  // as amr_ghost5; the line index is the transverse coordinate
    const StepBlock &N = a.blocks[B.amr.nbr[face][0]];
    S = &N;
    sc = amr_cell(N, p.ng, d, side == 0 ? N.nx[d] - 1 - depth : depth, B.amr.origin[td] + l - N.amr.origin[td]);
    flipv = -1;
    return true;
  }
  if (kind == FACE_BOUNDARY) {
    S = &B;
    if (p.bc[d][side] == 1) {  // outflow
      sc = amr_cell(B, p.ng, d, side == 0 ? 0 : n - 1, l);
      flipv = -1;
    } else {                   // reflecting
      sc = amr_cell(B, p.ng, d, side == 0 ? depth : n - 1 - depth, l);
      flipv = IV1 + d;
    }
    return true;
  }
  return false;
}

// Copied ghosts come from their sources unless the launch stages windows by TMA (which copies
// each block's own ghost cells), the caller filled the ghosts (a halo exchange) or the
// primitives of the entire domain are kept (the adjoint).
__device__ __forceinline__ bool ghosts_from_sources(const StageArgs &a) {
  return !a.full_domain && !a.ghosts_given && !a.tmaps;
}

__device__ __forceinline__ unsigned long long block_min(unsigned long long v) {
  __shared__ unsigned long long red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : ~0ULL;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
      v = x < v ? x : v;
    }
  }
  return v;
}

__device__ __forceinline__ unsigned long long dt_bits(double m) {
  return is_neg(m) ? ~0ULL : (unsigned long long)__double_as_longlong(m);
}

// ---- ensembles: per-member gas constants, clock and dt minimum ---------------------------
__device__ __forceinline__ GasConsts gas_of(const StageArgs &a, const StepBlock &B) {
  if (a.members) {
    const MemberCtl &m = a.members[B.member];
    return GasConsts{m.gm1, m.igm1, m.gamma, m.c2g, m.one_igm1, m.hlle_k, m.hllc_k};
  }
  return GasConsts{a.p.gm1, a.p.igm1, a.p.gamma, a.p.c2g, a.p.one_igm1, a.p.hlle_k, a.p.hllc_k};
}

__device__ __forceinline__ bool active_of(const StageArgs &a, const StepBlock &B) {
  return !a.members || a.members[B.member].active;
}

__device__ __forceinline__ double dt_of(const StageArgs &a, const StepBlock &B) {
  return a.members ? a.members[B.member].dt : a.ctl->dt;
}

// Fold each thread's dt candidate into its member's minimum.  Called by whole warps whose
// lanes all work on one block.
__device__ __forceinline__ void member_min(const StageArgs &a, int member, unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
  if ((threadIdx.x & 31) == 0 && v != ~0ULL) atomicMin(&a.members[member].min_bits, v);
}

// ---- refined meshes: the cells the coarse-fine correction changes ----------------------
// Bit f set: face f (x-, x+, y-, y+) of B has a finer neighbour.
template <class BLK>
__device__ __forceinline__ int amr_finer_mask(const BLK &B) {
  int m = 0;
#pragma unroll
  for (int f = 0; f < 4; ++f) m |= (B.amr.kind[f] == FACE_FINER ? 1 : 0) << f;
  return m;
}

// Whether interior cell ic (x fastest) of a 2D block lies on a face of the mask.
template <class BLK>
__device__ __forceinline__ bool amr_defers(int fmask, const BLK &B, long long ic) {
  const int j = (int)(ic / B.nx[0]), i = (int)(ic - (long long)j * B.nx[0]);
  return ((fmask & 1) && i == 0) || ((fmask & 2) && i == B.nx[0] - 1) ||
         ((fmask & 4) && j == 0) || ((fmask & 8) && j == B.nx[1] - 1);
}

// ---- line geometry of a pass ----------------------------------------------------------
// Line l of block B along DIR: the cell of interior position c on it is base + c*stride;
// its interior index (for du) is ibase + c*istride.
template <int DIR>
__device__ __forceinline__ void line_of(const StepBlock &B, int ndim, int ng, int l,
                                        long long &base, long long &stride, long long &ibase,
                                        long long &istride) {
  const int sj = ndim >= 2 ? ng : 0, sk = ndim >= 3 ? ng : 0;
  const int n0 = B.nx[0], n1 = B.nx[1];
  if (DIR == 1) {
    const int j = l % n1, k = l / n1;
    base = ((long long)(k + sk) * B.nj + (j + sj)) * B.ni + ng;
    stride = 1;
    ibase = (long long)l * n0;
    istride = 1;
  } else if (DIR == 2) {
    const int i = l % n0, k = l / n0;
    base = ((long long)(k + sk) * B.nj + sj) * B.ni + (i + ng);
    stride = B.ni;
    ibase = (long long)k * n1 * n0 + i;
    istride = n0;
  } else {
    const int i = l % n0, j = l / n0;
    base = ((long long)sk * B.nj + (j + sj)) * B.ni + (i + ng);
    stride = (long long)B.ni * B.nj;
    ibase = (long long)j * n0 + i;
    istride = (long long)n0 * n1;
  }
}

template <int RECON>
struct Halo {
  static constexpr int G = RECON == RECON_PPM ? 3 : RECON == RECON_PLM ? 2 : 1;
};

// Shared-memory doubles needed by one pass item of T lines of n cells with V
// reconstructed variables.
__host__ __device__ constexpr size_t pass_smem_doubles(int recon, int n, int T, int V) {
  return recon == RECON_PPM
             ? (size_t)V * T * ((n + 6) + 2 * (n + 4) + (n + 3) + (n + 2))
             : (size_t)V * T * ((n + 2 * (recon == RECON_PLM ? 2 : 1)) + 2 * (n + 2));
}

// Reconstructed slabs beyond the nvar primitives that shared memory is sized for: the exact
// build always reconstructs the two adiabatic-index fields; the fast build sizes for
// constant-gamma items and splits an item of a block where a floor fired (which needs the
// two extra slabs) into chunks of fewer lines (split_lines).
#if APH_EXACT
constexpr int kGammaSlabs = 2;
#else
constexpr int kGammaSlabs = 0;
#endif

// Lines of a chunk that fits the gamma slabs into the shared memory of T lines.
__host__ __device__ constexpr int split_lines(int T, int nvar) {
  return (nvar + kGammaSlabs) * T / (nvar + 2) > 1 ? (nvar + kGammaSlabs) * T / (nvar + 2) : 1;
}

// Doubles between the window region and the TMA staging area: the window (nvar +
// kGammaSlabs variables) is padded to a multiple of 16 doubles so that the staging area
// starts 128-byte aligned.
__host__ __device__ constexpr size_t tma_stage_offset(int recon, int n, int T, int nvar) {
  return ((size_t)(nvar + kGammaSlabs) * T * (n + 2 * (recon == RECON_PPM ? 3 : recon == RECON_PLM ? 2 : 1)) +
          15) /
         16 * 16;
}

// PPM of a pass item's window: W holds V x T lines of cells -G..n+G-1 (row width n + 2G);
// per cell the second differences D2 and centred differences DD (cells -2..n+1), per face
// the limited value DPH once (faces -1..n+1), then per cell the parabola limiter writes the
// left state of face c+1 to SL[c+1] and the right state of face c to SR[c+1] (cells -1..n).
template <bool TAME>
__device__ __forceinline__ void ppm_window(const double *W, double *D2, double *DD, double *DPH,
                                           double *SL, double *SR, int V, int nl, int T, int n,
                                           int G) {
  const int NW = n + 2 * G;
  const int tid = threadIdx.x, nth = blockDim.x;
  // row v * T + t of the slabs and position i in it, for element it of rows of width w (one
  // division where the item fills its T lines, as plain-load items do)
  const bool full = nl == T;
  auto decode = [&](int it, int w, int &row, int &i) {
    if (full) {
      row = it / w;
      i = it - row * w;
    } else {
      const int v = it / (nl * w);
      const int r = it - v * nl * w;
      const int t = r / w;
      i = r - t * w;
      row = v * T + t;
    }
  };
  auto w_at = [&](int row, int c) -> double { return W[(size_t)row * NW + c + G]; };
  const int w4 = n + 4, w3 = n + 3;
  for (int it = tid; it < V * nl * w4; it += nth) {  // cells -2..n+1
    int row, i;
    decode(it, w4, row, i);
    const int c = i - 2;
    const double qm = w_at(row, c - 1), q0 = w_at(row, c), qp = w_at(row, c + 1);
    D2[(size_t)row * w4 + c + 2] = ppm_d2<TAME>(qm, q0, qp);
    DD[(size_t)row * w4 + c + 2] = ppm_dd<TAME>(qm, q0, qp);
  }
  __syncthreads();
  for (int it = tid; it < V * nl * w3; it += nth) {  // faces -1..n+1
    int row, i;
    decode(it, w3, row, i);
    const int f = i - 1;
    const size_t o = (size_t)row * w4;
    DPH[(size_t)row * w3 + f + 1] =
        ppm_face<TAME>(w_at(row, f - 1), w_at(row, f), DD[o + f + 1], DD[o + f + 2],
                       D2[o + f + 1], D2[o + f + 2]);
  }
  __syncthreads();
  const int w2 = n + 2;
  for (int it = tid; it < V * nl * w2; it += nth) {  // cells -1..n
    int row, i;
    decode(it, w2, row, i);
    const int c = i - 1;
    const size_t o4 = (size_t)row * w4, o3 = (size_t)row * w3;
    double ql, qr;
    ppm_cell<TAME>(w_at(row, c - 2), w_at(row, c - 1), w_at(row, c), w_at(row, c + 1),
                   w_at(row, c + 2), D2[o4 + c + 1], D2[o4 + c + 2], D2[o4 + c + 3],
                   DPH[o3 + c + 1], DPH[o3 + c + 2], ql, qr);
    SL[(size_t)row * w2 + c + 1] = ql;
    SR[(size_t)row * w2 + c + 1] = qr;
  }
}

// One pass item: lines l0..l0+nl-1 of block B along DIR.  b: the block's index in the pack;
// tma_phase: the parity of the CTA's next mbarrier phase (TMA items flip it).  Returns false
// (the same in every thread of the CTA) when a TMA wait ran out: the window is then not used,
// the item computes and writes nothing, and the caller leaves the launch, whose status is
// already APH_ERR_TIMEOUT and whose results are invalid.
template <int DIR, int RECON, int RS>
__device__ bool pass_item(const StageArgs &a, const StepBlock &B, int b, int l0, int nl, int T,
                          bool constg, bool deferred, bool first_pass, bool last_pass, double *sm,
                          unsigned long long &dtmin, unsigned mbar, unsigned &tma_phase) {
  constexpr int G = Halo<RECON>::G;
  const int n = B.nx[DIR - 1];
  const int nv = a.p.nvar;  // 5 hydro variables, then the passive scalars
  const int V = constg ? nv : nv + 2;  // with gamma_c, gamma_e where the gas is not ideal
  const GasConsts gc = gas_of(a, B);
  const int NW = n + 2 * G;
  const long long nc = B.ncell;
  const int tid = threadIdx.x, nth = blockDim.x;
  // shared-memory regions (V x T x width each)
  double *W = sm;                                  // prim window, cells -G..n+G-1
  double *D2 = W + (size_t)V * T * NW;             // PPM: d2, cells -2..n+1
  double *DD = D2 + (RECON == RECON_PPM ? (size_t)V * T * (n + 4) : 0);  // PPM: dd
  double *DPH = DD + (RECON == RECON_PPM ? (size_t)V * T * (n + 4) : 0);  // PPM: face values
  double *SR = DPH + (RECON == RECON_PPM ? (size_t)V * T * (n + 3) : 0);  // right states
  double *SL = (RECON == RECON_PPM) ? DD : SR + (size_t)V * T * (n + 2);  // left states
  double *F = W;                                   // fluxes, after the window is dead
  auto w_at = [&](int v, int t, int c) -> double & { return W[((size_t)v * T + t) * NW + c + G]; };

  // A: load the window of prim (and gamma) along each line
  bool tame_ok = true;  // exact mode: whether every window value is tame (aph_math.cuh)
  (void)tame_ok;
  if (a.tmaps && constg) {
    // one tensor copy of the T lines' whole extent into the staging area, then the window
    // cells -G..n+G-1 into W (the staging layout is [v][t][i] along x, [v][w][t] along y, z)
    // 128-byte aligned staging area after the window region (the size reserves the slack)
    double *stg = (double *)(((unsigned long long)(sm + tma_stage_offset(RECON, n, T, nv)) + 127ULL) & ~127ULL);
    const int L = a.ext[DIR - 1];
    const int ng = a.p.ng;
    // order every thread's earlier generic accesses of this shared memory before the copy
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // the item's lines lie in one plane of the block, or in two consecutive planes: one box
    // of T lines at each (lines of a box beyond the item are loaded and not used)
    const int per_plane = DIR == 1 ? B.nx[1] : B.nx[0];
    const int lp = l0 % per_plane, plane = l0 / per_plane;
    const int T1 = min(nl, per_plane - lp);
    const size_t box = (size_t)nv * T * L;
    if (tid == 0) {
      const unsigned bytes = (unsigned)((nl > T1 ? 2 : 1) * box * sizeof(double));
      mbar_expect_tx(mbar, bytes);
      const char *maps = (const char *)a.tmaps;
      const int sj = a.p.ndim >= 2 ? ng : 0, sk = a.p.ndim >= 3 ? ng : 0;
      for (int part = 0; part < (nl > T1 ? 2 : 1); ++part) {
        const int pos = part == 0 ? lp : 0, pl = plane + part;
        const unsigned dst = smem_addr(stg + part * box);
        if (DIR == 1) tma_load_5d(dst, maps, mbar, 0, pos + sj, pl + sk, 0, b);
        else if (DIR == 2) tma_load_5d(dst, maps + 128, mbar, pos + ng, 0, pl + sk, 0, b);
        else tma_load_5d(dst, maps + 256, mbar, pos + ng, pl + sj, 0, 0, b);
      }
    }
    const bool arrived = mbar_wait_bounded(mbar, tma_phase, a.ctl, a.timeout_ns);
    tma_phase ^= 1u;
    if (__syncthreads_or(!arrived)) return false;
    for (int it = tid; it < nv * nl * NW; it += nth) {
      const int v = it / (nl * NW);
      const int r = it - v * nl * NW;
      const int t = r / NW, w = r - t * NW;
      const int cell = w - G + ng;  // position along the line's whole extent
      const double *src = t < T1 ? stg : stg + box;
      const int tt = t < T1 ? t : t - T1;
      W[((size_t)v * T + t) * NW + w] = DIR == 1 ? src[((size_t)v * T + tt) * L + cell]
                                                 : src[((size_t)v * L + cell) * T + tt];
    }
  } else {
    const int per = nl * NW;
    const bool src_ghosts = ghosts_from_sources(a);
    // per window cell: its line geometry and source once, then its V values
    for (int it = tid; it < per; it += nth) {
      int t, w;
      if (DIR == 1) { t = it / NW; w = it - t * NW; } else { w = it / nl; t = it - w * nl; }
      long long base, stride, ib, is;
      line_of<DIR>(B, a.p.ndim, a.p.ng, l0 + t, base, stride, ib, is);
      const int c = w - G;
      long long cell = base + (long long)c * stride;
      const StepBlock *S = &B;  // the block holding the cell's primitives
      int flipv = -1;
      if (src_ghosts && (c < 0 || c >= n)) ghost_copy_src<DIR>(a, B, l0 + t, c, base, stride, S, cell, flipv);
      const long long snc = S->ncell;
      for (int v = 0; v < nv; ++v) {
        const double x = flip_if(S->prim[v * snc + cell], v == flipv);
        W[((size_t)v * T + t) * NW + w] = x;
#if APH_EXACT
        tame_ok = tame_ok && tame(x);
#endif
      }
      if (V > nv) {
        double g_c, g_e;
#if APH_EXACT
        g_c = S->gamma[cell];
        g_e = S->gamma[snc + cell];
        tame_ok = tame_ok && tame(g_c) && tame(g_e);
#else
        // the fast ConsToPrim leaves the constants where no floor fired; the reference's
        // values (which the limiters see) are recomputed from the cell's state there (a
        // floored cell's state may still wait in du for the first pass to store it)
        if (__double_as_longlong(S->prim[IPR * snc + cell]) == __double_as_longlong(a.p.pfloor) ||
            __double_as_longlong(S->prim[IDN * snc + cell]) == __double_as_longlong(a.p.dfloor)) {
          g_c = S->gamma[cell];  // floored: the reference's values already
          g_e = S->gamma[snc + cell];
        } else {
          double uc[NHYDRO];
#pragma unroll
          for (int k = 0; k < NHYDRO; ++k) uc[k] = S->u0[k * snc + cell];
          gamma_ref(uc, gc.gm1, g_c, g_e);
        }
#endif
        W[((size_t)nv * T + t) * NW + w] = g_c;
        W[((size_t)(nv + 1) * T + t) * NW + w] = g_e;
      }
    }
  }
#if APH_EXACT
  // every window value tame: the reconstruction takes the integer-pipe forms (same bits)
  const bool tame_item = __syncthreads_and(tame_ok) != 0;
#else
  __syncthreads();
#endif
  // B-D: reconstruction; left state of face c+1 -> SL[c+1], right state of face c -> SR[c+1]
  if (RECON == RECON_PPM) {
#if APH_EXACT
    if (tame_item)
      ppm_window<true>(W, D2, DD, DPH, SL, SR, V, nl, T, n, G);
    else
#endif
      ppm_window<false>(W, D2, DD, DPH, SL, SR, V, nl, T, n, G);
  } else {
    const int w2 = n + 2;
    for (int it = tid; it < V * nl * w2; it += nth) {
      const int v = it / (nl * w2);
      const int r = it - v * nl * w2;
      const int t = r / w2, c = r - t * w2 - 1;
      double ql, qr;
      if (RECON == RECON_PLM) {
        plm(w_at(v, t, c - 1), w_at(v, t, c), w_at(v, t, c + 1), ql, qr);
      } else {
        ql = qr = w_at(v, t, c);
      }
      SL[((size_t)v * T + t) * w2 + c + 1] = ql;
      SR[((size_t)v * T + t) * w2 + c + 1] = qr;
    }
  }
  __syncthreads();
  // E: Riemann solve on faces 0..n
  {
    constexpr int ivx = DIR;
    constexpr int ivy = IV1 + ((ivx - IV1) + 1) % 3;
    constexpr int ivz = IV1 + ((ivx - IV1) + 2) % 3;
    const int w2 = n + 2, w1 = n + 1;
    const size_t vs = (size_t)T * w2;
    for (int it = tid; it < nl * w1; it += nth) {
      const int t = it / w1, f = it - t * w1;
      const size_t oL = (size_t)t * w2 + f, oR = oL + 1;
      double wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
      wl[IDN] = SL[IDN * vs + oL]; wl[IV1] = SL[ivx * vs + oL]; wl[IV2] = SL[ivy * vs + oL];
      wl[IV3] = SL[ivz * vs + oL]; wl[IPR] = SL[IPR * vs + oL];
      wr[IDN] = SR[IDN * vs + oR]; wr[IV1] = SR[ivx * vs + oR]; wr[IV2] = SR[ivy * vs + oR];
      wr[IV3] = SR[ivz * vs + oR]; wr[IPR] = SR[IPR * vs + oR];
#if APH_EXACT
      if (tame_item)
        riemann<RS, false, true>(wl, wr, SL[nv * vs + oL], SL[(nv + 1) * vs + oL], SR[nv * vs + oR],
                                 SR[(nv + 1) * vs + oR], gc, flx);
      else
        riemann<RS, false, false>(wl, wr, SL[nv * vs + oL], SL[(nv + 1) * vs + oL], SR[nv * vs + oR],
                                  SR[(nv + 1) * vs + oR], gc, flx);
#else
      if (constg) {
        riemann<RS, true>(wl, wr, 0.0, 0.0, 0.0, 0.0, gc, flx);
      } else {
        riemann<RS, false>(wl, wr, SL[nv * vs + oL], SL[(nv + 1) * vs + oL], SR[nv * vs + oR],
                           SR[(nv + 1) * vs + oR], gc, flx);
      }
#endif
      // store in cons order
      const size_t fs = (size_t)T * w1;
      const size_t of = (size_t)t * w1 + f;
      F[IDN * fs + of] = flx[IDN];
      F[ivx * fs + of] = flx[IV1];
      F[ivy * fs + of] = flx[IV2];
      F[ivz * fs + of] = flx[IV3];
      F[IEN * fs + of] = flx[IEN];
      // passive scalars: upwind by the mass flux (hydro.cpp:607-615)
      for (int v = NHYDRO; v < nv; ++v)
        F[v * fs + of] = flx[IDN] * (!is_neg(flx[IDN]) ? SL[v * vs + oL] : SR[v * vs + oR]);
    }
  }
  __syncthreads();
  if (a.cf) {  // keep the boundary-face fluxes of every line for the coarse-fine correction
    const int w1 = n + 1;
    const size_t fs = (size_t)T * w1;
    for (int it = tid; it < nl * 2 * nv; it += nth) {
      const int t = it / (2 * nv), r = it % (2 * nv), side = r / nv, v = r % nv;
      B.bflux[(size_t)(2 * (DIR - 1) + side) * a.bflux_stride + (size_t)(l0 + t) * nv + v] =
          F[v * fs + (size_t)t * w1 + (side == 0 ? 0 : n)];
    }
  }
  if (deferred) {  // first pass: store the floored interior values ConsToPrim left in du
    for (int it = tid; it < nl * n; it += nth) {
      const int t = it / n, c = it - t * n;
      long long base, stride, ib, is;
      line_of<DIR>(B, a.p.ndim, a.p.ng, l0 + t, base, stride, ib, is);
      const long long icell = ib + c * is;
      if (__double_as_longlong(B.du[IM1 * B.nint + icell]) == (long long)kDeferTag) {
        B.u0[IDN * nc + base + c * stride] = B.du[IDN * B.nint + icell];
        B.u0[IEN * nc + base + c * stride] = B.du[IEN * B.nint + icell];
      }
    }
    __syncthreads();
  }
  // F: flux difference of each interior cell; du accumulates x, y, z in order
  {
    const int w1 = n + 1;
    const size_t fs = (size_t)T * w1;
    const double area = DIR == 1 ? B.dx[1] * B.dx[2] : DIR == 2 ? B.dx[0] * B.dx[2] : B.dx[0] * B.dx[1];
    if (!last_pass) {
      for (int it = tid; it < nl * n; it += nth) {  // per cell: its geometry once, then its nv values
        const int t = it / n, c = it - t * n;
        long long base, stride, ib, is;
        line_of<DIR>(B, a.p.ndim, a.p.ng, l0 + t, base, stride, ib, is);
        double *du = B.du + ib + c * is;
        for (int v = 0; v < nv; ++v) {
          const size_t of = v * fs + (size_t)t * w1 + c;
          const double d = (area * F[of + 1] - area * F[of]);
          du[v * B.nint] = first_pass ? d : du[v * B.nint] + d;
        }
      }
    } else {
      const double vol = B.dx[0] * B.dx[1] * B.dx[2];
      const double ivol = 1.0 / vol;
#if APH_EXACT
      const bool vol_p2 = pow2_normal(vol);  // power-of-two volume: exact multiplication
#endif
      const double beta_dt = a.beta * dt_of(a, B);
      const int fmask = a.cf ? amr_finer_mask(B) : 0;
      unsigned long long mymin = ~0ULL;
      for (int it = tid; it < nl * n; it += nth) {
        const int t = it / n, c = it - t * n;
        long long base, stride, ib, is;
        line_of<DIR>(B, a.p.ndim, a.p.ng, l0 + t, base, stride, ib, is);
        const long long cell = base + c * stride;
        const long long icell = ib + c * is;
        if (fmask && amr_defers(fmask, B, icell)) {
          // a coarse cell at a face with a finer neighbour: its flux difference waits for
          // the correction, and amr_fix updates it
          for (int v = 0; v < nv; ++v) {
            const size_t of = v * fs + (size_t)t * w1 + c;
            const double d = (area * F[of + 1] - area * F[of]);
            double *du = B.du + v * B.nint + icell;
            *du = first_pass ? d : *du + d;
          }
          continue;
        }
        double u[NHYDRO];
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) {
          const size_t of = v * fs + (size_t)t * w1 + c;
          double du = (area * F[of + 1] - area * F[of]);
          if (!first_pass) du = B.du[v * B.nint + icell] + du;
#if APH_EXACT
          const double div = div_vol(-du, vol, ivol, vol_p2);
#else
          const double div = -du * ivol;
#endif
          u[v] = a.gam0 * B.u0[v * nc + cell] + a.gam1 * B.u1[v * nc + cell] + beta_dt * div;
        }
        bool bad = false;
        for (int v = NHYDRO; v < nv; ++v) {  // passive scalars
          const size_t of = v * fs + (size_t)t * w1 + c;
          double du = (area * F[of + 1] - area * F[of]);
          if (!first_pass) du = B.du[v * B.nint + icell] + du;
#if APH_EXACT
          const double div = div_vol(-du, vol, ivol, vol_p2);
#else
          const double div = -du * ivol;
#endif
          const double q = a.gam0 * B.u0[v * nc + cell] + a.gam1 * B.u1[v * nc + cell] + beta_dt * div;
          B.u0[v * nc + cell] = q;
          bad |= ((__double_as_longlong(q) >> 52) & 0x7ff) == 0x7ff;
        }
        if (a.gravity) {  // ApplyGravity with the stage input's prim (gravity.cpp:386-407)
          const double rho = B.prim[IDN * nc + cell];
          u[IM1] += a.grav[0] * rho * beta_dt;
          double de = a.grav[0] * B.prim[IV1 * nc + cell];
          if (a.p.ndim >= 2) {
            u[IM2] += a.grav[1] * rho * beta_dt;
            de += a.grav[1] * B.prim[IV2 * nc + cell];
          }
          if (a.p.ndim >= 3) {
            u[IM3] += a.grav[2] * rho * beta_dt;
            de += a.grav[2] * B.prim[IV3 * nc + cell];
          }
          u[IEN] += de * rho * beta_dt;
        }
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v)
          bad |= ((__double_as_longlong(u[v]) >> 52) & 0x7ff) == 0x7ff;  // NaN or inf
        if (bad) a.ctl->nonfinite = 1;
        if (a.last) {  // EstimateTimestep on the floored new state, which is stored floored
          double w[NHYDRO], gcc, gce;
          const double e_raw = u[IEN];
          const bool fl = cons_to_prim_cell(u, w, gcc, gce, gc.gm1, a.p.dfloor, a.p.pfloor);
          const unsigned long long b = dt_bits(dt_cell(w, u[IEN], B.dx, a.p.ndim, gc, fl));
          mymin = b < mymin ? b : mymin;
          store_floored_energy(B, cell, e_raw, u[IEN]);
        }
#pragma unroll
        for (int v = 0; v < NHYDRO; ++v) B.u0[v * nc + cell] = u[v];
      }
      if (a.last) {
        if (a.members) member_min(a, B.member, mymin);
        else dtmin = mymin < dtmin ? mymin : dtmin;
      }
    }
  }
  __syncthreads();
  return true;
}

// Refined meshes, after the last pass: the boundary cells of the coarse blocks at faces with
// a finer neighbour (the cells the last pass left).  Each such cell's accumulated flux
// difference takes, for every face of that kind it lies on (in the order x-, x+, y-, y+),
// its own face flux replaced by the mean of the two fine face fluxes; then the RK update,
// gravity and the dt candidate follow as in the last pass.
__device__ __forceinline__ double amr_fixed_du(const StageArgs &a, const StepBlock &B, int fmask, int i,
                                               int j, long long ic, int v) {
  const int nv = a.p.nvar;
  double x = B.du[v * B.nint + ic];
  for (int face = 0; face < 4; ++face) {
    if (!((fmask >> face) & 1)) continue;
    const int d = face / 2, s = face % 2, td = 1 - d;
    if ((d == 0 ? i : j) != (s == 0 ? 0 : B.nx[d] - 1)) continue;
    const int t = d == 0 ? j : i;
    const double area = d == 0 ? B.dx[1] * B.dx[2] : B.dx[0] * B.dx[2];
    const int tg2 = 2 * (B.amr.origin[td] + t);
    const StepBlock &F = amr_fine_nbr(a.blocks, B, face, td, tg2);
    const int ft = tg2 - F.amr.origin[td];
    const double *fb = F.bflux + (size_t)(2 * d + 1 - s) * a.bflux_stride;
    const double Fold = B.bflux[(size_t)face * a.bflux_stride + (size_t)t * nv + v];
    const double Fnew = 0.5 * (fb[(size_t)ft * nv + v] + fb[(size_t)(ft + 1) * nv + v]);
    x = s == 0 ? x + (area * Fold - area * Fnew) : x + (area * Fnew - area * Fold);
  }
  return x;
}

__device__ void amr_fix(const StageArgs &a, const Sched &sched, unsigned int *ctr,
                        unsigned long long &dtmin) {
  const PackDev &p = a.p;
  for (int it = sched.first(ctr, a.nfix_items); it < a.nfix_items; it = sched.next(ctr, a.nfix_items, it)) {
    const StepBlock &B = a.blocks[a.fix_items[it]];
    const int fmask = amr_finer_mask(B);
    const GasConsts gc = gas_of(a, B);
    const double beta_dt = a.beta * dt_of(a, B);
    const long long nc = B.ncell;
    const double vol = B.dx[0] * B.dx[1] * B.dx[2];
    const double ivol = 1.0 / vol;
#if APH_EXACT
    const bool vol_p2 = pow2_normal(vol);  // power-of-two volume: exact multiplication
#endif
    for (long long ic = threadIdx.x; ic < B.nint; ic += blockDim.x) {
      if (!amr_defers(fmask, B, ic)) continue;
      const int j = (int)(ic / B.nx[0]), i = (int)(ic - (long long)j * B.nx[0]);
      const long long c = (long long)(j + p.ng) * B.ni + (i + p.ng);
      double u[NHYDRO];
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) {
        const double du = amr_fixed_du(a, B, fmask, i, j, ic, v);
#if APH_EXACT
        const double div = div_vol(-du, vol, ivol, vol_p2);
#else
        const double div = -du * ivol;
#endif
        u[v] = a.gam0 * B.u0[v * nc + c] + a.gam1 * B.u1[v * nc + c] + beta_dt * div;
      }
      bool bad = false;
      for (int v = NHYDRO; v < p.nvar; ++v) {  // passive scalars
        const double du = amr_fixed_du(a, B, fmask, i, j, ic, v);
#if APH_EXACT
        const double div = div_vol(-du, vol, ivol, vol_p2);
#else
        const double div = -du * ivol;
#endif
        const double x = a.gam0 * B.u0[v * nc + c] + a.gam1 * B.u1[v * nc + c] + beta_dt * div;
        B.u0[v * nc + c] = x;
        bad |= ((__double_as_longlong(x) >> 52) & 0x7ff) == 0x7ff;
      }
      if (a.gravity) {  // ApplyGravity with the stage input's prim (gravity.cpp:386-407)
        const double rho = B.prim[IDN * nc + c];
        u[IM1] += a.grav[0] * rho * beta_dt;
        double de = a.grav[0] * B.prim[IV1 * nc + c];
        u[IM2] += a.grav[1] * rho * beta_dt;
        de += a.grav[1] * B.prim[IV2 * nc + c];
        u[IEN] += de * rho * beta_dt;
      }
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v)
        bad |= ((__double_as_longlong(u[v]) >> 52) & 0x7ff) == 0x7ff;  // NaN or inf
      if (bad) a.ctl->nonfinite = 1;
      if (a.last) {  // dt of the floored new state, which is stored floored (as in pass_item)
        double wv[NHYDRO], gcc, gce;
        const double e_raw = u[IEN];
        const bool fl = cons_to_prim_cell(u, wv, gcc, gce, gc.gm1, p.dfloor, p.pfloor);
        const unsigned long long b = dt_bits(dt_cell(wv, u[IEN], B.dx, p.ndim, gc, fl));
        dtmin = b < dtmin ? b : dtmin;
        store_floored_energy(B, c, e_raw, u[IEN]);
      }
#pragma unroll
      for (int v = 0; v < NHYDRO; ++v) B.u0[v * nc + c] = u[v];
    }
  }
}

// MINB: resident CTAs per SM the registers are budgeted for (1: as many registers as the code
// wants; 3: capped near 80 per thread for 256-thread CTAs, trading a few spills for occupancy).
template <int RECON, int RS, int MINB>
__global__ void __launch_bounds__(kStageThreads, MINB) k_stage(StageArgs a) {
  extern __shared__ __align__(128) double sm[];
  __shared__ __align__(8) unsigned long long s_mbar;
  const unsigned mbar = smem_addr(&s_mbar);
  unsigned tma_phase = 0;
  if (a.tmaps && threadIdx.x == 0) {
    mbar_init(mbar);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  const PackDev &p = a.p;
  const Sched sched{a.schedule};
  unsigned long long dtmin = ~0ULL;
  unsigned int *ctr = a.ctl->work;

  // this launch's number (read by every CTA before the first barrier, advanced after it)
  const unsigned long long epoch = *(volatile unsigned long long *)&a.block_flags[2 * p.nblocks] + 1;

  // phase 1: per cell, its ghost values (from the neighbours' interiors and the physical
  // boundaries, unless the caller filled them, e.g. by a halo exchange), then ConsToPrim.
  // Ghost cells are floored in place.  Other blocks read interior cells for their ghosts
  // during this phase, so a floored interior cell's density and energy wait in its du slots
  // (tagged) until the first pass stores them.  In init mode only the dt estimate of the
  // interior is made and nothing is written.
  for (int it = sched.first(ctr + 1, a.ncell_items); it < a.ncell_items;
       it = sched.next(ctr + 1, a.ncell_items, it)) {
    const int2 w = a.cell_items[it];
    const StepBlock &B = a.blocks[w.x];
    if (!active_of(a, B)) continue;
    const long long c = (long long)w.y + threadIdx.x;
    const double gm1 = a.members ? a.members[B.member].gm1 : p.gm1;
    if (a.init) {  // dt estimate of the interior
      unsigned long long cand = ~0ULL;
      int i, j, k;
      if (c < B.ncell && is_interior(p, B, c, i, j, k)) {
        double u[NHYDRO], wv[NHYDRO], g_c, g_e;
#pragma unroll
        for (int n = 0; n < NHYDRO; ++n) u[n] = B.u0[n * B.ncell + c];
        u[IEN] = energy_in(B, c, true);  // the state of a step boundary
        cons_to_prim_cell(u, wv, g_c, g_e, gm1, p.dfloor, p.pfloor);
        cand = dt_bits(dt_candidate(wv, u[IEN], B.dx, p.ndim, gm1));
      }
      if (a.members) member_min(a, B.member, cand);
      else dtmin = cand < dtmin ? cand : dtmin;
      continue;
    }
    if (c >= B.ncell) continue;
    int i, j, k;
    const bool inner = is_interior(p, B, c, i, j, k);
    // the passes read ghost cells only along their lines, at most G cells beyond the interior:
    // the others (edges, corners, the layers beyond G) are neither filled nor converted
    if (!inner && !a.full_domain && !pass_reads(p, B, i, j, k, Halo<RECON>::G)) continue;
    // and a ghost that copies an interior cell is read at that cell (ghost_copy_src)
    if (!inner && ghosts_from_sources(a) && ghost_is_copy(p, B, i, j, k)) continue;
    if (!inner && !a.ghosts_given) {  // the ghost values of u0 (read back below by this thread)
      if (p.amr) {
        const bool start = a.copy_u1;
        amr_fill_cell(
            a.blocks, B,
            [start](const StepBlock &X, int v, long long q) {
              return v == IEN ? energy_in(X, q, start) : X.u0[v * X.ncell + q];
            },
            B.u0, p.nvar, p.bc, p.ng, c);
      } else {
        ghost_cell(a, B, c);
      }
    }
    const long long nc = B.ncell;
    double u[NHYDRO], wv[NHYDRO], g_c, g_e;
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) u[n] = B.u0[n * nc + c];
    const double ud0 = u[IDN], ue0 = u[IEN];
    u[IEN] = energy_in(B, c, a.copy_u1);
    const bool fl = cons_to_prim_cell(u, wv, g_c, g_e, gm1, p.dfloor, p.pfloor);
    const bool changed = __double_as_longlong(u[IDN]) != __double_as_longlong(ud0) ||
                         __double_as_longlong(u[IEN]) != __double_as_longlong(ue0);
    if (changed && !inner) {
      B.u0[IDN * nc + c] = u[IDN];
      B.u0[IEN * nc + c] = u[IEN];
    } else if (changed) {
      const int sj = p.ndim >= 2 ? p.ng : 0, sk = p.ndim >= 3 ? p.ng : 0;
      const long long ic = ((long long)(k - sk) * B.nx[1] + (j - sj)) * B.nx[0] + (i - p.ng);
      B.du[IDN * B.nint + ic] = u[IDN];
      B.du[IEN * B.nint + ic] = u[IEN];
      B.du[IM1 * B.nint + ic] = __longlong_as_double((long long)kDeferTag);
      a.block_flags[2 * w.x + 1] = epoch;
    }
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) B.prim[n * nc + c] = wv[n];
    B.gamma[c] = g_c;
    B.gamma[nc + c] = g_e;
    if (p.nvar > NHYDRO) {  // passive scalars: concentration = cons / floored density
      const double di = 1.0 / u[IDN];
      for (int n = NHYDRO; n < p.nvar; ++n) {
        const double q = B.u0[n * nc + c];
        B.prim[n * nc + c] = q * di;
        if (a.copy_u1 && inner) B.u1[n * nc + c] = q;
      }
    }
    if (fl) a.block_flags[2 * w.x] = epoch;
    if (a.copy_u1 && inner) {
#pragma unroll
      for (int n = 0; n < NHYDRO; ++n) B.u1[n * nc + c] = u[n];
    }
  }
  if (a.init) {
    dtmin = block_min(dtmin);
    if (threadIdx.x == 0 && dtmin != ~0ULL) atomicMin(&a.ctl->min_bits, dtmin);
    return;
  }
  if (!grid_barrier(a.ctl, a.timeout_ns, gridDim.x)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) a.block_flags[2 * p.nblocks] = epoch;

  // phases 2..: one pass per direction
  for (int pi = 0; pi < p.ndim; ++pi) {
    const int dir = a.order[pi];
    const int nit = a.nline_items[dir - 1];
    const int T = a.T[dir - 1];
    const bool first_pass = pi == 0, last_pass = pi == p.ndim - 1;
    for (int it = sched.first(ctr + 2 + pi, nit); it < nit; it = sched.next(ctr + 2 + pi, nit, it)) {
      const int2 w = a.line_items[dir - 1][it];
      const StepBlock &B = a.blocks[w.x];
      if (!active_of(a, B)) continue;
      const int lfirst = w.y >> kItemLineBits, nl = w.y & ((1 << kItemLineBits) - 1);
      // shared-memory layout: the TMA box's lines, else the item's own
      const int Ti = a.tmaps ? T : nl;
#if APH_EXACT
      const bool constg = false;
#else
      const bool constg = a.block_flags[2 * w.x] != epoch;
#endif
      const bool deferred = first_pass && a.block_flags[2 * w.x + 1] == epoch;
      // the item's lines, in chunks that fit the gamma slabs where they are reconstructed
      const int Tc = constg ? Ti : split_lines(Ti, p.nvar);
      for (int o = 0; o < nl; o += Tc) {
        const int l0 = lfirst + o, nc = min(Tc, nl - o);
        bool ok;
        if (dir == 1)
          ok = pass_item<1, RECON, RS>(a, B, w.x, l0, nc, Tc, constg, deferred, first_pass, last_pass, sm, dtmin,
                                       mbar, tma_phase);
        else if (dir == 2)
          ok = pass_item<2, RECON, RS>(a, B, w.x, l0, nc, Tc, constg, deferred, first_pass, last_pass, sm, dtmin,
                                       mbar, tma_phase);
        else
          ok = pass_item<3, RECON, RS>(a, B, w.x, l0, nc, Tc, constg, deferred, first_pass, last_pass, sm, dtmin,
                                       mbar, tma_phase);
        if (!ok) return;  // a TMA wait ran out (APH_ERR_TIMEOUT is recorded)
      }
    }
    if (!last_pass && !grid_barrier(a.ctl, a.timeout_ns, gridDim.x)) return;
  }
  if (a.cf) {  // the coarse-fine boundary cells, once every block's face fluxes are kept
    if (!grid_barrier(a.ctl, a.timeout_ns, gridDim.x)) return;
    amr_fix(a, sched, ctr + 6, dtmin);
  }
  if (a.last) {
    dtmin = block_min(dtmin);
    if (threadIdx.x == 0 && dtmin != ~0ULL) atomicMin(&a.ctl->min_bits, dtmin);
  }
}

// Failure-path probe: one CTA waits at a grid barrier for one more CTA than the launch has,
// so the wait runs out after timeout_ns and records APH_ERR_TIMEOUT in ctl.
__global__ void k_barrier_probe(StepCtl *ctl, unsigned long long timeout_ns) {
  grid_barrier(ctl, timeout_ns, gridDim.x + 1);
}

// ---- host side ---------------------------------------------------------------------------
cudaError_t launch_barrier_probe(StepCtl *ctl, unsigned long long timeout_ns, cudaStream_t s) {
  k_barrier_probe<<<1, 32, 0, s>>>(ctl, timeout_ns);
  return cudaGetLastError();
}

// Items of T lines with nvar + kGammaSlabs slabs, and single-line chunks with the gamma slabs
// (split_lines never returns less than one line).
size_t stage_smem_bytes(int recon, int n, int T, int nvar) {
  const size_t a = pass_smem_doubles(recon, n, T, nvar + kGammaSlabs);
  const size_t b = pass_smem_doubles(recon, n, 1, nvar + 2);
  return (a > b ? a : b) * sizeof(double);
}

// With TMA staging: the window region padded to 128 bytes, then the larger of the remaining
// pass regions and the staging area (nvar variables x T lines x the line's entire extent L).
size_t stage_smem_bytes_tma(int recon, int n, int T, int L, int nvar) {
  const int V = nvar + kGammaSlabs;
  const size_t rest = pass_smem_doubles(recon, n, T, V) -
                      (size_t)V * T * (n + 2 * (recon == RECON_PPM ? 3 : recon == RECON_PLM ? 2 : 1));
  const size_t stage = (size_t)2 * nvar * T * L;  // two boxes for items that cross a plane
  const size_t tma = (tma_stage_offset(recon, n, T, nvar) + 16 + (rest > stage ? rest : stage)) * sizeof(double);
  const size_t plain = stage_smem_bytes(recon, n, T, nvar);
  return tma > plain ? tma : plain;
}

template <int RECON, int MINB>
static const void *kernel_for_rs(int rs) {
  switch (rs) {
    case RS_HLLE: return (const void *)k_stage<RECON, RS_HLLE, MINB>;
    case RS_HLLC: return (const void *)k_stage<RECON, RS_HLLC, MINB>;
    case RS_LHLLC: return (const void *)k_stage<RECON, RS_LHLLC, MINB>;
    case RS_NONE: return RECON == RECON_DC ? (const void *)k_stage<RECON_DC, RS_NONE, MINB> : nullptr;
    default: return nullptr;
  }
}

template <int MINB>
static const void *stage_kernel_t(int recon, int rsolver) {
  if (recon == RECON_PPM) return kernel_for_rs<RECON_PPM, MINB>(rsolver);
  if (recon == RECON_PLM) return kernel_for_rs<RECON_PLM, MINB>(rsolver);
  if (recon == RECON_DC) return kernel_for_rs<RECON_DC, MINB>(rsolver);
  return nullptr;
}

const void *stage_kernel(int recon, int rsolver, int reg_cap) {
  return reg_cap ? stage_kernel_t<3>(recon, rsolver) : stage_kernel_t<1>(recon, rsolver);
}

cudaError_t stage_occupancy(int recon, int rsolver, int threads, size_t smem, int reg_cap, int *blocks) {
  const void *k = stage_kernel(recon, rsolver, reg_cap);
  if (!k) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, k, threads, smem);
}

cudaError_t launch_stage(const StageArgs &a, int recon, int rsolver, int grid, int threads,
                         size_t smem, bool cooperative, int reg_cap, cudaStream_t s) {
  const void *k = stage_kernel(recon, rsolver, reg_cap);
  if (!k) return cudaErrorInvalidValue;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = cooperative ? 1 : 0;
  void *args[] = {(void *)&a};
  return cudaLaunchKernelExC(&cfg, k, args);
}

}  // namespace APH_NS
