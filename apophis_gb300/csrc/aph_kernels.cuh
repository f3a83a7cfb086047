// aph_kernels.cuh -- per-pack kernels of the hydro path (the reference-style launch
// granularity: one kernel per operation over all meshblocks of a pack).
//
// Included once per arithmetic mode with APH_NS naming the namespace
// (aph_fast.cu, aph_exact.cu).
#pragma once
#include "aph_amr.cuh"
#include "aph_internal.h"
#include "aph_math.cuh"

#ifndef APH_NS
#error "APH_NS must name the namespace of this translation unit"
#endif

namespace APH_NS {

using namespace aph;

constexpr int kThreads = 256;

__device__ __forceinline__ int dim_start(int d, int ndim, int ng) { return d < ndim ? ng : 0; }

// ---------------------------------------------------------------------------------------
// ConsToPrim over the entire domain of every block (hydro.cpp:450-532)
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_cons_to_prim(PackDev p, const BlockDev *blocks,
                                                           int *floor_flag) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= B.ncell) return;
  const long long nc = B.ncell;
  double u[NHYDRO], w[NHYDRO], g_c, g_e;
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) u[n] = B.cons[n * nc + c];
  const bool fl = cons_to_prim_cell(u, w, g_c, g_e, p.gm1, p.dfloor, p.pfloor);
  B.cons[IDN * nc + c] = u[IDN];
  B.cons[IEN * nc + c] = u[IEN];
#pragma unroll
  for (int n = 0; n < NHYDRO; ++n) B.prim[n * nc + c] = w[n];
  if (B.gamma) {
#if !APH_EXACT
    // the flux kernels reconstruct these fields: the reference's values, not the constants
    // the fast ConsToPrim leaves where no floor fired
    if (!fl) gamma_ref(u, p.gm1, g_c, g_e);
#endif
    B.gamma[c] = g_c;
    B.gamma[nc + c] = g_e;
  }
  if (p.nvar > NHYDRO) {
    const double di = 1.0 / u[IDN];
    for (int n = NHYDRO; n < p.nvar; ++n) B.prim[n * nc + c] = B.cons[n * nc + c] * di;
  }
  if (B.eos_lambda && B.eos_lambda[2 * nc + c] == 0.0) B.eos_lambda[2 * nc + c] = 7.0;  // hydro.cpp:491-493
  if (fl && floor_flag) atomicOr(floor_flag, 1);
}

// ---------------------------------------------------------------------------------------
// CalculateFluxes for one direction (hydro.cpp:580-740): reconstruction of every
// primitive and both adiabatic indices on the cells s-1..e+1 of each line, then the
// Riemann solve on the faces s..e+1.  A CTA takes T whole lines; the face states go
// through shared memory and never reach HBM.  Only lines through the interior are
// computed (the reference also fills the unused fluxes on ghost rows).
// ---------------------------------------------------------------------------------------
template <int RECON>
__device__ __forceinline__ void recon_strided(const double *q, long long s, double &ql, double &qr) {
  if (RECON == RECON_DC) {
    ql = qr = q[0];
  } else if (RECON == RECON_PLM) {
    plm(q[-s], q[0], q[s], ql, qr);
  } else {
    ppm(q[-2 * s], q[-s], q[0], q[s], q[2 * s], ql, qr);
  }
}

template <int DIR>
__device__ __forceinline__ void line_geometry(const BlockDev &B, int ndim, int ng, int line,
                                              int &i0, int &j0, int &k0, long long &s,
                                              int &n) {
  const int si = ng, sj = dim_start(1, ndim, ng), sk = dim_start(2, ndim, ng);
  if (DIR == 1) {
    n = B.nx[0];
    s = 1;
    j0 = sj + line % B.nx[1];
    k0 = sk + line / B.nx[1];
    i0 = si;
  } else if (DIR == 2) {
    n = B.nx[1];
    s = B.ni;
    i0 = si + line % B.nx[0];
    k0 = sk + line / B.nx[0];
    j0 = sj;
  } else {
    n = B.nx[2];
    s = (long long)B.ni * B.nj;
    i0 = si + line % B.nx[0];
    j0 = sj + line / B.nx[0];
    k0 = sk;
  }
}

template <int DIR, int RECON, int RS>
__global__ void __launch_bounds__(kThreads) k_fluxes(PackDev p, const BlockDev *blocks, int T) {
  extern __shared__ double sm[];
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  const int ntrans = (DIR == 1) ? B.nx[1] * B.nx[2] : (DIR == 2) ? B.nx[0] * B.nx[2] : B.nx[0] * B.nx[1];
  const int line0 = blockIdx.x * T;
  if (line0 >= ntrans) return;
  const int nl = min(T, ntrans - line0);
  const int n = B.nx[DIR - 1];
  const int P = n + 2;  // slots: cell c in [-1, n] stores at slot c+1
  const int V = p.nvar + 2;
  const int maxP = p.max_nx[DIR - 1] + 2;
  double *sL = sm;                      // [V][T][maxP]: left state of face slot
  double *sR = sm + (size_t)V * T * maxP;  // [V][T][maxP]: right state of face slot-1
  const long long nc = B.ncell;
  const int nvar = p.nvar;

  // phase 1: reconstruction, one item per (line, cell)
  const int n1 = nl * P;
  for (int it = threadIdx.x; it < n1; it += blockDim.x) {
    int t, slot;
    if (DIR == 1) { t = it / P; slot = it - t * P; }
    else { slot = it / nl; t = it - slot * nl; }
    int i0, j0, k0, ln;
    long long s;
    line_geometry<DIR>(B, p.ndim, p.ng, line0 + t, i0, j0, k0, s, ln);
    const long long cell = ((long long)k0 * B.nj + j0) * B.ni + i0 + (long long)(slot - 1) * s;
    const size_t o = ((size_t)t) * maxP + slot;
    for (int v = 0; v < nvar; ++v) {
      double ql, qr;
      recon_strided<RECON>(B.prim + v * nc + cell, s, ql, qr);
      sL[(size_t)v * T * maxP + o] = ql;  // left state of face c+1 (slot c+1)
      sR[(size_t)v * T * maxP + o] = qr;  // right state of face c   (slot c+1)
    }
    for (int v = 0; v < 2; ++v) {
      double ql, qr;
      recon_strided<RECON>(B.gamma + v * nc + cell, s, ql, qr);
      sL[(size_t)(nvar + v) * T * maxP + o] = ql;
      sR[(size_t)(nvar + v) * T * maxP + o] = qr;
    }
  }
  __syncthreads();

  // phase 2: Riemann solve, one item per (line, face); face f in [0, n]
  constexpr int ivx = DIR;
  constexpr int ivy = IV1 + ((ivx - IV1) + 1) % 3;
  constexpr int ivz = IV1 + ((ivx - IV1) + 2) % 3;
  const GasConsts gc{};
  double *flux = B.flux[DIR - 1];
  const int nf = n + 1;
  const int n2 = nl * nf;
  for (int it = threadIdx.x; it < n2; it += blockDim.x) {
    int t, f;
    if (DIR == 1) { t = it / nf; f = it - t * nf; }
    else { f = it / nl; t = it - f * nl; }
    int i0, j0, k0, ln;
    long long s;
    line_geometry<DIR>(B, p.ndim, p.ng, line0 + t, i0, j0, k0, s, ln);
    // face f of the line: cell (k0, j0, i0) moved f cells along DIR, in flux[DIR-1]'s layout
    const long long* fs = B.fs[DIR - 1];
    const long long fcell = (long long)(k0 + (DIR == 3 ? f : 0)) * fs[1] +
                            (long long)(j0 + (DIR == 2 ? f : 0)) * fs[2] + (i0 + (DIR == 1 ? f : 0));
    const long long fn = fs[0];
    const size_t oL = ((size_t)t) * maxP + f;      // ql_f  (from cell f-1)
    const size_t oR = ((size_t)t) * maxP + f + 1;  // qr_f  (from cell f)
    const size_t vs = (size_t)T * maxP;
    double wl[NHYDRO], wr[NHYDRO], flx[NHYDRO];
    wl[IDN] = sL[IDN * vs + oL]; wl[IV1] = sL[ivx * vs + oL]; wl[IV2] = sL[ivy * vs + oL];
    wl[IV3] = sL[ivz * vs + oL]; wl[IPR] = sL[IPR * vs + oL];
    wr[IDN] = sR[IDN * vs + oR]; wr[IV1] = sR[ivx * vs + oR]; wr[IV2] = sR[ivy * vs + oR];
    wr[IV3] = sR[ivz * vs + oR]; wr[IPR] = sR[IPR * vs + oR];
    riemann<RS, false>(wl, wr, sL[nvar * vs + oL], sL[(nvar + 1) * vs + oL],
                       sR[nvar * vs + oR], sR[(nvar + 1) * vs + oR], gc, flx);
    flux[IDN * fn + fcell] = flx[IDN];
    flux[ivx * fn + fcell] = flx[IV1];
    flux[ivy * fn + fcell] = flx[IV2];
    flux[ivz * fn + fcell] = flx[IV3];
    flux[IEN * fn + fcell] = flx[IEN];
    // passive scalars: upwind by the mass flux (hydro.cpp:607-615)
    for (int v = NHYDRO; v < nvar; ++v)
      flux[v * fn + fcell] = flx[IDN] * (!is_neg(flx[IDN]) ? sL[v * vs + oL] : sR[v * vs + oR]);
  }
}

// ---------------------------------------------------------------------------------------
// UpdateWithFluxDivergence over the interior: u0 = gam0 u0 + gam1 u1 + beta_dt (-div F)
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool interior_cell(const BlockDev &B, int ndim, int ng, int idx,
                                              long long &cell, int &ci, int &cj, int &ck) {
  const int n0 = B.nx[0], n1 = B.nx[1], n2 = B.nx[2];
  if (idx >= n0 * n1 * n2) return false;
  const int i = idx % n0, j = (idx / n0) % n1, k = idx / (n0 * n1);
  const int si = ng, sj = dim_start(1, ndim, ng), sk = dim_start(2, ndim, ng);
  ci = i + si;
  cj = j + sj;
  ck = k + sk;
  cell = ((long long)ck * B.nj + cj) * B.ni + ci;
  return true;
}
// Index of face (k, j, i) of component n in flux[d] (face i on the low side of cell i).
__device__ __forceinline__ long long flux_index(const BlockDev &B, int d, int n, int k, int j, int i) {
  return n * B.fs[d][0] + k * B.fs[d][1] + j * B.fs[d][2] + i;
}

__global__ void __launch_bounds__(kThreads) k_update(PackDev p, const BlockDev *blocks,
                                                     double gam0, double gam1, double beta,
                                                     double beta_dt_host, const double *dt_dev) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  long long c;
  int ci, cj, ck;
  if (!interior_cell(B, p.ndim, p.ng, blockIdx.x * blockDim.x + threadIdx.x, c, ci, cj, ck)) return;
  const double beta_dt = dt_dev ? beta * dt_dev[0] : beta_dt_host;
  const double a1 = B.dx[1] * B.dx[2], a2 = B.dx[0] * B.dx[2], a3 = B.dx[0] * B.dx[1];
  const double vol = B.dx[0] * B.dx[1] * B.dx[2];
  const long long nc = B.ncell;
  for (int n = 0; n < p.nvar; ++n) {
    const long long q = n * nc + c;
    const long long f1 = flux_index(B, 0, n, ck, cj, ci);
    double du = (a1 * B.flux[0][f1 + 1] - a1 * B.flux[0][f1]);
    if (p.ndim >= 2) {
      const long long f2 = flux_index(B, 1, n, ck, cj, ci);
      du += (a2 * B.flux[1][f2 + B.fs[1][2]] - a2 * B.flux[1][f2]);
    }
    if (p.ndim == 3) {
      const long long f3 = flux_index(B, 2, n, ck, cj, ci);
      du += (a3 * B.flux[2][f3 + B.fs[2][1]] - a3 * B.flux[2][f3]);
    }
    const double div = -du / vol;
    B.cons[q] = gam0 * B.cons[q] + gam1 * B.u1[q] + beta_dt * div;
  }
}

// Face (a along d, t across) of component n of flux[d] of a 2D block (as amr_cell).
__device__ __forceinline__ long long amr_face(const BlockDev &B, int ng, int d, int n, int a, int t) {
  const int i = d == 0 ? ng + a : ng + t;
  const int j = d == 0 ? ng + t : ng + a;
  return flux_index(B, d, n, 0, j, i);
}

// Refined 2D meshes: the same update with the coarse-fine correction of each coarse
// boundary cell's flux difference to the mean of the fine face fluxes (faces x-, x+, y-, y+).
__global__ void __launch_bounds__(kThreads) k_update_amr(PackDev p, const BlockDev *blocks,
                                                         double gam0, double gam1, double beta,
                                                         double beta_dt_host, const double *dt_dev) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  long long c;
  int ci, cj, ck;
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (!interior_cell(B, p.ndim, p.ng, idx, c, ci, cj, ck)) return;
  const int ii = idx % B.nx[0], jj = idx / B.nx[0];
  const double beta_dt = dt_dev ? beta * dt_dev[0] : beta_dt_host;
  const double a1 = B.dx[1] * B.dx[2], a2 = B.dx[0] * B.dx[2];
  const double vol = B.dx[0] * B.dx[1] * B.dx[2];
  const long long nc = B.ncell;
  for (int n = 0; n < p.nvar; ++n) {
    const long long q = n * nc + c;
    const long long f1 = flux_index(B, 0, n, 0, cj, ci), f2 = flux_index(B, 1, n, 0, cj, ci);
    double du = (a1 * B.flux[0][f1 + 1] - a1 * B.flux[0][f1]);
    du += (a2 * B.flux[1][f2 + B.fs[1][2]] - a2 * B.flux[1][f2]);
    for (int face = 0; face < 4; ++face) {
      if (B.amr.kind[face] != FACE_FINER) continue;
      const int d = face / 2, s = face % 2, td = 1 - d;
      const int a = d == 0 ? ii : jj, t = d == 0 ? jj : ii;
      if (a != (s == 0 ? 0 : B.nx[d] - 1)) continue;
      const double area = d == 0 ? a1 : a2;
      const int tg2 = 2 * (B.amr.origin[td] + t);
      const BlockDev &F = amr_fine_nbr(blocks, B, face, td, tg2);
      const int ft = tg2 - F.amr.origin[td];
      const long long fo = amr_face(B, p.ng, d, n, s == 0 ? 0 : B.nx[d], t);
      const int ffa = s == 0 ? F.nx[d] : 0;
      const long long g0 = amr_face(F, p.ng, d, n, ffa, ft);
      const long long g1 = amr_face(F, p.ng, d, n, ffa, ft + 1);
      const double Fold = B.flux[d][fo];
      const double Fnew = 0.5 * (F.flux[d][g0] + F.flux[d][g1]);
      du = s == 0 ? du + (area * Fold - area * Fnew) : du + (area * Fnew - area * Fold);
    }
    const double div = -du / vol;
    B.cons[q] = gam0 * B.cons[q] + gam1 * B.u1[q] + beta_dt * div;
  }
}

// ---------------------------------------------------------------------------------------
// EstimateTimestep (hydro.cpp:369-417): per-cell candidate, warp-shuffle min, one
// atomic per CTA on the bit pattern (positive doubles order like unsigned integers,
// NaN candidates sort above +inf and are ignored as fmin ignores them).
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long block_min_bits(unsigned long long v) {
  __shared__ unsigned long long red[kThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x < v ? x : v;
  }
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

__global__ void __launch_bounds__(kThreads) k_estimate_dt(PackDev p, const BlockDev *blocks,
                                                          unsigned long long *min_bits) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  long long c;
  unsigned long long v = ~0ULL;
  int ci, cj, ck;
  if (interior_cell(B, p.ndim, p.ng, blockIdx.x * blockDim.x + threadIdx.x, c, ci, cj, ck)) {
    const long long nc = B.ncell;
    double w[NHYDRO];
#pragma unroll
    for (int n = 0; n < NHYDRO; ++n) w[n] = B.prim[n * nc + c];
    const double m = dt_candidate(w, B.cons[IEN * nc + c], B.dx, p.ndim, p.gm1);
    v = (unsigned long long)__double_as_longlong(m);
    if (is_neg(m)) v = ~0ULL;
  }
  v = block_min_bits(v);
  if (threadIdx.x == 0 && v != ~0ULL) atomicMin(min_bits, v);
}

// ---------------------------------------------------------------------------------------
// ApplyGravity, constant field (gravity.cpp:386-407); prim is the state of the previous
// FillDerived, as in the reference.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_apply_gravity(PackDev p, const BlockDev *blocks,
                                                            double g0, double g1, double g2,
                                                            double beta, double beta_dt_host,
                                                            const double *dt_dev) {
  const BlockDev &B = blocks[p.block0 + blockIdx.y];
  long long c;
  int ci, cj, ck;
  if (!interior_cell(B, p.ndim, p.ng, blockIdx.x * blockDim.x + threadIdx.x, c, ci, cj, ck)) return;
  const double dt = dt_dev ? beta * dt_dev[0] : beta_dt_host;
  const long long nc = B.ncell;
  const double rho = B.prim[IDN * nc + c];
  B.cons[IM1 * nc + c] += g0 * rho * dt;
  double de = g0 * B.prim[IV1 * nc + c];
  if (p.ndim >= 2) {
    B.cons[IM2 * nc + c] += g1 * rho * dt;
    de += g1 * B.prim[IV2 * nc + c];
  }
  if (p.ndim >= 3) {
    B.cons[IM3 * nc + c] += g2 * rho * dt;
    de += g2 * B.prim[IV3 * nc + c];
  }
  B.cons[IEN * nc + c] += de * rho * dt;
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
static inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

// Launch shapes.  FP64 issue is a per-SM resource (a few lanes per clock), so a launch
// that covers few SMs -- one small meshblock at a time -- is bound by the latency of its
// longest thread.  Small launches therefore use fewer threads (or lines) per CTA, down to
// one warp, until the grid spans about two CTAs per SM; launches over a whole pack keep the
// full CTA.  The arithmetic of every cell is the same for any shape.
static int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  if (!cached[dev]) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 152;
    cached[dev] = n;
  }
  return cached[dev];
}

static int launch_threads(long long work, int nblocks) {
  const long long want = 2LL * sm_count();
  int t = kThreads;
  while (t > 32 && (long long)cdiv(work, t) * nblocks < want) t >>= 1;
  return t;
}

cudaError_t launch_cons_to_prim(const PackDev &p, const BlockDev *blocks, int max_ncell,
                                int *floor_flag, cudaStream_t s) {
  const int nt = launch_threads(max_ncell, p.nblocks);
  dim3 grid(cdiv(max_ncell, nt), p.nblocks);
  k_cons_to_prim<<<grid, nt, 0, s>>>(p, blocks, floor_flag);
  return cudaGetLastError();
}

template <int DIR, int RECON, int RS>
static cudaError_t launch_fluxes_t(const PackDev &p, const BlockDev *blocks, cudaStream_t s) {
  const int n = p.max_nx[DIR - 1];
  long long ntrans;
  if (DIR == 1) ntrans = (long long)p.max_nx[1] * p.max_nx[2];
  else if (DIR == 2) ntrans = (long long)p.max_nx[0] * p.max_nx[2];
  else ntrans = (long long)p.max_nx[0] * p.max_nx[1];
  int T = (n + 2 >= kThreads) ? 1 : kThreads / (n + 2);
  while (T > 1 && (long long)cdiv(ntrans, T) * p.nblocks < 2LL * sm_count()) T = (T + 1) / 2;
  const int nt = (int)std::min<long long>(kThreads, 32LL * cdiv((long long)T * (n + 2), 32));
  const int V = p.nvar + 2;
  const size_t smem = (size_t)2 * V * T * (n + 2) * sizeof(double);
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  static bool attr_set = false;
  if (!attr_set || smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_fluxes<DIR, RECON, RS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  dim3 grid(cdiv(ntrans, T), p.nblocks);
  k_fluxes<DIR, RECON, RS><<<grid, nt, smem, s>>>(p, blocks, T);
  return cudaGetLastError();
}

template <int DIR>
static cudaError_t launch_fluxes_dir(const PackDev &p, const BlockDev *blocks, int recon,
                                     int rsolver, cudaStream_t s) {
#define APH_RS_CASES(RC)                                                      \
  switch (rsolver) {                                                          \
    case RS_HLLE: return launch_fluxes_t<DIR, RC, RS_HLLE>(p, blocks, s);     \
    case RS_HLLC: return launch_fluxes_t<DIR, RC, RS_HLLC>(p, blocks, s);     \
    case RS_LHLLC: return launch_fluxes_t<DIR, RC, RS_LHLLC>(p, blocks, s);   \
    default: break;                                                           \
  }
  if (recon == RECON_DC) {
    if (rsolver == RS_NONE) return launch_fluxes_t<DIR, RECON_DC, RS_NONE>(p, blocks, s);
    APH_RS_CASES(RECON_DC)
  } else if (recon == RECON_PLM) {
    APH_RS_CASES(RECON_PLM)
  } else if (recon == RECON_PPM) {
    APH_RS_CASES(RECON_PPM)
  }
#undef APH_RS_CASES
  return cudaErrorInvalidValue;
}

cudaError_t launch_fluxes(const PackDev &p, const BlockDev *blocks, int dir, int recon,
                          int rsolver, cudaStream_t s) {
  if (dir == 1) return launch_fluxes_dir<1>(p, blocks, recon, rsolver, s);
  if (dir == 2) return launch_fluxes_dir<2>(p, blocks, recon, rsolver, s);
  if (dir == 3) return launch_fluxes_dir<3>(p, blocks, recon, rsolver, s);
  return cudaErrorInvalidValue;
}

cudaError_t launch_update(const PackDev &p, const BlockDev *blocks, double gam0, double gam1,
                          double beta, double beta_dt_host, const double *dt_dev,
                          int max_interior, cudaStream_t s) {
  const int nt = launch_threads(max_interior, p.nblocks);
  dim3 grid(cdiv(max_interior, nt), p.nblocks);
  if (p.amr)
    k_update_amr<<<grid, nt, 0, s>>>(p, blocks, gam0, gam1, beta, beta_dt_host, dt_dev);
  else
    k_update<<<grid, nt, 0, s>>>(p, blocks, gam0, gam1, beta, beta_dt_host, dt_dev);
  return cudaGetLastError();
}

cudaError_t launch_estimate_dt(const PackDev &p, const BlockDev *blocks, int max_interior,
                               unsigned long long *min_bits, cudaStream_t s) {
  const int nt = launch_threads(max_interior, p.nblocks);
  dim3 grid(cdiv(max_interior, nt), p.nblocks);
  k_estimate_dt<<<grid, nt, 0, s>>>(p, blocks, min_bits);
  return cudaGetLastError();
}

cudaError_t launch_apply_gravity(const PackDev &p, const BlockDev *blocks, double g0, double g1,
                                 double g2, double beta, double beta_dt_host,
                                 const double *dt_dev, int max_interior, cudaStream_t s) {
  const int nt = launch_threads(max_interior, p.nblocks);
  dim3 grid(cdiv(max_interior, nt), p.nblocks);
  k_apply_gravity<<<grid, nt, 0, s>>>(p, blocks, g0, g1, g2, beta, beta_dt_host, dt_dev);
  return cudaGetLastError();
}

}  // namespace APH_NS
