// aph_adjoint.cu -- hand-written adjoint of the full hydro step, exposed through the C ABI.
//
// For a step U^n -> U^{n+1} with stages u_{s+1} = gam0_s u_s + gam1_s U^n + beta_s dt R(u_s),
// R(u) = -div F(recon(ConsToPrim(ghosts(u)))), the vector-Jacobian product runs the stages
// backwards:
//     a_{S+1} = lambda^{n+1};   for s = S..1:  acc += gam1_s a_{s+1},
//     a_s = gam0_s a_{s+1} + R'(u_s)^T (beta_s dt a_{s+1});      lambda^n = a_1 + acc.
// R'(u)^T mu is one pass per direction (recompute the face states, HLLE/HLLC vjp, PPM/PLM/DC
// vjp, gathered per cell without atomics), then the ConsToPrim vjp per cell, then the ghost
// map transposed (each interior cell gathers the ghost copies made of it).  The forward is the
// batched stage kernel of an internal stepper over the adjoint's state, so the adjoint
// linearises exactly the step the batched path takes, ensembles (per-member gamma and dt)
// included.  Rollouts store a checkpoint every K steps; the reverse sweep recomputes each
// segment once, keeping the primitives of every stage input.  Floors are taken as inactive
// (the derivative of a floored cell is undefined); a forward that fires one is reported as
// APH_ERR_STATE.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/aph_hydro.h"
#include "aph_adjoint_math.cuh"
#include "aph_capi_internal.h"

using namespace aph;

namespace {

struct AdjBlock {
  double dx[3];
  int member;
  int loc[3];       // position in a uniform block grid
  AmrFaces faces;   // face tables (same-level and boundary faces)
};

struct AdjMember {
  GasConsts gc;
  double ic2g;      // 1 / (C^2 gamma)
};

// Geometry of the pack (all blocks have the same interior size) and per-block / per-member
// descriptors on the device.
struct AdjGeom {
  int nblocks, ndim, ng;
  int nx[3], ni, nj, nk;
  long long ncell;       // per block, entire
  int nb[3];
  int bc[3][2];
  int faces;             // 1: the ghost map comes from face tables
  const AdjBlock *blk;
  const AdjMember *mem;
};

__host__ __device__ __forceinline__ long long blk_off(const AdjGeom &g, int b) {
  return (long long)b * 5 * g.ncell;
}
__device__ __forceinline__ int dstart(const AdjGeom &g, int d) { return d < g.ndim ? g.ng : 0; }

// ---- per-direction adjoint pass ----------------------------------------------------------
template <int DIR>
__device__ __forceinline__ void adj_line(const AdjGeom &g, int l, long long &base, long long &stride) {
  const int sj = dstart(g, 1), sk = dstart(g, 2);
  if (DIR == 1) {
    base = ((long long)(l / g.nx[1] + sk) * g.nj + (l % g.nx[1] + sj)) * g.ni + g.ng;
    stride = 1;
  } else if (DIR == 2) {
    base = ((long long)(l / g.nx[0] + sk) * g.nj + sj) * g.ni + (l % g.nx[0] + g.ng);
    stride = g.ni;
  } else {
    base = ((long long)sk * g.nj + (l / g.nx[0] + sj)) * g.ni + (l % g.nx[0] + g.ng);
    stride = (long long)g.ni * g.nj;
  }
}

// mu-difference scale of a block: beta dt (of its member) * area / volume
template <int DIR>
__device__ __forceinline__ double pass_scale(const AdjGeom &g, int b, double beta, const double *dt) {
  const AdjBlock &B = g.blk[b];
  const double vol = B.dx[0] * B.dx[1] * B.dx[2];
  const double area = DIR == 1 ? B.dx[1] * B.dx[2] : DIR == 2 ? B.dx[0] * B.dx[2] : B.dx[0] * B.dx[1];
  return beta * dt[B.member] * (area / vol);
}

// Riemann vjp of faces 0..n of nl lines: SL/SR are the face states (slot f / f+1 of width W2),
// MU the stage adjoint of the interior cells; writes GL/GR (adjoints of the face states).
template <int DIR, int RS>
__device__ __forceinline__ void riemann_pass_vjp(const AdjMember &M, int T, int nl, int n, int W2,
                                                 const double *SL, const double *SR,
                                                 const double *MU, double scale, double *GL,
                                                 double *GR) {
  constexpr int ivx = DIR;
  constexpr int ivy = IV1 + ((ivx - IV1) + 1) % 3;
  constexpr int ivz = IV1 + ((ivx - IV1) + 2) % 3;
  const int perm[5] = {IDN, ivx, ivy, ivz, IEN};
  for (int it = threadIdx.x; it < nl * (n + 1); it += blockDim.x) {  // faces 0..n
    const int t = it / (n + 1), f = it % (n + 1);
    double wl[5], wr[5], gf[5], gwl[5], gwr[5];
    for (int k = 0; k < 5; ++k) {
      const int v = perm[k];
      wl[k] = SL[(v * T + t) * W2 + f];
      wr[k] = SR[(v * T + t) * W2 + f + 1];
      const double mhi = f < n ? MU[(v * T + t) * n + f] : 0.0;
      const double mlo = f > 0 ? MU[(v * T + t) * n + f - 1] : 0.0;
      gf[k] = scale * (mhi - mlo);
    }
    if (RS == RS_HLLE) hlle_vjp(wl, wr, M.gc, M.ic2g, gf, gwl, gwr);
    else hllc_vjp(wl, wr, M.gc, M.ic2g, gf, gwl, gwr);
    for (int k = 0; k < 5; ++k) {
      GL[(perm[k] * T + t) * W2 + f] = gwl[k];
      GR[(perm[k] * T + t) * W2 + f] = gwr[k];
    }
  }
}

// PLM / donor-cell pass.
template <int DIR, int RECON, int RS>
__global__ void __launch_bounds__(256, 2) k_adj_pass(AdjGeom g, const double *prim, const double *mu,
                                                  double *lam_w, double beta, const double *dt, int T) {
  extern __shared__ double sm[];
  constexpr int G = RECON == RECON_PLM ? 2 : 1;
  const int b = blockIdx.y;
  const int n = g.nx[DIR - 1];
  const int ntrans = DIR == 1 ? g.nx[1] * g.nx[2] : DIR == 2 ? g.nx[0] * g.nx[2] : g.nx[0] * g.nx[1];
  const int l0 = blockIdx.x * T;
  if (l0 >= ntrans || dt[g.blk[b].member] == 0.0) return;  // a member that did not move
  const int nl = min(T, ntrans - l0);
  const int NW = n + 2 * G, W2 = n + 2;
  double *W = sm;                             // [5][T][NW]  prim window
  double *MU = W + 5 * T * NW;                // [5][T][n]   stage adjoint (interior)
  double *SL = MU + 5 * T * n;                // [5][T][W2]  left state of face slot
  double *SR = SL + 5 * T * W2;               // [5][T][W2]  right state (slot c+1 <- cell c)
  double *GL = SR + 5 * T * W2;               // [5][T][W2]  adjoint of left state, face f
  double *GR = GL + 5 * T * W2;               // [5][T][W2]  adjoint of right state, face f
  double *CC = GR + 5 * T * W2;               // [3][5][T][W2] recon vjp contributions
  double *RR = CC + 3 * 5 * T * W2;           // [5][T][W2]  PLM reciprocal per cell (0: flat)
  const double *P = prim + blk_off(g, b);
  const double *Mu = mu + blk_off(g, b);
  double *LW = lam_w + blk_off(g, b);
  const long long nc = g.ncell;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int it = tid; it < 5 * nl * NW; it += nth) {
    const int v = it / (nl * NW), r = it % (nl * NW), t = r / NW, w = r % NW;
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    W[(v * T + t) * NW + w] = P[v * nc + base + (long long)(w - G) * s];
  }
  for (int it = tid; it < 5 * nl * n; it += nth) {
    const int v = it / (nl * n), r = it % (nl * n), t = r / n, c = r % n;
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    MU[(v * T + t) * n + c] = Mu[v * nc + base + (long long)c * s];
  }
  __syncthreads();
  auto q = [&](int v, int t, int c) { return W[(v * T + t) * NW + c + G]; };
  for (int it = tid; it < 5 * nl * W2; it += nth) {  // cells -1..n
    const int v = it / (nl * W2), r = it % (nl * W2), t = r / W2, c = r % W2 - 1;
    double ql, qr;
    if (RECON == RECON_PLM) RR[(v * T + t) * W2 + c + 1] = plm_keep(q(v, t, c - 1), q(v, t, c), q(v, t, c + 1), ql, qr);
    else ql = qr = q(v, t, c);
    SL[(v * T + t) * W2 + c + 1] = ql;
    SR[(v * T + t) * W2 + c + 1] = qr;
  }
  __syncthreads();
  riemann_pass_vjp<DIR, RS>(g.mem[g.blk[b].member], T, nl, n, W2, SL, SR, MU,
                            pass_scale<DIR>(g, b, beta, dt), GL, GR);
  __syncthreads();
  const size_t cs = (size_t)5 * T * W2;
  for (int it = tid; it < 5 * nl * W2; it += nth) {  // cells -1..n: recon vjp
    const int v = it / (nl * W2), r = it % (nl * W2), t = r / W2, c = r % W2 - 1;
    const size_t o = (size_t)(v * T + t) * W2;
    const double gL = c + 1 <= n ? GL[o + c + 1] : 0.0;  // adjoint of ql_{c+1}
    const double gR = c >= 0 ? GR[o + c] : 0.0;          // adjoint of qr_c
    double gm, g0, gp;
    if (RECON == RECON_PLM) {
      plm_vjp(q(v, t, c - 1), q(v, t, c), q(v, t, c + 1), RR[o + c + 1], gL, gR, gm, g0, gp);
    } else {
      gm = 0.0;
      g0 = gL + gR;
      gp = 0.0;
    }
    CC[0 * cs + o + c + 1] = gm;
    CC[1 * cs + o + c + 1] = g0;
    CC[2 * cs + o + c + 1] = gp;
  }
  __syncthreads();
  for (int it = tid; it < 5 * nl * (n + 4); it += nth) {  // cells -2..n+1: gather
    const int v = it / (nl * (n + 4)), r = it % (nl * (n + 4)), t = r / (n + 4), c = r % (n + 4) - 2;
    const size_t o = (size_t)(v * T + t) * W2;
    double acc = 0.0;
    if (c >= -1 && c <= n) acc += CC[1 * cs + o + c + 1];
    if (c + 1 >= -1 && c + 1 <= n) acc += CC[0 * cs + o + c + 2];
    if (c - 1 >= -1 && c - 1 <= n) acc += CC[2 * cs + o + c];
    if (c < -G || c > n + G - 1) continue;
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    LW[v * nc + base + (long long)c * s] += acc;
  }
}

// PPM pass.  Shared memory: 14 slabs of [5][T][n+6] doubles.
__host__ __device__ constexpr size_t ppm_pass_slab(int n, int T) { return (size_t)5 * T * (n + 6); }

template <int DIR, int RS>
__global__ void __launch_bounds__(256, 2) k_adj_pass_ppm(AdjGeom g, const double *prim, const double *mu,
                                                      double *lam_w, double beta, const double *dt, int T) {
  extern __shared__ double sm[];
  constexpr int G = 3;
  const int b = blockIdx.y;
  const int n = g.nx[DIR - 1];
  const int ntrans = DIR == 1 ? g.nx[1] * g.nx[2] : DIR == 2 ? g.nx[0] * g.nx[2] : g.nx[0] * g.nx[1];
  const int l0 = blockIdx.x * T;
  if (l0 >= ntrans || dt[g.blk[b].member] == 0.0) return;  // a member that did not move
  const int nl = min(T, ntrans - l0);
  const int NW = n + 6, W4 = n + 4, W3 = n + 3, W2 = n + 2;
  const size_t S = ppm_pass_slab(n, T);
  double *W = sm;             // cells -3..n+2            (later FQ0)
  double *MU = sm + 1 * S;    // interior                 (later FQ1)
  double *D2 = sm + 2 * S;    // cells -2..n+1            (later GL, then FQ2)
  double *DD = sm + 3 * S;    // cells -2..n+1            (later GR, then FQ3)
  double *DPH = sm + 4 * S;   // faces -1..n+1
  double *SL = sm + 5 * S;    // cells -1..n              (later CQ0)
  double *SR = sm + 6 * S;    //                          (later CQ1)
  double *RHO = sm + 7 * S;   // cells -1..n
  double *CQ2 = sm + 8 * S, *CQ3 = sm + 9 * S, *CQ4 = sm + 10 * S;
  double *GDL = sm + 11 * S, *GDH = sm + 12 * S;  // adjoints of each cell's two face values
  int *FB = (int *)(sm + 13 * S);                  // face branch, faces -1..n+1
  int *CB = FB + 5 * T * W3;                       // cell branch, cells -1..n
  double *GL = D2, *GR = DD;
  double *const CQ[5] = {SL, SR, CQ2, CQ3, CQ4};
  double *const FQ[4] = {W, MU, D2, DD};
  const double *P = prim + blk_off(g, b);
  const double *Mu = mu + blk_off(g, b);
  double *LW = lam_w + blk_off(g, b);
  const long long nc = g.ncell;
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int it = tid; it < 5 * nl * NW; it += nth) {
    const int v = it / (nl * NW), r = it % (nl * NW), t = r / NW, w = r % NW;
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    W[(v * T + t) * NW + w] = P[v * nc + base + (long long)(w - G) * s];
  }
  for (int it = tid; it < 5 * nl * n; it += nth) {
    const int v = it / (nl * n), r = it % (nl * n), t = r / n, c = r % n;
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    MU[(v * T + t) * n + c] = Mu[v * nc + base + (long long)c * s];
  }
  __syncthreads();
  auto q = [&](int v, int t, int c) { return W[(v * T + t) * NW + c + G]; };
  for (int it = tid; it < 5 * nl * W4; it += nth) {  // cells -2..n+1
    const int v = it / (nl * W4), r = it % (nl * W4), t = r / W4, c = r % W4 - 2;
    D2[(v * T + t) * W4 + c + 2] = ppm_d2(q(v, t, c - 1), q(v, t, c), q(v, t, c + 1));
    DD[(v * T + t) * W4 + c + 2] = ppm_dd(q(v, t, c - 1), q(v, t, c), q(v, t, c + 1));
  }
  __syncthreads();
  for (int it = tid; it < 5 * nl * W3; it += nth) {  // faces -1..n+1
    const int v = it / (nl * W3), r = it % (nl * W3), t = r / W3, f = r % W3 - 1;
    const size_t o4 = (size_t)(v * T + t) * W4;
    int code;
    DPH[(v * T + t) * W3 + f + 1] = ppm_face_code(q(v, t, f - 1), q(v, t, f), DD[o4 + f + 1], DD[o4 + f + 2],
                                                  D2[o4 + f + 1], D2[o4 + f + 2], code);
    FB[(v * T + t) * W3 + f + 1] = code;
  }
  __syncthreads();
  for (int it = tid; it < 5 * nl * W2; it += nth) {  // cells -1..n
    const int v = it / (nl * W2), r = it % (nl * W2), t = r / W2, c = r % W2 - 1;
    const size_t o4 = (size_t)(v * T + t) * W4, o3 = (size_t)(v * T + t) * W3, o2 = (size_t)(v * T + t) * W2;
    double ql, qr, rho;
    int code;
    ppm_cell_code(q(v, t, c - 2), q(v, t, c - 1), q(v, t, c), q(v, t, c + 1), q(v, t, c + 2), D2[o4 + c + 1],
                  D2[o4 + c + 2], D2[o4 + c + 3], DPH[o3 + c + 1], DPH[o3 + c + 2], ql, qr, code, rho);
    SL[o2 + c + 1] = ql;
    SR[o2 + c + 1] = qr;
    RHO[o2 + c + 1] = rho;
    CB[o2 + c + 1] = code;
  }
  __syncthreads();
  riemann_pass_vjp<DIR, RS>(g.mem[g.blk[b].member], T, nl, n, W2, SL, SR, MU,
                            pass_scale<DIR>(g, b, beta, dt), GL, GR);
  __syncthreads();
  // cells -1..n: limiter vjp (CQ0/CQ1 overwrite SL/SR, dead after the Riemann vjp)
  for (int it = tid; it < 5 * nl * W2; it += nth) {
    const int v = it / (nl * W2), r = it % (nl * W2), t = r / W2, c = r % W2 - 1;
    const size_t o2 = (size_t)(v * T + t) * W2, o3 = (size_t)(v * T + t) * W3;
    const double gL = c + 1 <= n ? GL[o2 + c + 1] : 0.0;  // adjoint of ql_{c+1}
    const double gR = c >= 0 ? GR[o2 + c] : 0.0;          // adjoint of qr_c
    double gq[5], glo, ghi;
    ppm_cell_vjp(q(v, t, c), DPH[o3 + c + 1], DPH[o3 + c + 2], CB[o2 + c + 1], RHO[o2 + c + 1], gL, gR, gq,
                 glo, ghi);
#pragma unroll
    for (int k = 0; k < 5; ++k) CQ[k][o2 + c + 1] = gq[k];
    GDL[o2 + c + 1] = glo;
    GDH[o2 + c + 1] = ghi;
  }
  __syncthreads();
  // faces -1..n+1: face-value vjp (FQ overwrite W, MU, GL, GR, all dead now)
  for (int it = tid; it < 5 * nl * W3; it += nth) {
    const int v = it / (nl * W3), r = it % (nl * W3), t = r / W3, f = r % W3 - 1;
    const size_t o2 = (size_t)(v * T + t) * W2, o3 = (size_t)(v * T + t) * W3;
    // face f is the high face of cell f-1 and the low face of cell f (cells -1..n)
    double gd = 0.0;
    if (f - 1 >= -1) gd += GDH[o2 + f];
    if (f <= n) gd += GDL[o2 + f + 1];
    double cf[4];
    ppm_face_coef(FB[o3 + f + 1], cf);
#pragma unroll
    for (int k = 0; k < 4; ++k) FQ[k][o3 + f + 1] = gd * cf[k];
  }
  __syncthreads();
  for (int it = tid; it < 5 * nl * NW; it += nth) {  // cells -3..n+2: gather
    const int v = it / (nl * NW), r = it % (nl * NW), t = r / NW, c = r % NW - 3;
    const size_t o2 = (size_t)(v * T + t) * W2, o3 = (size_t)(v * T + t) * W3;
    double acc = 0.0;
#pragma unroll
    for (int k = 0; k < 5; ++k) {  // cell c' = c - (k - 2) in -1..n: its gq[k] is for cell c
      const int cp = c - (k - 2);
      if (cp >= -1 && cp <= n) acc += CQ[k][o2 + cp + 1];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // face f = c - (k - 2) in -1..n+1: its coefficient k is for cell c
      const int f = c - (k - 2);
      if (f >= -1 && f <= n + 1) acc += FQ[k][o3 + f + 1];
    }
    long long base, s;
    adj_line<DIR>(g, l0 + t, base, s);
    LW[v * nc + base + (long long)c * s] += acc;
  }
}

// ---- ConsToPrim vjp over the entire domain ----------------------------------------------
__global__ void k_c2p_vjp(AdjGeom g, const double *w, const double *lam_w, double *lam_u) {
  const int b = blockIdx.y;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const long long o = blk_off(g, b), nc = g.ncell;
  double ww[5], gw[5], gu[5];
  bool flows = false;
  for (int v = 0; v < 5; ++v) {
    ww[v] = w[o + v * nc + c];
    gw[v] = lam_w[o + v * nc + c];
    flows |= (__double_as_longlong(gw[v]) << 1) != 0;
  }
  // the map is linear in gw: a cell no pass reads (whose primitives the forward may not have
  // formed, e.g. a ghost corner of a finished member's block) gets exactly zero
  if (!flows) {
    for (int v = 0; v < 5; ++v) lam_u[o + v * nc + c] = 0.0;
    return;
  }
  cons_to_prim_vjp(ww, gw, g.mem[g.blk[b].member].gc.gm1, gu);
  for (int v = 0; v < 5; ++v) lam_u[o + v * nc + c] = gu[v];
}

// ---- ghost map transposed: each interior cell gathers the ghost copies made of it, giving
// r = R'(u)^T mu; fused with the stage combination  acc += gam1 a;  a = gam0 a + r  (acc
// starts at zero when acc_zero), and at the first stage with  lam_n = a + acc  (when lam_n is
// given, a and acc are not stored).
__global__ void k_ghost_vjp(AdjGeom g, const double *lam_u, double *a, double *acc_buf,
                            double gam0, double gam1, int acc_zero, double *lam_n) {
  const int b = blockIdx.y;
  const int nint = g.nx[0] * g.nx[1] * g.nx[2];
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nint) return;
  const int ii[3] = {idx % g.nx[0], (idx / g.nx[0]) % g.nx[1], idx / (g.nx[0] * g.nx[1])};
  const AdjBlock &B = g.blk[b];
  const long long nc = g.ncell;
  auto cell_of = [&](const int *e) {  // entire-domain index from per-dim entire indices
    return ((long long)e[2] * g.nj + e[1]) * g.ni + e[0];
  };
  int e[3];
  for (int d = 0; d < 3; ++d) e[d] = ii[d] + dstart(g, d);
  const long long self = cell_of(e);
  double acc[5];
  for (int v = 0; v < 5; ++v) acc[v] = lam_u[blk_off(g, b) + v * nc + self];
  for (int d = 0; d < g.ndim; ++d) {
    for (int side = 0; side < 2; ++side) {
      const int dist = side == 0 ? ii[d] : g.nx[d] - 1 - ii[d];  // distance from that face
      if (dist >= g.ng) continue;
      // the block across that face (if any) holds a ghost copy of this cell at depth dist
      int nbk = -1, bc = APH_BC_PERIODIC;
      if (g.faces) {
        const int face = 2 * d + side;
        if (B.faces.kind[face] == FACE_SAME) nbk = B.faces.nbr[face][0];
        else bc = g.bc[d][side];
      } else {
        const bool edge = side == 0 ? B.loc[d] == 0 : B.loc[d] == g.nb[d] - 1;
        bc = g.bc[d][side];
        if (!edge || bc == APH_BC_PERIODIC) {
          int nl[3] = {B.loc[0], B.loc[1], B.loc[2]};
          nl[d] += side == 0 ? -1 : 1;
          if (nl[d] < 0) nl[d] += g.nb[d];
          if (nl[d] >= g.nb[d]) nl[d] -= g.nb[d];
          nbk = (nl[2] * g.nb[1] + nl[1]) * g.nb[0] + nl[0];
        }
      }
      if (nbk >= 0) {
        int ge[3] = {e[0], e[1], e[2]};
        ge[d] = side == 0 ? g.ng + g.nx[d] + dist : g.ng - 1 - dist;
        const long long gc = cell_of(ge);
        for (int v = 0; v < 5; ++v) acc[v] += lam_u[blk_off(g, nbk) + v * nc + gc];
      } else if (bc == APH_BC_REFLECT) {
        int ge[3] = {e[0], e[1], e[2]};
        ge[d] = side == 0 ? g.ng - 1 - dist : g.ng + g.nx[d] + dist;
        const long long gc = cell_of(ge);
        for (int v = 0; v < 5; ++v) {
          const double x = lam_u[blk_off(g, b) + v * nc + gc];
          acc[v] += (v == 1 + d) ? -x : x;
        }
      } else if (dist == 0) {  // outflow: every ghost beyond the face copies the edge cell
        for (int k = 0; k < g.ng; ++k) {
          int ge[3] = {e[0], e[1], e[2]};
          ge[d] = side == 0 ? g.ng - 1 - k : g.ng + g.nx[d] + k;
          const long long gc = cell_of(ge);
          for (int v = 0; v < 5; ++v) acc[v] += lam_u[blk_off(g, b) + v * nc + gc];
        }
      }
    }
  }
  for (int v = 0; v < 5; ++v) {
    const long long o = blk_off(g, b) + v * nc + self;
    const double av = a[o];
    const double cv = (acc_zero ? 0.0 : acc_buf[o]) + gam1 * av;
    const double an = gam0 * av + acc[v];
    if (lam_n) {
      lam_n[o] = an + cv;
    } else {
      acc_buf[o] = cv;
      a[o] = an;
    }
  }
}

// out = x on interior cells, zero on ghost cells
__global__ void k_copy_interior(AdjGeom g, const double *x, double *out) {
  const int b = blockIdx.y;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const int i = (int)(c % g.ni), j = (int)((c / g.ni) % g.nj), k = (int)(c / ((long long)g.ni * g.nj));
  bool in = i >= g.ng && i < g.ng + g.nx[0];
  if (g.ndim >= 2) in = in && j >= g.ng && j < g.ng + g.nx[1];
  if (g.ndim >= 3) in = in && k >= g.ng && k < g.ng + g.nx[2];
  for (int v = 0; v < 5; ++v) {
    const long long o = blk_off(g, b) + v * g.ncell + c;
    out[o] = in ? x[o] : 0.0;
  }
}

struct StageC {
  double gam0, gam1, beta;
};
std::vector<StageC> stages_for(int integrator) {
  switch (integrator) {
    case APH_INTEGRATOR_RK1: return {{0.0, 1.0, 1.0}};
    case APH_INTEGRATOR_RK2: return {{0.0, 1.0, 1.0}, {0.5, 0.5, 0.5}};
    case APH_INTEGRATOR_RK3:
      return {{0.0, 1.0, 1.0}, {0.25, 0.75, 0.25}, {2.0 / 3.0, 1.0 / 3.0, 2.0 / 3.0}};
    case APH_INTEGRATOR_VL2: return {{0.0, 1.0, 0.5}, {0.0, 1.0, 1.0}};
    default: return {};
  }
}

}  // namespace

struct aph_adjoint_s {
  AdjGeom g;
  aph_hydro_params params;
  int integrator = 0;
  int nmembers = 1;
  size_t n = 0;  // doubles per pack field
  double *x = nullptr;  // the forward stepper's state (pack layout)
  double *lam_w = nullptr, *lam_u = nullptr, *a = nullptr, *acc = nullptr;
  double *states = nullptr;  // stage-input primitives of the step being differentiated
  AdjBlock *d_blk = nullptr;
  AdjMember *d_mem = nullptr;
  int *floor_flag = nullptr;
  aph_stepper st = nullptr;  // the forward
  std::vector<aph_block> blocks;
  // rollout
  int nsteps = 0;
  double *d_dts = nullptr;   // [nsteps][nmembers], then one scratch row
  size_t d_dts_len = 0;
  int ckpt_every = 0;
  double *ckpts = nullptr;
  int nckpt = 0;
  // the reverse sweep's segment storage (stage-input primitives of every step of one
  // checkpoint segment), sized by the rollout that recorded the checkpoints
  double *seg = nullptr;
  size_t seg_len = 0;
};

namespace {

aph_status ensure_dts(aph_adjoint A, size_t len) {
  if (len <= A->d_dts_len) return APH_OK;
  cudaFree(A->d_dts);
  A->d_dts = nullptr;
  A->d_dts_len = 0;
  cudaError_t e = cudaMalloc(&A->d_dts, len * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "adjoint dt table");
  A->d_dts_len = len;
  return APH_OK;
}

// One step of A->x with the per-member dt dt_dev (device); keep: stage-input primitives.
aph_status fwd_step(aph_adjoint A, const double *dt_dev, double *keep, cudaStream_t s) {
  cudaError_t e = stepper_step_dt(A->st, dt_dev, keep, A->floor_flag, s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "adjoint forward");
}

template <int DIR>
cudaError_t launch_pass(aph_adjoint A, int recon, double beta, const double *dt_dev,
                        const double *prim, cudaStream_t s) {
  const AdjGeom &g = A->g;
  const int n = g.nx[DIR - 1];
  int T;
  size_t smem;
  const void *k = nullptr;
  const bool hlle = A->params.rsolver == APH_RSOLVER_HLLE;
  if (recon == APH_RECON_PPM) {
    const size_t per_line = 14 * ppm_pass_slab(n, 1) * sizeof(double);
    T = std::max(1, std::min(256 / (n + 6), (int)((96 * 1024) / per_line)));
    smem = 14 * ppm_pass_slab(n, T) * sizeof(double);
    k = hlle ? (const void *)k_adj_pass_ppm<DIR, RS_HLLE> : (const void *)k_adj_pass_ppm<DIR, RS_HLLC>;
  } else {
    T = std::max(1, 256 / (n + 2));
    const int G = recon == APH_RECON_PLM ? 2 : 1;
    smem = sizeof(double) * (5 * T * (n + 2 * G) + 5 * T * n + 4 * 5 * T * (n + 2) +
                             3 * 5 * T * (n + 2) + 5 * T * (n + 2));
    if (recon == APH_RECON_PLM)
      k = hlle ? (const void *)k_adj_pass<DIR, RECON_PLM, RS_HLLE> : (const void *)k_adj_pass<DIR, RECON_PLM, RS_HLLC>;
    else
      k = hlle ? (const void *)k_adj_pass<DIR, RECON_DC, RS_HLLE> : (const void *)k_adj_pass<DIR, RECON_DC, RS_HLLC>;
  }
  if (smem > 200 * 1024) return cudaErrorInvalidValue;
  const int ntrans = DIR == 1 ? g.nx[1] * g.nx[2] : DIR == 2 ? g.nx[0] * g.nx[2] : g.nx[0] * g.nx[1];
  dim3 grid((ntrans + T - 1) / T, g.nblocks);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  AdjGeom gg = g;
  const double *mu = A->a;
  double *lw = A->lam_w;
  int TT = T;
  void *args[] = {&gg, &prim, &mu, &lw, &beta, &dt_dev, &TT};
  return cudaLaunchKernel(k, grid, dim3(256), args, smem, s);
}

// R'(u)^T (beta dt a) for the stage input whose primitives (entire domain, ghosts included)
// are prim, combined into a / acc (k_ghost_vjp).
cudaError_t stage_vjp(aph_adjoint A, int recon, double beta, const double *dt_dev, const double *prim,
                      double gam0, double gam1, bool acc_zero, double *lam_n, cudaStream_t s) {
  const AdjGeom &g = A->g;
  const unsigned gx = (unsigned)((g.ncell + 255) / 256);
  cudaError_t e = cudaMemsetAsync(A->lam_w, 0, A->n * sizeof(double), s);
  for (int d = 1; d <= g.ndim && e == cudaSuccess; ++d)
    e = d == 1 ? launch_pass<1>(A, recon, beta, dt_dev, prim, s)
               : d == 2 ? launch_pass<2>(A, recon, beta, dt_dev, prim, s)
                        : launch_pass<3>(A, recon, beta, dt_dev, prim, s);
  if (e == cudaSuccess) {
    k_c2p_vjp<<<dim3(gx, g.nblocks), 256, 0, s>>>(g, prim, A->lam_w, A->lam_u);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    const int nint = g.nx[0] * g.nx[1] * g.nx[2];
    k_ghost_vjp<<<dim3((nint + 255) / 256, g.nblocks), 256, 0, s>>>(g, A->lam_u, A->a, A->acc, gam0,
                                                                   gam1, acc_zero ? 1 : 0, lam_n);
    e = cudaGetLastError();
  }
  return e;
}

// lam_n = (d U^{n+1} / d U^n)^T lam_next for the step with per-member dt dt_dev whose
// stage-input primitives (one pack field per stage) are `kept`.  lam_n may alias lam_next.
aph_status step_vjp_kept(aph_adjoint A, const double *kept, const double *dt_dev,
                         const double *lam_next, double *lam_n, cudaStream_t s) {
  const std::vector<StageC> st = stages_for(A->integrator);
  const AdjGeom &g = A->g;
  const unsigned gx = (unsigned)((g.ncell + 255) / 256);
  k_copy_interior<<<dim3(gx, g.nblocks), 256, 0, s>>>(g, lam_next, A->a);
  cudaError_t e = cudaGetLastError();
  const int ns = (int)st.size();
  for (int i = ns - 1; i >= 0 && e == cudaSuccess; --i) {
    const int recon = (A->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : A->params.recon;
    e = stage_vjp(A, recon, st[i].beta, dt_dev, kept + (size_t)i * A->n, st[i].gam0, st[i].gam1,
                  i == ns - 1, i == 0 ? lam_n : nullptr, s);
  }
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "adjoint step");
}

void adj_free(aph_adjoint A) {
  if (A->st) aph_stepper_destroy(A->st);
  A->st = nullptr;
  double *bufs[] = {A->x, A->lam_w, A->lam_u, A->a, A->acc, A->states, A->ckpts, A->d_dts, A->seg};
  for (double *p : bufs) cudaFree(p);
  cudaFree(A->d_blk);
  cudaFree(A->d_mem);
  cudaFree(A->floor_flag);
}

aph_status check_state(aph_adjoint A, cudaStream_t s) {
  int f = 0;
  cudaError_t e = cudaMemcpyAsync(&f, A->floor_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint");
  if (aph_status st = aph_stepper_status(A->st, nullptr, nullptr, nullptr, s)) return st;
  if (f) return fail(APH_ERR_STATE, "a density or pressure floor fired: the step is not differentiable there");
  return APH_OK;
}

// the same dt for every member, in the scratch row after the rollout table
aph_status scalar_dt(aph_adjoint A, double dt, const double **dt_dev, cudaStream_t s) {
  const size_t row = (size_t)A->nsteps * A->nmembers;
  if (aph_status st = ensure_dts(A, row + A->nmembers)) return st;
  std::vector<double> v(A->nmembers, dt);
  cudaError_t e = cudaMemcpyAsync(A->d_dts + row, v.data(), v.size() * sizeof(double),
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // v is a host temporary
  if (e != cudaSuccess) return cuda_fail(e, "adjoint dt");
  *dt_dev = A->d_dts + row;
  return APH_OK;
}

}  // namespace

extern "C" {

aph_status aph_adjoint_create(const aph_stepper_desc *desc, aph_adjoint *out) {
  clear_error();
  if (!desc || !out) return fail(APH_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (aph_status st = validate_params(&desc->params)) return st;
  const aph_hydro_params &q = desc->params;
  if (q.nvar != 5) return fail(APH_ERR_UNSUPPORTED, "the adjoint carries no passive scalars");
  if (q.rsolver != APH_RSOLVER_HLLE && q.rsolver != APH_RSOLVER_HLLC)
    return fail(APH_ERR_UNSUPPORTED, "the adjoint differentiates the hlle and hllc solvers");
  if (q.exact) return fail(APH_ERR_UNSUPPORTED, "the adjoint runs on the fast arithmetic");
  if (desc->use_gravity) return fail(APH_ERR_UNSUPPORTED, "the adjoint has no gravity source");
  if (stages_for(desc->integrator).empty()) return fail(APH_ERR_INVALID, "integrator not recognized");
  if (desc->nblocks <= 0 || !desc->blocks) return fail(APH_ERR_INVALID, "no blocks");
  for (int b = 0; b < desc->nblocks; ++b)
    for (int d = 0; d < 3; ++d)
      if (desc->blocks[b].nx[d] != desc->blocks[0].nx[d])
        return fail(APH_ERR_UNSUPPORTED, "the adjoint's pack layout needs blocks of equal size");
  if (desc->amr)
    for (int b = 0; b < desc->nblocks; ++b)
      for (int f = 0; f < 4; ++f) {
        const int k = desc->amr[b].face_kind[f];
        if (k == APH_FACE_COARSER || k == APH_FACE_FINER)
          return fail(APH_ERR_UNSUPPORTED, "the adjoint has no coarse-fine faces");
        // the transposed gather relies on reciprocal same-level neighbours
        if (k == APH_FACE_SAME) {
          const int nb = desc->amr[b].face_nbr[f][0];
          if (nb < 0 || nb >= desc->nblocks || desc->amr[nb].face_kind[f ^ 1] != APH_FACE_SAME ||
              desc->amr[nb].face_nbr[f ^ 1][0] != b)
            return fail(APH_ERR_INVALID, "block %d face %d: same-level neighbours must be reciprocal", b, f);
        }
      }
  const int nmembers = desc->ensemble ? desc->ensemble->nmembers : 1;
  if (nmembers < 1 || (desc->ensemble && (!desc->ensemble->member || !desc->ensemble->gm1)))
    return fail(APH_ERR_INVALID, "ensemble: nmembers, member and gm1 are required");
  aph_adjoint A = new aph_adjoint_s();
  A->params = q;
  A->integrator = desc->integrator;
  A->nmembers = nmembers;
  AdjGeom &g = A->g;
  std::memset(&g, 0, sizeof(g));
  g.nblocks = desc->nblocks;
  g.ndim = q.ndim;
  g.ng = q.nghost;
  for (int d = 0; d < 3; ++d) {
    g.nx[d] = desc->blocks[0].nx[d];
    g.nb[d] = desc->nb[d];
    g.bc[d][0] = desc->bc[2 * d];
    g.bc[d][1] = desc->bc[2 * d + 1];
  }
  g.faces = desc->amr ? 1 : 0;
  g.ni = g.nx[0] + 2 * g.ng;
  g.nj = g.ndim >= 2 ? g.nx[1] + 2 * g.ng : 1;
  g.nk = g.ndim >= 3 ? g.nx[2] + 2 * g.ng : 1;
  g.ncell = (long long)g.ni * g.nj * g.nk;
  A->n = (size_t)g.nblocks * 5 * g.ncell;
  const size_t bytes = A->n * sizeof(double);
  const int ns = (int)stages_for(A->integrator).size();
  // per-block and per-member descriptors
  std::vector<AdjBlock> hb(g.nblocks);
  for (int b = 0; b < g.nblocks; ++b) {
    AdjBlock &B = hb[b];
    std::memset(&B, 0, sizeof(B));
    for (int d = 0; d < 3; ++d) B.dx[d] = desc->blocks[b].dx[d];
    B.member = desc->ensemble ? desc->ensemble->member[b] : 0;
    if (B.member < 0 || B.member >= nmembers) {
      delete A;
      return fail(APH_ERR_INVALID, "block %d: member out of range", b);
    }
    if (desc->amr) {
      std::memcpy(&B.faces, &desc->amr[b], sizeof(AmrFaces));
    } else {
      const int n0 = std::max(1, g.nb[0]), n1 = std::max(1, g.nb[1]);
      B.loc[0] = b % n0;
      B.loc[1] = (b / n0) % n1;
      B.loc[2] = b / (n0 * n1);
    }
  }
  std::vector<AdjMember> hm(nmembers);
  for (int m = 0; m < nmembers; ++m) {
    PackDev tmp;
    std::memset(&tmp, 0, sizeof(tmp));
    tmp.gm1 = desc->ensemble ? desc->ensemble->gm1[m] : q.gm1;
    if (!(tmp.gm1 > 0.0)) {
      delete A;
      return fail(APH_ERR_INVALID, "member %d: gm1 must be > 0", m);
    }
    fill_gas_consts(tmp);
    hm[m].gc = GasConsts{tmp.gm1, tmp.igm1, tmp.gamma, tmp.c2g, tmp.one_igm1, tmp.hlle_k, tmp.hllc_k};
    hm[m].ic2g = 1.0 / tmp.c2g;
  }
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  double **bufs[] = {&A->x, &A->lam_w, &A->lam_u, &A->a, &A->acc};
  for (double **b : bufs) ck(cudaMalloc(b, bytes));
  ck(cudaMalloc(&A->states, bytes * ns));
  ck(cudaMalloc(&A->floor_flag, sizeof(int)));
  ck(cudaMalloc(&A->d_blk, sizeof(AdjBlock) * hb.size()));
  ck(cudaMalloc(&A->d_mem, sizeof(AdjMember) * hm.size()));
  if (e == cudaSuccess) e = cudaMemcpy(A->d_blk, hb.data(), sizeof(AdjBlock) * hb.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(A->d_mem, hm.data(), sizeof(AdjMember) * hm.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(A->floor_flag, 0, sizeof(int));
  if (e != cudaSuccess) {
    adj_free(A);
    delete A;
    return cuda_fail(e, "adjoint allocation");
  }
  g.blk = A->d_blk;
  g.mem = A->d_mem;
  // the forward: a stepper over the adjoint's state (a uniform placeholder state, rho = E = 1,
  // for its initial dt estimate)
  A->blocks.assign(desc->blocks, desc->blocks + desc->nblocks);
  for (int b = 0; b < g.nblocks; ++b) A->blocks[b].cons = A->x + (size_t)b * 5 * g.ncell;
  {
    std::vector<double> one(5 * g.ncell, 0.0);
    for (long long c = 0; c < g.ncell; ++c) {
      one[c] = 1.0;
      one[4 * g.ncell + c] = 1.0;
    }
    for (int b = 0; b < g.nblocks && e == cudaSuccess; ++b)
      e = cudaMemcpy(A->blocks[b].cons, one.data(), one.size() * sizeof(double), cudaMemcpyHostToDevice);
  }
  aph_stepper_desc sd = *desc;
  sd.blocks = A->blocks.data();
  sd.fixed_dt = 0.0;  // each forward step sets its dt (stepper_step_dt); the policy only tunes
  sd.tlim = 0.0;
  aph_status st = e == cudaSuccess ? aph_stepper_create(&sd, &A->st) : cuda_fail(e, "adjoint setup");
  if (st) {
    adj_free(A);
    delete A;
    return st;
  }
  *out = A;
  return APH_OK;
}

aph_status aph_adjoint_destroy(aph_adjoint A) {
  if (!A) return APH_OK;
  adj_free(A);
  delete A;
  return APH_OK;
}

aph_status aph_adjoint_step(aph_adjoint A, const double *u_n, double dt, double *u_next, void *stream) {
  clear_error();
  if (!A || !u_n || !u_next) return fail(APH_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  const double *dt_dev = nullptr;
  if (aph_status st = scalar_dt(A, dt, &dt_dev, s)) return st;
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  cudaError_t e = cudaMemcpyAsync(A->x, u_n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint forward");
  if (aph_status st = fwd_step(A, dt_dev, nullptr, s)) return st;
  e = cudaMemcpyAsync(u_next, A->x, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint forward");
  return check_state(A, s);
}

aph_status aph_adjoint_step_vjp(aph_adjoint A, const double *u_n, double dt, const double *lam_next,
                                double *lam_n, void *stream) {
  clear_error();
  if (!A || !u_n || !lam_next || !lam_n) return fail(APH_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  const double *dt_dev = nullptr;
  if (aph_status st = scalar_dt(A, dt, &dt_dev, s)) return st;
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  cudaError_t e = cudaMemcpyAsync(A->x, u_n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint step");
  if (aph_status st = fwd_step(A, dt_dev, A->states, s)) return st;
  if (aph_status st = step_vjp_kept(A, A->states, dt_dev, lam_next, lam_n, s)) return st;
  return check_state(A, s);
}

aph_status aph_adjoint_forward_members(aph_adjoint A, const double *u0, int nsteps, const double *dts,
                                       int checkpoint_every, double *u_final, void *stream) {
  clear_error();
  if (!A || !u0 || !dts || nsteps < 1 || !u_final) return fail(APH_ERR_INVALID, "bad argument");
  if (checkpoint_every < 1) checkpoint_every = nsteps;
  cudaStream_t s = (cudaStream_t)stream;
  const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every;
  if (nck != A->nckpt) {
    cudaFree(A->ckpts);
    A->ckpts = nullptr;
    A->nckpt = 0;
    cudaError_t e = cudaMalloc(&A->ckpts, (size_t)nck * A->n * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "checkpoint allocation");
    A->nckpt = nck;
  }
  const size_t nm = A->nmembers;
  A->nsteps = 0;
  if (aph_status st = ensure_dts(A, (size_t)nsteps * nm + nm)) return st;
  {  // the backward sweep's segment storage, allocated here once per rollout shape
    const size_t need = (size_t)std::min(checkpoint_every, nsteps) * stages_for(A->integrator).size() * A->n;
    if (need > A->seg_len) {
      cudaFree(A->seg);
      A->seg = nullptr;
      A->seg_len = 0;
      cudaError_t e = cudaMalloc(&A->seg, need * sizeof(double));
      if (e != cudaSuccess) return cuda_fail(e, "segment allocation");
      A->seg_len = need;
    }
  }
  cudaError_t e = cudaMemcpyAsync(A->d_dts, dts, (size_t)nsteps * nm * sizeof(double), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // dts is the caller's host array
  if (e != cudaSuccess) return cuda_fail(e, "adjoint dt table");
  A->nsteps = nsteps;
  A->ckpt_every = checkpoint_every;
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  e = cudaMemcpyAsync(A->x, u0, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) {
    if (k % checkpoint_every == 0)
      e = cudaMemcpyAsync(A->ckpts + (size_t)(k / checkpoint_every) * A->n, A->x, A->n * sizeof(double),
                          cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) break;
    if (aph_status st = fwd_step(A, A->d_dts + (size_t)k * nm, nullptr, s)) return st;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(u_final, A->x, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint rollout");
  return check_state(A, s);
}

aph_status aph_adjoint_forward(aph_adjoint A, const double *u0, int nsteps, const double *dts,
                               int checkpoint_every, double *u_final, void *stream) {
  clear_error();
  if (!A || !dts || nsteps < 1) return fail(APH_ERR_INVALID, "bad argument");
  std::vector<double> table((size_t)nsteps * A->nmembers);
  for (int k = 0; k < nsteps; ++k)
    for (int m = 0; m < A->nmembers; ++m) table[(size_t)k * A->nmembers + m] = dts[k];
  return aph_adjoint_forward_members(A, u0, nsteps, table.data(), checkpoint_every, u_final, stream);
}

aph_status aph_adjoint_autotune(aph_adjoint A, const double *u, void *stream) {
  clear_error();
  if (!A || !u) return fail(APH_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  // the forward stepper's launch configuration, timed on the state u (restored afterwards)
  // (the trial steps take the CFL dt of u: the stepper's clock restarts from u)
  cudaError_t e = cudaMemcpyAsync(A->x, u, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = stepper_restart(A->st, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint autotune");
  return aph_stepper_autotune(A->st, 1, nullptr, nullptr);
}

aph_status aph_adjoint_backward(aph_adjoint A, const double *lam_final, double *lam_initial,
                                void *stream) {
  clear_error();
  if (!A || !lam_final || !lam_initial) return fail(APH_ERR_INVALID, "NULL argument");
  if (A->nsteps < 1 || !A->ckpts) return fail(APH_ERR_INVALID, "no recorded rollout");
  cudaStream_t s = (cudaStream_t)stream;
  const int nsteps = A->nsteps, K = A->ckpt_every;
  const size_t nm = A->nmembers;
  const int ns = (int)stages_for(A->integrator).size();
  // segment storage (allocated by the rollout): the stage-input primitives of every step of
  // one segment, recomputed once from the segment's checkpoint
  double *seg = A->seg;
  const size_t per_step = (size_t)ns * A->n;
  if (!seg || (size_t)std::min(K, nsteps) * per_step > A->seg_len)
    return fail(APH_ERR_INVALID, "no segment storage for the recorded rollout");
  cudaError_t e =
      cudaMemcpyAsync(lam_initial, lam_final, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  aph_status st = APH_OK;
  for (int j = A->nckpt - 1; j >= 0 && st == APH_OK && e == cudaSuccess; --j) {
    const int k0 = j * K, k1 = std::min(nsteps, k0 + K);
    e = cudaMemcpyAsync(A->x, A->ckpts + (size_t)j * A->n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    for (int k = k0; k < k1 && st == APH_OK && e == cudaSuccess; ++k)
      st = fwd_step(A, A->d_dts + (size_t)k * nm, seg + (size_t)(k - k0) * per_step, s);
    for (int k = k1 - 1; k >= k0 && st == APH_OK && e == cudaSuccess; --k)
      st = step_vjp_kept(A, seg + (size_t)(k - k0) * per_step, A->d_dts + (size_t)k * nm, lam_initial,
                         lam_initial, s);
  }
  if (e == cudaSuccess && st == APH_OK) e = cudaStreamSynchronize(s);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(e, "adjoint backward");
  return check_state(A, s);
}

}  // extern "C"
