// aph_adjoint.cu -- hand-written adjoint of the full hydro step, exposed through the C ABI.
//
// For a step U^n -> U^{n+1} with stages u_{s+1} = gam0_s u_s + gam1_s U^n + beta_s dt R(u_s),
// R(u) = -div F(recon(ConsToPrim(ghosts(u)))), the vector-Jacobian product runs the stages
// backwards:
//     a_{S+1} = lambda^{n+1};   for s = S..1:  acc += gam1_s a_{s+1},
//     a_s = gam0_s a_{s+1} + R'(u_s)^T (beta_s dt a_{s+1});      lambda^n = a_1 + acc.
// R'(u)^T mu is one pass per direction (recompute the face states, HLLE/HLLC vjp, PLM/DC
// vjp, gathered per cell without atomics), then the ConsToPrim vjp per cell, then the ghost
// map transposed (each interior cell gathers the ghost copies made of it).  The forward
// used for the tape and the recomputation is the per-pack fast path.  Rollouts store a
// checkpoint every K steps and recompute each segment during the backward sweep, so the
// memory is (N/K + K) states.  Floors are taken as inactive (the derivative of a floored
// cell is undefined); a forward that fires a floor is reported as APH_ERR_STATE.
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/aph_hydro.h"
#include "aph_adjoint_math.cuh"
#include "aph_capi_internal.h"

using namespace aph;

namespace {

struct AdjGeom {
  int nblocks, ndim, ng;
  int nx[3], ni, nj, nk;
  long long ncell;       // per block, entire
  int nb[3];
  int bc[3][2];
  double dx[3];
  GasConsts gc;
  double ic2g;  // 1 / (C^2 gamma)
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

template <int DIR, int RECON, int RS>
__global__ void __launch_bounds__(256) k_adj_pass(AdjGeom g, const double *prim, const double *mu,
                                                  double *lam_w, double scale, int T) {
  extern __shared__ double sm[];
  constexpr int G = RECON == RECON_PLM ? 2 : 1;
  const int b = blockIdx.y;
  const int n = g.nx[DIR - 1];
  const int ntrans = DIR == 1 ? g.nx[1] * g.nx[2] : DIR == 2 ? g.nx[0] * g.nx[2] : g.nx[0] * g.nx[1];
  const int l0 = blockIdx.x * T;
  if (l0 >= ntrans) return;
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
  const double *M = mu + blk_off(g, b);
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
    MU[(v * T + t) * n + c] = M[v * nc + base + (long long)c * s];
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
  constexpr int ivx = DIR;
  constexpr int ivy = IV1 + ((ivx - IV1) + 1) % 3;
  constexpr int ivz = IV1 + ((ivx - IV1) + 2) % 3;
  const int perm[5] = {IDN, ivx, ivy, ivz, IEN};
  for (int it = tid; it < nl * (n + 1); it += nth) {  // faces 0..n
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
    if (RS == RS_HLLE) hlle_vjp(wl, wr, g.gc, g.ic2g, gf, gwl, gwr);
    else hllc_vjp(wl, wr, g.gc, g.ic2g, gf, gwl, gwr);
    for (int k = 0; k < 5; ++k) {
      GL[(perm[k] * T + t) * W2 + f] = gwl[k];
      GR[(perm[k] * T + t) * W2 + f] = gwr[k];
    }
  }
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

// ---- ConsToPrim vjp over the entire domain ----------------------------------------------
__global__ void k_c2p_vjp(AdjGeom g, const double *w, const double *lam_w, double *lam_u) {
  const int b = blockIdx.y;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const long long o = blk_off(g, b), nc = g.ncell;
  double ww[5], gw[5], gu[5];
  for (int v = 0; v < 5; ++v) {
    ww[v] = w[o + v * nc + c];
    gw[v] = lam_w[o + v * nc + c];
  }
  cons_to_prim_vjp(ww, gw, g.gc.gm1, gu);
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
  const int loc[3] = {b % g.nb[0], (b / g.nb[0]) % g.nb[1], b / (g.nb[0] * g.nb[1])};
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
      const bool edge = side == 0 ? loc[d] == 0 : loc[d] == g.nb[d] - 1;
      const int bc = g.bc[d][side];
      if (!edge || bc == APH_BC_PERIODIC) {
        // the neighbour across that face holds a ghost copy at depth dist
        int nl[3] = {loc[0], loc[1], loc[2]};
        nl[d] += side == 0 ? -1 : 1;
        if (nl[d] < 0) nl[d] += g.nb[d];
        if (nl[d] >= g.nb[d]) nl[d] -= g.nb[d];
        const int nbk = (nl[2] * g.nb[1] + nl[1]) * g.nb[0] + nl[0];
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

// out = alpha * x + beta * y on interior cells (ghost entries of out set to zero)
__global__ void k_axpby(AdjGeom g, double alpha, const double *x, double beta, const double *y,
                        double *out) {
  const int b = blockIdx.y;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.ncell) return;
  const int i = (int)(c % g.ni), j = (int)((c / g.ni) % g.nj), k = (int)(c / ((long long)g.ni * g.nj));
  bool in = i >= g.ng && i < g.ng + g.nx[0];
  if (g.ndim >= 2) in = in && j >= g.ng && j < g.ng + g.nx[1];
  if (g.ndim >= 3) in = in && k >= g.ng && k < g.ng + g.nx[2];
  for (int v = 0; v < 5; ++v) {
    const long long o = blk_off(g, b) + v * g.ncell + c;
    out[o] = in ? alpha * x[o] + (y ? beta * y[o] : 0.0) : 0.0;
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
  size_t n = 0;  // doubles per pack field
  double *x = nullptr, *u1 = nullptr, *prim = nullptr, *gamma = nullptr, *flux[3] = {nullptr, nullptr, nullptr};
  double *lam_w = nullptr, *lam_u = nullptr, *a = nullptr, *acc = nullptr;
  double *states = nullptr;  // per stage input of the step being differentiated
  int *floor_flag = nullptr;
  aph_pack pack = nullptr;
  // rollout
  std::vector<double> dts;
  int ckpt_every = 0;
  double *ckpts = nullptr;
  int nckpt = 0;
};

namespace {

cudaError_t fwd_prepare(aph_adjoint A, cudaStream_t s) {
  // ghosts + FillDerived of A->x
  if (aph_hydro_fill_ghosts(A->pack, s) != APH_OK) return cudaErrorUnknown;
  const PackDev &p = pack_dev(A->pack);
  return aph_fast::launch_cons_to_prim(p, pack_blocks(A->pack), pack_max_ncell(A->pack),
                                       A->floor_flag, s);
}

// One fixed-dt RK step of A->x (interior in, interior + ghosts + prim out).  With keep
// non-null the primitives of every stage input (entire domain) are saved there, one pack
// field per stage.
aph_status fwd_step(aph_adjoint A, double dt, double *keep, cudaStream_t s) {
  const std::vector<StageC> st = stages_for(A->integrator);
  cudaError_t e = fwd_prepare(A, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(A->u1, A->x, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  for (size_t i = 0; i < st.size() && e == cudaSuccess; ++i) {
    if (keep)
      e = cudaMemcpyAsync(keep + i * A->n, A->prim, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) break;
    const int recon = (A->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : A->params.recon;
    if (aph_hydro_calculate_fluxes(A->pack, recon, A->params.rsolver, s) != APH_OK) return APH_ERR_CUDA;
    if (aph_hydro_update_with_flux_divergence(A->pack, st[i].gam0, st[i].gam1, st[i].beta * dt, s) != APH_OK)
      return APH_ERR_CUDA;
    e = fwd_prepare(A, s);
  }
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "adjoint forward");
}

template <int DIR>
cudaError_t launch_pass(aph_adjoint A, int recon, double scale, const double *prim_in,
                        cudaStream_t s) {
  const AdjGeom &g = A->g;
  const int n = g.nx[DIR - 1];
  const int T = std::max(1, 256 / (n + 2));
  const int G = recon == APH_RECON_PLM ? 2 : 1;
  const size_t smem = sizeof(double) * (5 * T * (n + 2 * G) + 5 * T * n + 4 * 5 * T * (n + 2) +
                                        3 * 5 * T * (n + 2) + 5 * T * (n + 2));
  const int ntrans = DIR == 1 ? g.nx[1] * g.nx[2] : DIR == 2 ? g.nx[0] * g.nx[2] : g.nx[0] * g.nx[1];
  dim3 grid((ntrans + T - 1) / T, g.nblocks);
  const void *k = nullptr;
  if (recon == APH_RECON_PLM)
    k = A->params.rsolver == APH_RSOLVER_HLLE ? (const void *)k_adj_pass<DIR, RECON_PLM, RS_HLLE>
                                              : (const void *)k_adj_pass<DIR, RECON_PLM, RS_HLLC>;
  else
    k = A->params.rsolver == APH_RSOLVER_HLLE ? (const void *)k_adj_pass<DIR, RECON_DC, RS_HLLE>
                                              : (const void *)k_adj_pass<DIR, RECON_DC, RS_HLLC>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  AdjGeom gg = g;
  const double *prim = prim_in;
  const double *mu = A->a;
  double *lw = A->lam_w;
  int TT = T;
  void *args[] = {&gg, &prim, &mu, &lw, &scale, &TT};
  return cudaLaunchKernel(k, grid, dim3(256), args, smem, s);
}

// R'(u)^T (beta dt a) for the stage input whose primitives (entire domain, ghosts included)
// are prim, combined into a / acc (k_ghost_vjp).
cudaError_t stage_vjp(aph_adjoint A, int recon, double bdt, const double *prim, double gam0,
                      double gam1, bool acc_zero, double *lam_n, cudaStream_t s) {
  const AdjGeom &g = A->g;
  const unsigned gx = (unsigned)((g.ncell + 255) / 256);
  cudaError_t e = cudaMemsetAsync(A->lam_w, 0, A->n * sizeof(double), s);
  const double vol = g.dx[0] * g.dx[1] * g.dx[2];
  const double area[3] = {g.dx[1] * g.dx[2], g.dx[0] * g.dx[2], g.dx[0] * g.dx[1]};
  for (int d = 1; d <= g.ndim && e == cudaSuccess; ++d) {
    const double scale = bdt * (area[d - 1] / vol);  // mu = beta dt a
    e = d == 1 ? launch_pass<1>(A, recon, scale, prim, s)
               : d == 2 ? launch_pass<2>(A, recon, scale, prim, s) : launch_pass<3>(A, recon, scale, prim, s);
  }
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

// lam_n = (d U^{n+1} / d U^n)^T lam_next for the step whose stage inputs' primitives (as
// fwd_step keeps them: one pack field per stage) are `kept`, with dt.  lam_n may alias
// lam_next.
aph_status step_vjp_kept(aph_adjoint A, const double *kept, double dt, const double *lam_next,
                         double *lam_n, cudaStream_t s) {
  const std::vector<StageC> st = stages_for(A->integrator);
  const AdjGeom &g = A->g;
  const unsigned gx = (unsigned)((g.ncell + 255) / 256);
  k_axpby<<<dim3(gx, g.nblocks), 256, 0, s>>>(g, 1.0, lam_next, 0.0, nullptr, A->a);
  cudaError_t e = cudaGetLastError();
  const int ns = (int)st.size();
  for (int i = ns - 1; i >= 0 && e == cudaSuccess; --i) {
    const int recon = (A->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : A->params.recon;
    e = stage_vjp(A, recon, st[i].beta * dt, kept + (size_t)i * A->n, st[i].gam0, st[i].gam1,
                  i == ns - 1, i == 0 ? lam_n : nullptr, s);
  }
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "adjoint step");
}

// The same from the step's input u_n: recompute the step, keeping its stage inputs.
aph_status step_vjp(aph_adjoint A, const double *u_n, double dt, const double *lam_next,
                    double *lam_n, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(A->x, u_n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint step");
  if (aph_status r = fwd_step(A, dt, A->states, s)) return r;
  return step_vjp_kept(A, A->states, dt, lam_next, lam_n, s);
}

void adj_free(aph_adjoint A) {
  if (A->pack) aph_pack_destroy(A->pack);
  double *bufs[] = {A->x, A->u1, A->prim, A->gamma, A->flux[0], A->flux[1], A->flux[2], A->lam_w,
                    A->lam_u, A->a, A->acc, A->states, A->ckpts};
  for (double *p : bufs) cudaFree(p);
  cudaFree(A->floor_flag);
}

aph_status check_floor(aph_adjoint A, cudaStream_t s) {
  int f = 0;
  cudaError_t e = cudaMemcpyAsync(&f, A->floor_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint");
  if (f) return fail(APH_ERR_STATE, "a density or pressure floor fired: the step is not differentiable there");
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
  if (q.recon != APH_RECON_PLM && q.recon != APH_RECON_DC)
    return fail(APH_ERR_UNSUPPORTED, "the adjoint differentiates dc and plm reconstruction");
  if (q.rsolver != APH_RSOLVER_HLLE && q.rsolver != APH_RSOLVER_HLLC)
    return fail(APH_ERR_UNSUPPORTED, "the adjoint differentiates the hlle and hllc solvers");
  if (q.exact) return fail(APH_ERR_UNSUPPORTED, "the adjoint runs on the fast arithmetic");
  if (desc->use_gravity) return fail(APH_ERR_UNSUPPORTED, "the adjoint has no gravity source");
  if (stages_for(desc->integrator).empty()) return fail(APH_ERR_INVALID, "integrator not recognized");
  if (desc->nblocks <= 0 || !desc->blocks) return fail(APH_ERR_INVALID, "no blocks");
  aph_adjoint A = new aph_adjoint_s();
  A->params = q;
  A->integrator = desc->integrator;
  AdjGeom &g = A->g;
  std::memset(&g, 0, sizeof(g));
  g.nblocks = desc->nblocks;
  g.ndim = q.ndim;
  g.ng = q.nghost;
  for (int d = 0; d < 3; ++d) {
    g.nx[d] = desc->blocks[0].nx[d];
    g.dx[d] = desc->blocks[0].dx[d];
    g.nb[d] = desc->nb[d];
    g.bc[d][0] = desc->bc[2 * d];
    g.bc[d][1] = desc->bc[2 * d + 1];
  }
  g.ni = g.nx[0] + 2 * g.ng;
  g.nj = g.ndim >= 2 ? g.nx[1] + 2 * g.ng : 1;
  g.nk = g.ndim >= 3 ? g.nx[2] + 2 * g.ng : 1;
  g.ncell = (long long)g.ni * g.nj * g.nk;
  PackDev tmp;
  std::memset(&tmp, 0, sizeof(tmp));
  tmp.gm1 = q.gm1;
  fill_gas_consts(tmp);
  g.gc = GasConsts{tmp.gm1, tmp.igm1, tmp.gamma, tmp.c2g, tmp.one_igm1, tmp.hlle_k, tmp.hllc_k};
  g.ic2g = 1.0 / tmp.c2g;
  A->n = (size_t)g.nblocks * 5 * g.ncell;
  const size_t bytes = A->n * sizeof(double);
  const int ns = (int)stages_for(A->integrator).size();
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  double **bufs[] = {&A->x, &A->u1, &A->prim, &A->lam_w, &A->lam_u, &A->a, &A->acc};
  for (double **b : bufs) ck(cudaMalloc(b, bytes));
  ck(cudaMalloc(&A->gamma, bytes / 5 * 2));
  for (int d = 0; d < g.ndim; ++d) ck(cudaMalloc(&A->flux[d], bytes));
  ck(cudaMalloc(&A->states, bytes * ns));
  ck(cudaMalloc(&A->floor_flag, sizeof(int)));
  if (e == cudaSuccess) e = cudaMemset(A->floor_flag, 0, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(A->x, 0, bytes);
  if (e != cudaSuccess) {
    adj_free(A);
    delete A;
    return cuda_fail(e, "adjoint allocation");
  }
  std::vector<aph_block> blocks(g.nblocks);
  for (int b = 0; b < g.nblocks; ++b) {
    aph_block &B = blocks[b];
    std::memset(&B, 0, sizeof(B));
    const size_t o = (size_t)b * 5 * g.ncell;
    B.cons = A->x + o;
    B.u1 = A->u1 + o;
    B.prim = A->prim + o;
    B.gamma = A->gamma + (size_t)b * 2 * g.ncell;
    for (int d = 0; d < g.ndim; ++d) B.flux[d] = A->flux[d] + o;
    for (int d = 0; d < 3; ++d) {
      B.nx[d] = g.nx[d];
      B.dx[d] = g.dx[d];
    }
  }
  aph_hydro_params pq = q;
  aph_status st = aph_pack_create(&pq, blocks.data(), g.nblocks, &A->pack);
  if (st == APH_OK) st = aph_pack_set_topology(A->pack, desc->nb, desc->bc);
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
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  cudaError_t e = cudaMemcpyAsync(A->x, u_n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint forward");
  if (aph_status st = fwd_step(A, dt, nullptr, s)) return st;
  e = cudaMemcpyAsync(u_next, A->x, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint forward");
  return check_floor(A, s);
}

aph_status aph_adjoint_step_vjp(aph_adjoint A, const double *u_n, double dt, const double *lam_next,
                                double *lam_n, void *stream) {
  clear_error();
  if (!A || !u_n || !lam_next || !lam_n) return fail(APH_ERR_INVALID, "NULL argument");
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  if (aph_status st = step_vjp(A, u_n, dt, lam_next, lam_n, s)) return st;
  return check_floor(A, s);
}

aph_status aph_adjoint_forward(aph_adjoint A, const double *u0, int nsteps, const double *dts,
                               int checkpoint_every, double *u_final, void *stream) {
  clear_error();
  if (!A || !u0 || !dts || nsteps < 1 || !u_final) return fail(APH_ERR_INVALID, "bad argument");
  if (checkpoint_every < 1) checkpoint_every = nsteps;
  cudaStream_t s = (cudaStream_t)stream;
  const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every;
  if (nck != A->nckpt) {
    cudaFree(A->ckpts);
    A->ckpts = nullptr;
    cudaError_t e = cudaMalloc(&A->ckpts, (size_t)nck * A->n * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "checkpoint allocation");
    A->nckpt = nck;
  }
  A->dts.assign(dts, dts + nsteps);
  A->ckpt_every = checkpoint_every;
  cudaMemsetAsync(A->floor_flag, 0, sizeof(int), s);
  cudaError_t e = cudaMemcpyAsync(A->x, u0, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) {
    if (k % checkpoint_every == 0)
      e = cudaMemcpyAsync(A->ckpts + (size_t)(k / checkpoint_every) * A->n, A->x, A->n * sizeof(double),
                          cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) break;
    if (aph_status st = fwd_step(A, dts[k], nullptr, s)) return st;
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(u_final, A->x, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint rollout");
  return check_floor(A, s);
}

aph_status aph_adjoint_backward(aph_adjoint A, const double *lam_final, double *lam_initial,
                                void *stream) {
  clear_error();
  if (!A || !lam_final || !lam_initial) return fail(APH_ERR_INVALID, "NULL argument");
  if (A->dts.empty()) return fail(APH_ERR_INVALID, "no recorded rollout");
  cudaStream_t s = (cudaStream_t)stream;
  const int nsteps = (int)A->dts.size(), K = A->ckpt_every;
  const int ns = (int)stages_for(A->integrator).size();
  // segment storage: the stage inputs of every step of one segment, recomputed once from the
  // segment's checkpoint
  double *seg = nullptr;
  const size_t per_step = (size_t)ns * A->n;
  cudaError_t e = cudaMalloc(&seg, (size_t)K * per_step * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "segment allocation");
  e = cudaMemcpyAsync(lam_initial, lam_final, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  aph_status st = APH_OK;
  for (int j = A->nckpt - 1; j >= 0 && st == APH_OK && e == cudaSuccess; --j) {
    const int k0 = j * K, k1 = std::min(nsteps, k0 + K);
    e = cudaMemcpyAsync(A->x, A->ckpts + (size_t)j * A->n, A->n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    for (int k = k0; k < k1 && st == APH_OK && e == cudaSuccess; ++k)
      st = fwd_step(A, A->dts[k], seg + (size_t)(k - k0) * per_step, s);
    for (int k = k1 - 1; k >= k0 && st == APH_OK && e == cudaSuccess; --k)
      st = step_vjp_kept(A, seg + (size_t)(k - k0) * per_step, A->dts[k], lam_initial, lam_initial, s);
  }
  if (e == cudaSuccess && st == APH_OK) e = cudaStreamSynchronize(s);
  cudaFree(seg);
  if (st) return st;
  if (e != cudaSuccess) return cuda_fail(e, "adjoint backward");
  return check_floor(A, s);
}

}  // extern "C"
