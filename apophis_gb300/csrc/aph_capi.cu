// aph_capi.cu -- the C ABI of include/aph_hydro.h: argument checks, device-resident
// pack descriptors, dispatch to the fast or exact kernels, boundary fill.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/aph_hydro.h"
#include "aph_capi_internal.h"
#include "aph_internal.h"

namespace aph {

static thread_local std::string g_last_error;

aph_status fail(aph_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

aph_status cuda_fail(cudaError_t e, const char *where) {
  return fail(APH_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

void clear_error() { g_last_error.clear(); }

const char *last_error() { return g_last_error.c_str(); }

void fill_gas_consts(PackDev &p) {
  p.gamma = p.gm1 + 1.0;
  p.igm1 = 1.0 / p.gm1;
  p.c2g = 2.99792458e10 * 2.99792458e10 * p.gamma;
  p.one_igm1 = 1.0 + p.igm1;
  p.hlle_k = (p.gamma + 1.0) / std::sqrt(2.0 * p.gamma);
  p.hllc_k = (p.gamma + 1.0) / (2.0 * p.gamma);
}

aph_status validate_params(const aph_hydro_params *params) {
  if (!params) return fail(APH_ERR_INVALID, "params is NULL");
  const aph_hydro_params &q = *params;
  if (q.ndim < 1 || q.ndim > 3) return fail(APH_ERR_INVALID, "ndim %d not in 1..3", q.ndim);
  if (q.nvar < 5 || q.nvar > 64) return fail(APH_ERR_INVALID, "nvar %d not in 5..64", q.nvar);
  if (q.recon < APH_RECON_DC || q.recon > APH_RECON_PPM)
    return fail(APH_ERR_INVALID, "reconstruction %d not recognized", q.recon);
  if (q.rsolver < APH_RSOLVER_NONE || q.rsolver > APH_RSOLVER_LHLLC)
    return fail(APH_ERR_INVALID, "Riemann solver %d not recognized", q.rsolver);
  const int need = q.recon == APH_RECON_DC ? 1 : q.recon == APH_RECON_PLM ? 2 : 3;
  if (q.nghost < need)  // hydro.cpp:72-75
    return fail(APH_ERR_INVALID, "Not enough ghost zones for reconstruction (%d < %d)",
                q.nghost, need);
  if (q.rsolver == APH_RSOLVER_NONE && q.recon != APH_RECON_DC)  // hydro.cpp:89-93
    return fail(APH_ERR_INVALID, "'none' Riemann solver only works with dc reconstruction");
  if (!(q.gm1 > 0.0) || !std::isfinite(q.gm1))
    return fail(APH_ERR_INVALID, "eos gm1 must be positive and finite");
  if (!(q.cfl > 0.0)) return fail(APH_ERR_INVALID, "cfl must be positive");
  if (!(q.dfloor >= 0.0) || !(q.pfloor >= 0.0)) return fail(APH_ERR_INVALID, "floors must be >= 0");
  return APH_OK;
}

}  // namespace aph

using namespace aph;

struct aph_pack_s {
  aph_hydro_params params;
  PackDev dev;
  std::vector<BlockDev> host_blocks;
  BlockDev *d_blocks = nullptr;
  unsigned long long *d_scratch = nullptr;  // [0] dt min bits, [1] floor flag
  double *d_dt = nullptr;
  double *d_hist = nullptr;  // history partial sums (allocated on first use)
  size_t hist_len = 0;
  int max_ncell = 0, max_interior = 0;
  bool uniform = true;
  bool has_topology = false;
  aph_pack parent = nullptr;  // a partition shares its parent's descriptors
  int children = 0;           // live partitions of this pack
};

namespace aph {
const char *amr_check(int nb, const AmrFaces *F, const int (*nx)[2], int ng, char *msg, size_t len) {
  for (int b = 0; b < nb; ++b) {
    const AmrFaces &A = F[b];
    if (nx[b][0] < 2 * ng || nx[b][1] < 2 * ng) {
      snprintf(msg, len, "block %d: refined meshes need >= 2*nghost cells per side", b);
      return msg;
    }
    for (int f = 0; f < 4; ++f) {
      const int d = f / 2, td = 1 - d, kind = A.kind[f];
      if (kind < FACE_SAME || kind > FACE_BOUNDARY) {
        snprintf(msg, len, "block %d face %d: kind %d", b, f, kind);
        return msg;
      }
      const int need = kind == FACE_BOUNDARY ? 0 : 1;
      const int maxn = kind == FACE_FINER ? 4 : need;
      if (A.cnt[f] < need || A.cnt[f] > maxn) {
        snprintf(msg, len, "block %d face %d: %d neighbours", b, f, A.cnt[f]);
        return msg;
      }
      for (int n = 0; n < A.cnt[f]; ++n)
        if (A.nbr[f][n] < 0 || A.nbr[f][n] >= nb) {
          snprintf(msg, len, "block %d face %d: neighbour out of range", b, f);
          return msg;
        }
      const int t0 = A.origin[td], t1 = A.origin[td] + nx[b][td];
      if (kind == FACE_SAME) {
        const int m = A.nbr[f][0];
        if (F[m].level != A.level || F[m].origin[td] > t0 || F[m].origin[td] + nx[m][td] < t1) {
          snprintf(msg, len, "block %d face %d: same-level neighbour does not cover the face", b, f);
          return msg;
        }
      } else if (kind == FACE_COARSER) {
        const int m = A.nbr[f][0];
        if (F[m].level != A.level - 1 || (t0 & 1) || (nx[b][td] & 1) ||
            F[m].origin[td] > (t0 >> 1) || F[m].origin[td] + nx[m][td] < (t1 >> 1)) {
          snprintf(msg, len, "block %d face %d: coarser neighbour does not cover the face", b, f);
          return msg;
        }
      } else if (kind == FACE_FINER) {
        // every fine cell pair (2t, 2t+1) lies in one listed neighbour
        for (int t = t0; t < t1; ++t) {
          bool ok = false;
          for (int n = 0; n < A.cnt[f]; ++n) {
            const int m = A.nbr[f][n];
            ok |= F[m].level == A.level + 1 && F[m].origin[td] <= 2 * t &&
                  2 * t + 1 < F[m].origin[td] + nx[m][td];
          }
          if (!ok) {
            snprintf(msg, len, "block %d face %d: finer neighbours do not cover the face", b, f);
            return msg;
          }
        }
      }
    }
  }
  return nullptr;
}

const BlockDev *pack_blocks(aph_pack p) { return p->d_blocks; }
const PackDev &pack_dev(aph_pack p) { return p->dev; }
int pack_max_interior(aph_pack p) { return p->max_interior; }
int pack_max_ncell(aph_pack p) { return p->max_ncell; }
const aph_hydro_params &pack_params(aph_pack p) { return p->params; }
const std::vector<BlockDev> &pack_host_blocks(aph_pack p) { return p->host_blocks; }
bool pack_has_topology(aph_pack p) { return p->has_topology; }
}  // namespace aph

extern "C" {

const char *aph_last_error(void) { return aph::last_error(); }
int aph_version(void) { return 1; }

aph_status aph_pack_create(const aph_hydro_params *params, const aph_block *blocks, int nblocks,
                           aph_pack *out) {
  clear_error();
  if (!out) return fail(APH_ERR_INVALID, "out is NULL");
  *out = nullptr;
  aph_status st = validate_params(params);
  if (st) return st;
  if (!blocks || nblocks <= 0) return fail(APH_ERR_INVALID, "no blocks");
  aph_pack p = new aph_pack_s();
  p->params = *params;
  PackDev &d = p->dev;
  std::memset(&d, 0, sizeof(d));
  d.nblocks = nblocks;
  d.ndim = params->ndim;
  d.ng = params->nghost;
  d.nvar = params->nvar;
  d.gm1 = params->gm1;
  d.dfloor = params->dfloor;
  d.pfloor = params->pfloor;
  d.cfl = params->cfl;
  fill_gas_consts(d);
  p->host_blocks.resize(nblocks);
  for (int b = 0; b < nblocks; ++b) {
    const aph_block &a = blocks[b];
    BlockDev &B = p->host_blocks[b];
    std::memset(&B, 0, sizeof(B));
    for (int dd = 0; dd < 3; ++dd) {
      const int nx = a.nx[dd];
      if (dd < d.ndim ? nx < 1 : nx != 1) {
        delete p;
        return fail(APH_ERR_INVALID, "block %d: nx%d = %d invalid for ndim %d", b, dd + 1, nx, d.ndim);
      }
      if (!(a.dx[dd] > 0.0)) {
        delete p;
        return fail(APH_ERR_INVALID, "block %d: dx%d must be positive", b, dd + 1);
      }
      B.nx[dd] = nx;
      B.dx[dd] = a.dx[dd];
      d.max_nx[dd] = std::max(d.max_nx[dd], nx);
      if (nx != blocks[0].nx[dd]) p->uniform = false;
    }
    if (!a.cons) {
      delete p;
      return fail(APH_ERR_INVALID, "block %d: cons is NULL", b);
    }
    B.cons = a.cons;
    B.prim = a.prim;
    B.gamma = a.gamma;
    B.u1 = a.u1;
    for (int dd = 0; dd < 3; ++dd) B.flux[dd] = a.flux[dd];
    B.eos_lambda = a.eos_lambda;
    B.ni = a.nx[0] + 2 * d.ng;
    B.nj = d.ndim >= 2 ? a.nx[1] + 2 * d.ng : 1;
    B.nk = d.ndim >= 3 ? a.nx[2] + 2 * d.ng : 1;
    B.ncell = (long long)B.ni * B.nj * B.nk;
    if (B.ncell > (1LL << 31) / 64) {
      delete p;
      return fail(APH_ERR_INVALID, "block %d too large", b);
    }
    for (int dd = 0; dd < 3; ++dd) {  // flux layouts: the cons shape, or the caller's strides
      const long long *fs = a.flux_stride[dd];
      if (fs[0] == 0 && fs[1] == 0 && fs[2] == 0) {
        B.fs[dd][0] = B.ncell;
        B.fs[dd][1] = (long long)B.ni * B.nj;
        B.fs[dd][2] = B.ni;
        continue;
      }
      // rows hold the faces of a cons row (one more along d), planes their rows, components
      // their planes: every face the kernels address lies inside its own slot
      const long long ri = B.ni + (dd == 0 ? 1 : 0);
      const long long rj = B.nj + (dd == 1 && d.ndim >= 2 ? 1 : 0);
      const long long rk = B.nk + (dd == 2 && d.ndim >= 3 ? 1 : 0);
      if (fs[2] < ri || fs[1] < fs[2] * rj || fs[0] < fs[1] * rk || fs[0] > (1LL << 40)) {
        delete p;
        return fail(APH_ERR_INVALID,
                    "block %d: flux[%d] strides (%lld, %lld, %lld) do not hold a (%lld, %lld, %lld) "
                    "face array per component", b, dd, fs[0], fs[1], fs[2], rk, rj, ri);
      }
      for (int q = 0; q < 3; ++q) B.fs[dd][q] = fs[q];
    }
    p->max_ncell = std::max<long long>(p->max_ncell, B.ncell);
    p->max_interior = std::max(p->max_interior, a.nx[0] * a.nx[1] * a.nx[2]);
  }
  cudaError_t e = cudaMalloc(&p->d_blocks, sizeof(BlockDev) * nblocks);
  if (e == cudaSuccess)
    e = cudaMemcpy(p->d_blocks, p->host_blocks.data(), sizeof(BlockDev) * nblocks,
                   cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_scratch, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_dt, 2 * sizeof(double));
  if (e != cudaSuccess) {
    aph_pack_destroy(p);
    return cuda_fail(e, "aph_pack_create");
  }
  *out = p;
  return APH_OK;
}

aph_status aph_pack_set_topology(aph_pack p, const int nb[3], const int bc[6]) {
  clear_error();
  if (!p || !nb || !bc) return fail(APH_ERR_INVALID, "NULL argument");
  if (!p->uniform) return fail(APH_ERR_UNSUPPORTED, "block grid topology needs equal blocks");
  if ((long long)nb[0] * nb[1] * nb[2] != p->dev.nblocks)
    return fail(APH_ERR_INVALID, "nb product %d*%d*%d != nblocks %d", nb[0], nb[1], nb[2],
                p->dev.nblocks);
  for (int dd = 0; dd < 3; ++dd) {
    if (dd >= p->dev.ndim && nb[dd] != 1) return fail(APH_ERR_INVALID, "nb%d must be 1", dd + 1);
    for (int s = 0; s < 2; ++s)
      if (bc[2 * dd + s] < APH_BC_PERIODIC || bc[2 * dd + s] > APH_BC_REFLECT)
        return fail(APH_ERR_INVALID, "bc %d not recognized", bc[2 * dd + s]);
    p->dev.nb[dd] = nb[dd];
    p->dev.bc[dd][0] = bc[2 * dd];
    p->dev.bc[dd][1] = bc[2 * dd + 1];
    p->dev.mesh_nx[dd] = nb[dd] * p->host_blocks[0].nx[dd];
  }
  for (int b = 0; b < p->dev.nblocks; ++b) {
    BlockDev &B = p->host_blocks[b];
    B.loc[0] = b % nb[0];
    B.loc[1] = (b / nb[0]) % nb[1];
    B.loc[2] = b / (nb[0] * nb[1]);
  }
  cudaError_t e = cudaMemcpy(p->d_blocks, p->host_blocks.data(),
                             sizeof(BlockDev) * p->dev.nblocks, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "aph_pack_set_topology");
  p->has_topology = true;
  return APH_OK;
}

aph_status aph_pack_set_amr(aph_pack p, const aph_amr_block *amr, const int bc[6]) {
  clear_error();
  if (!p || !amr || !bc) return fail(APH_ERR_INVALID, "NULL argument");
  if (p->parent) return fail(APH_ERR_INVALID, "set the mesh on the parent pack");
  if (p->dev.ndim != 2) return fail(APH_ERR_UNSUPPORTED, "refined meshes are 2D");
  if (p->children) return fail(APH_ERR_INVALID, "set the mesh before partitioning the pack");
  const int nb = p->dev.nblocks;
  static_assert(sizeof(AmrFaces) == sizeof(aph_amr_block), "face table layout");
  std::vector<AmrFaces> faces(nb);
  std::vector<int> nxs(2 * nb);
  for (int b = 0; b < nb; ++b) {
    std::memcpy(&faces[b], &amr[b], sizeof(AmrFaces));
    nxs[2 * b] = p->host_blocks[b].nx[0];
    nxs[2 * b + 1] = p->host_blocks[b].nx[1];
  }
  char msg[160];
  if (amr_check(nb, faces.data(), (const int(*)[2])nxs.data(), p->dev.ng, msg, sizeof(msg)))
    return fail(APH_ERR_INVALID, "%s", msg);
  for (int d = 0; d < 2; ++d)
    for (int s = 0; s < 2; ++s)
      if (bc[2 * d + s] < 0 || bc[2 * d + s] > 2)
        return fail(APH_ERR_INVALID, "boundary condition %d not recognized", bc[2 * d + s]);
  for (int b = 0; b < nb; ++b) p->host_blocks[b].amr = faces[b];
  for (int d = 0; d < 3; ++d) {
    p->dev.bc[d][0] = bc[2 * d];
    p->dev.bc[d][1] = bc[2 * d + 1];
  }
  p->dev.amr = 1;
  cudaError_t e = cudaMemcpy(p->d_blocks, p->host_blocks.data(), sizeof(BlockDev) * nb,
                             cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "aph_pack_set_amr");
  p->has_topology = true;
  return APH_OK;
}

aph_status aph_amr_check(const aph_amr_block *amr, const int *nx, int nblocks, int nghost) {
  clear_error();
  if (!amr || !nx || nblocks <= 0 || nghost < 1) return fail(APH_ERR_INVALID, "bad argument");
  std::vector<AmrFaces> faces(nblocks);
  for (int b = 0; b < nblocks; ++b) std::memcpy(&faces[b], &amr[b], sizeof(AmrFaces));
  char msg[160];
  if (amr_check(nblocks, faces.data(), (const int(*)[2])nx, nghost, msg, sizeof(msg)))
    return fail(APH_ERR_INVALID, "%s", msg);
  return APH_OK;
}

aph_status aph_pack_partition(aph_pack parent, int first, int count, aph_pack *out) {
  clear_error();
  if (!parent || !out) return fail(APH_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (parent->parent) return fail(APH_ERR_INVALID, "partition of a partition");
  if (first < 0 || count < 1 || first + count > parent->dev.nblocks)
    return fail(APH_ERR_INVALID, "blocks %d..%d outside the pack", first, first + count - 1);
  aph_pack p = new aph_pack_s();
  p->params = parent->params;
  p->dev = parent->dev;
  p->dev.block0 = first;
  p->dev.nblocks = count;
  p->host_blocks.assign(parent->host_blocks.begin() + first, parent->host_blocks.begin() + first + count);
  p->d_blocks = parent->d_blocks;
  p->parent = parent;
  parent->children++;
  p->uniform = parent->uniform;
  p->has_topology = parent->has_topology;
  for (int d = 0; d < 3; ++d) p->dev.max_nx[d] = 0;
  for (const BlockDev &B : p->host_blocks) {
    p->max_ncell = std::max<long long>(p->max_ncell, B.ncell);
    p->max_interior = std::max(p->max_interior, B.nx[0] * B.nx[1] * B.nx[2]);
    for (int d = 0; d < 3; ++d) p->dev.max_nx[d] = std::max(p->dev.max_nx[d], B.nx[d]);
  }
  cudaError_t e = cudaMalloc(&p->d_scratch, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&p->d_dt, 2 * sizeof(double));
  if (e != cudaSuccess) {
    aph_pack_destroy(p);
    return cuda_fail(e, "aph_pack_partition");
  }
  *out = p;
  return APH_OK;
}

aph_status aph_pack_destroy(aph_pack p) {
  clear_error();
  if (!p) return APH_OK;
  if (p->children)
    return fail(APH_ERR_INVALID, "pack has %d live partitions: destroy them first", p->children);
  if (p->parent) {
    p->parent->children--;
    p->d_blocks = nullptr;
  }
  if (p->d_blocks) cudaFree(p->d_blocks);
  if (p->d_scratch) cudaFree(p->d_scratch);
  if (p->d_dt) cudaFree(p->d_dt);
  if (p->d_hist) cudaFree(p->d_hist);
  delete p;
  return APH_OK;
}

static aph_status check_fields(aph_pack p, bool prim, bool gamma, bool flux, bool u1) {
  for (int b = 0; b < p->dev.nblocks; ++b) {
    const BlockDev &B = p->host_blocks[b];
    if (prim && !B.prim) return fail(APH_ERR_INVALID, "block %d: prim is NULL", b);
    if (gamma && !B.gamma) return fail(APH_ERR_INVALID, "block %d: gamma is NULL", b);
    if (u1 && !B.u1) return fail(APH_ERR_INVALID, "block %d: u1 is NULL", b);
    if (flux)
      for (int dd = 0; dd < p->dev.ndim; ++dd)
        if (!B.flux[dd]) return fail(APH_ERR_INVALID, "block %d: flux[%d] is NULL", b, dd);
  }
  return APH_OK;
}

aph_status aph_hydro_cons_to_prim(aph_pack p, void *stream) {
  clear_error();
  if (!p) return fail(APH_ERR_INVALID, "pack is NULL");
  if (aph_status st = check_fields(p, true, false, false, false)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = p->params.exact
                      ? aph_exact::launch_cons_to_prim(p->dev, p->d_blocks, p->max_ncell, nullptr, s)
                      : aph_fast::launch_cons_to_prim(p->dev, p->d_blocks, p->max_ncell, nullptr, s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "cons_to_prim");
}

aph_status aph_hydro_calculate_fluxes(aph_pack p, int recon, int rsolver, void *stream) {
  clear_error();
  if (!p) return fail(APH_ERR_INVALID, "pack is NULL");
  if (recon < APH_RECON_DC || recon > APH_RECON_PPM)
    return fail(APH_ERR_INVALID, "reconstruction %d not recognized", recon);
  if (rsolver < APH_RSOLVER_NONE || rsolver > APH_RSOLVER_LHLLC)
    return fail(APH_ERR_INVALID, "Riemann solver %d not recognized", rsolver);
  if (rsolver == APH_RSOLVER_NONE && recon != APH_RECON_DC)
    return fail(APH_ERR_INVALID, "'none' Riemann solver only works with dc reconstruction");
  const int need = recon == APH_RECON_DC ? 1 : recon == APH_RECON_PLM ? 2 : 3;
  if (p->dev.ng < need) return fail(APH_ERR_INVALID, "Not enough ghost zones for reconstruction");
  if (aph_status st = check_fields(p, true, true, true, false)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  for (int dir = 1; dir <= p->dev.ndim; ++dir) {
    cudaError_t e = p->params.exact
                        ? aph_exact::launch_fluxes(p->dev, p->d_blocks, dir, recon, rsolver, s)
                        : aph_fast::launch_fluxes(p->dev, p->d_blocks, dir, recon, rsolver, s);
    if (e != cudaSuccess) return cuda_fail(e, "calculate_fluxes");
  }
  return APH_OK;
}

static aph_status update_impl(aph_pack p, double gam0, double gam1, double beta, double beta_dt,
                              const double *dt_dev, void *stream) {
  clear_error();
  if (!p) return fail(APH_ERR_INVALID, "pack is NULL");
  if (aph_status st = check_fields(p, false, false, true, true)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = p->params.exact
                      ? aph_exact::launch_update(p->dev, p->d_blocks, gam0, gam1, beta, beta_dt,
                                                 dt_dev, p->max_interior, s)
                      : aph_fast::launch_update(p->dev, p->d_blocks, gam0, gam1, beta, beta_dt,
                                                dt_dev, p->max_interior, s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "update_with_flux_divergence");
}

aph_status aph_hydro_update_with_flux_divergence(aph_pack p, double gam0, double gam1,
                                                 double beta_dt, void *stream) {
  return update_impl(p, gam0, gam1, 0.0, beta_dt, nullptr, stream);
}

aph_status aph_hydro_update_with_flux_divergence_dev(aph_pack p, double gam0, double gam1,
                                                     double beta, const double *dt_dev,
                                                     void *stream) {
  if (!dt_dev) return fail(APH_ERR_INVALID, "dt_dev is NULL");
  return update_impl(p, gam0, gam1, beta, 0.0, dt_dev, stream);
}

__global__ void k_dt_init(unsigned long long *bits) { bits[0] = ~0ULL; }

__global__ void k_dt_finish(const unsigned long long *bits, double cfl, double *dt_out) {
  const unsigned long long b = bits[0];
  // no interior cell gave a finite candidate: numeric_limits<Real>::max() as the reference
  const double m = (b == ~0ULL) ? 1.7976931348623157e308 : __longlong_as_double((long long)b);
  dt_out[0] = cfl * m;
}

aph_status aph_hydro_estimate_timestep_async(aph_pack p, double *dt_dev, void *stream) {
  clear_error();
  if (!p || !dt_dev) return fail(APH_ERR_INVALID, "NULL argument");
  if (aph_status st = check_fields(p, true, false, false, false)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  k_dt_init<<<1, 1, 0, s>>>(p->d_scratch);
  cudaError_t e = p->params.exact
                      ? aph_exact::launch_estimate_dt(p->dev, p->d_blocks, p->max_interior, p->d_scratch, s)
                      : aph_fast::launch_estimate_dt(p->dev, p->d_blocks, p->max_interior, p->d_scratch, s);
  if (e != cudaSuccess) return cuda_fail(e, "estimate_timestep");
  k_dt_finish<<<1, 1, 0, s>>>(p->d_scratch, p->dev.cfl, dt_dev);
  e = cudaGetLastError();
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "estimate_timestep");
}

aph_status aph_hydro_estimate_timestep(aph_pack p, double *dt_host, void *stream) {
  if (!dt_host) return fail(APH_ERR_INVALID, "dt_host is NULL");
  aph_status st = aph_hydro_estimate_timestep_async(p, p ? p->d_dt : nullptr, stream);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemcpyAsync(dt_host, p->d_dt, sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "estimate_timestep");
}

aph_status aph_hydro_history(aph_pack p, double out[2], void *stream) {
  clear_error();
  if (!p || !out) return fail(APH_ERR_INVALID, "NULL argument");
  const size_t need = history_scratch_doubles(p->max_interior, p->dev.nblocks);
  if (p->hist_len < need) {
    if (p->d_hist) cudaFree(p->d_hist);
    p->d_hist = nullptr;
    p->hist_len = 0;
    cudaError_t e = cudaMalloc(&p->d_hist, need * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "history scratch");
    p->hist_len = need;
  }
  cudaStream_t s = (cudaStream_t)stream;
  double *res = p->d_hist + need - 2;
  cudaError_t e = launch_history(p->dev, p->d_blocks, p->max_interior, p->d_hist, need - 2, res, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "history");
}

aph_status aph_hydro_apply_gravity(aph_pack p, const double g[3], double beta_dt, void *stream) {
  clear_error();
  if (!p || !g) return fail(APH_ERR_INVALID, "NULL argument");
  if (aph_status st = check_fields(p, true, false, false, false)) return st;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = p->params.exact
                      ? aph_exact::launch_apply_gravity(p->dev, p->d_blocks, g[0], g[1], g[2], 0.0,
                                                        beta_dt, nullptr, p->max_interior, s)
                      : aph_fast::launch_apply_gravity(p->dev, p->d_blocks, g[0], g[1], g[2], 0.0,
                                                       beta_dt, nullptr, p->max_interior, s);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "apply_gravity");
}

aph_status aph_hydro_fill_ghosts(aph_pack p, void *stream) {
  clear_error();
  if (!p) return fail(APH_ERR_INVALID, "pack is NULL");
  if (!p->has_topology) return fail(APH_ERR_INVALID, "pack has no block-grid topology");
  cudaError_t e = launch_fill_ghosts(p->dev, p->d_blocks, p->max_ncell, 0, (cudaStream_t)stream);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "fill_ghosts");
}

}  // extern "C"
