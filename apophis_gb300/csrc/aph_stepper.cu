// aph_stepper.cu -- the batched path: a whole RK step of a pack as persistent stage
// launches, dt and time kept on the device, the step captured once as a CUDA graph and
// replayed; plus the autotuner that picks CTA size, lines per work item, sweep order
// and the CTA schedule.
#include <algorithm>
#include <utility>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "../../include/aph_hydro.h"
#include "aph_capi_internal.h"
#include "aph_internal.h"

using namespace aph;

namespace {

constexpr int kCellChunk = 256;

__global__ void k_ctl_init(StepCtl *c, double tlim, double dt_fixed) {
  c->dt = 0.0;
  c->time = 0.0;
  c->tlim = tlim;
  c->dt_fixed = dt_fixed;
  c->min_bits = ~0ULL;
  c->ncycle = 0;
  c->error = 0;
  c->nonfinite = 0;
  c->bar_count = 0;
  c->bar_gen = 0;
  for (int i = 0; i < 8; ++i) c->work[i] = 0;
}

__device__ __forceinline__ double min_to_dt(unsigned long long b, double cfl) {
  const double m = (b == ~0ULL) ? DBL_MAX : __longlong_as_double((long long)b);
  return cfl * m;
}

// After the initial estimate: dt_0 = cfl * min, clipped at tlim.
__global__ void k_dt_initial(StepCtl *c, double cfl) {
  double dt = c->dt_fixed > 0.0 ? c->dt_fixed : min_to_dt(c->min_bits, cfl);
  if (c->dt_fixed <= 0.0 && c->time < c->tlim && (c->tlim - c->time) < dt) dt = c->tlim - c->time;
  if (c->time >= c->tlim) dt = 0.0;
  c->dt = dt;
  c->min_bits = ~0ULL;
}

// End of a step: advance time, dt_{n+1} = min(2 dt_n, cfl * min), clipped at tlim.  given >= 0:
// the estimate cfl * min comes from the caller (sharded packs: the minimum over all ranks).
__global__ void k_dt_policy(StepCtl *c, double cfl, double given = -1.0) {
  const double used = c->dt;
  if (used > 0.0) {
    c->time += used;
    c->ncycle += 1;
  }
  double next;
  if (c->dt_fixed > 0.0) {
    next = c->time < c->tlim ? c->dt_fixed : 0.0;
  } else {
    const double est = given >= 0.0 ? given : min_to_dt(c->min_bits, cfl);
    const double two = 2.0 * used;
    next = (est < two) ? est : two;
    if (c->time < c->tlim && (c->tlim - c->time) < next) next = c->tlim - c->time;
    if (c->time >= c->tlim) next = 0.0;
  }
  c->dt = next;
  c->min_bits = ~0ULL;
  c->bar_count = 0;
}

// Ensembles: the same policy per member (one CTA over all members), and a summary in the
// pack's control block: the earliest member time, the largest next dt, the largest cycle
// count.  initial: dt_0 from the initial estimate.
__global__ void k_members_policy(StepCtl *c, MemberCtl *m, int n, double cfl, int initial) {
  __shared__ double s_time[256], s_dt[256];
  __shared__ int s_cyc[256];
  double tmin = DBL_MAX, dmax = 0.0;
  int cyc = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    MemberCtl &x = m[i];
    double next;
    if (initial) {
      next = c->dt_fixed > 0.0 ? c->dt_fixed : min_to_dt(x.min_bits, cfl);
    } else {
      const double used = x.active ? x.dt : 0.0;
      if (used > 0.0) {
        x.time += used;
        x.ncycle += 1;
      }
      if (c->dt_fixed > 0.0) {
        next = c->dt_fixed;
      } else {
        const double est = min_to_dt(x.min_bits, cfl);
        const double two = 2.0 * used;
        next = (est < two) ? est : two;
      }
    }
    if (c->dt_fixed <= 0.0 && x.time < x.tlim && (x.tlim - x.time) < next) next = x.tlim - x.time;
    x.active = x.time < x.tlim && next > 0.0;
    x.dt = x.active ? next : 0.0;
    x.min_bits = ~0ULL;
    tmin = x.time < tmin ? x.time : tmin;
    dmax = x.dt > dmax ? x.dt : dmax;
    cyc = x.ncycle > cyc ? x.ncycle : cyc;
  }
  s_time[threadIdx.x] = tmin;
  s_dt[threadIdx.x] = dmax;
  s_cyc[threadIdx.x] = cyc;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < blockDim.x; ++i) {
      tmin = s_time[i] < tmin ? s_time[i] : tmin;
      dmax = s_dt[i] > dmax ? s_dt[i] : dmax;
      cyc = s_cyc[i] > cyc ? s_cyc[i] : cyc;
    }
    c->time = tmin;
    c->dt = dmax;
    c->ncycle = cyc;
    c->min_bits = ~0ULL;
    c->bar_count = 0;
  }
}

struct Stage {
  double gam0, gam1, beta;
};

std::vector<Stage> stages_of(int integrator) {
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

struct aph_stepper_s {
  aph_hydro_params params;
  int integrator = 0;
  PackDev dev;
  std::vector<StepBlock> hblocks;
  StepBlock *d_blocks = nullptr;
  double *d_u1 = nullptr, *d_prim = nullptr, *d_gamma = nullptr, *d_du = nullptr;
  double *d_eraw = nullptr, *d_efl = nullptr;  // energy before / after the step-end floors
  double *d_backup = nullptr;  // autotuner state backup
  unsigned long long *d_flags = nullptr;  // block flags, then the launch counter (StageArgs)
  StepCtl *d_ctl = nullptr;
  int2 *d_cell_items = nullptr;
  int ncell_items = 0;
  int2 *d_line_items[3] = {nullptr, nullptr, nullptr};
  int nline_items[3] = {0, 0, 0};
  int *d_fix_items = nullptr;   // refined meshes: blocks with a finer neighbour
  int nfix_items = 0;
  double *d_bflux = nullptr;
  int bflux_stride = 0;
  int T[3] = {0, 0, 0};
  aph_stepper_config cfg;
  int grid = 0;
  size_t smem = 0;
  bool cooperative = true;
  double grav[3] = {0, 0, 0};
  int gravity = 0;
  long long total_cells = 0, total_interior = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  std::vector<std::vector<double *>> u0_ptrs;
  MemberCtl *d_members = nullptr;  // ensembles
  int nmembers = 0;
  double *d_hist = nullptr;        // history partial sums (allocated on first use)
  size_t hist_len = 0;
  void *d_tmaps = nullptr;         // TMA: tensor maps of the x, y, z windows (3 x 128 bytes)
};

namespace {

aph_status upload_items(aph_stepper s, int2 **dst, const std::vector<int2> &v) {
  if (*dst) cudaFree(*dst);
  *dst = nullptr;
  if (v.empty()) return APH_OK;
  cudaError_t e = cudaMalloc(dst, v.size() * sizeof(int2));
  if (e == cudaSuccess) e = cudaMemcpy(*dst, v.data(), v.size() * sizeof(int2), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "stepper items");
}

int auto_lines(int n) { return (n + 2 >= 256) ? 1 : std::max(1, 256 / (n + 2)); }

void destroy_graph(aph_stepper s) {
  if (s->exec) cudaGraphExecDestroy(s->exec);
  if (s->graph) cudaGraphDestroy(s->graph);
  s->exec = nullptr;
  s->graph = nullptr;
}

// TMA staging of pass windows (cfg.tma): every block of the same size, laid out back to back
// in prim as [block][var][k][j][i]; TMA's rules: 16-byte strides (ni even), each box side
// <= 256, the innermost box side a multiple of 16 bytes (T even across y and z) starting on
// a 16-byte boundary (nghost even, item starts even); an item spans at most two planes of
// lines (T <= the lines of a plane).  Returns nullptr or the reason.
const char *tma_unsupported(aph_stepper s, const int T[3]) {
  const PackDev &p = s->dev;
  const StepBlock &B0 = s->hblocks[0];
  for (const StepBlock &B : s->hblocks)
    for (int d = 0; d < 3; ++d)
      if (B.nx[d] != B0.nx[d]) return "blocks of different sizes";
  if (B0.ni % 2) return "an odd row length";
  if (p.ng % 2) return "an odd ghost width";
  const int ext[3] = {B0.ni, B0.nj, B0.nk};
  for (int d = 0; d < p.ndim; ++d) {
    if (ext[d] > 256 || T[d] > 256) return "a window side above 256";
    if (d == 0 && T[0] > B0.nx[1]) return "x items longer than a plane of lines";
    if (d > 0 && (T[d] % 2 || B0.nx[0] % 2 || T[d] > B0.nx[0]))
      return "y/z items of an odd line count, odd planes or items longer than a plane";
  }
  return nullptr;
}

aph_status encode_tmaps(aph_stepper s) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000,
                                                     cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(APH_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled is not available");
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const StepBlock &B0 = s->hblocks[0];
  const PackDev &p = s->dev;
  const cuuint64_t dims[5] = {(cuuint64_t)B0.ni, (cuuint64_t)B0.nj, (cuuint64_t)B0.nk,
                              (cuuint64_t)p.nvar, (cuuint64_t)p.nblocks};
  const cuuint64_t strides[4] = {(cuuint64_t)B0.ni * 8, (cuuint64_t)B0.ni * B0.nj * 8,
                                 (cuuint64_t)B0.ncell * 8, (cuuint64_t)B0.ncell * p.nvar * 8};
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  CUtensorMap maps[3];
  std::memset(maps, 0, sizeof(maps));
  for (int d = 0; d < 3; ++d) {
    cuuint32_t box[5] = {1, 1, 1, (cuuint32_t)p.nvar, 1};
    const int T = std::max(1, s->T[d]);
    if (d == 0) { box[0] = B0.ni; box[1] = T; }
    else if (d == 1) { box[0] = T; box[1] = B0.nj; }
    else { box[0] = T; box[2] = B0.nk; }
    if (d >= p.ndim) continue;
    CUresult r = encode(&maps[d], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 5, (void *)s->d_prim, dims, strides, box,
                        estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(APH_ERR_UNSUPPORTED, "tensor map encoding failed (%d)", (int)r);
  }
  cudaError_t e = cudaSuccess;
  if (!s->d_tmaps) e = cudaMalloc(&s->d_tmaps, sizeof(maps));
  if (e == cudaSuccess) e = cudaMemcpy(s->d_tmaps, maps, sizeof(maps), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "tensor maps");
}

// Lines per item of every direction (requested counts, 0 = automatic, capped by the lines
// of the largest block) and the shared memory a CTA needs for them.
size_t stage_lines(aph_stepper s, const int lines[3], bool tma, int T_out[3]) {
  const PackDev &p = s->dev;
  const int recon = s->params.recon;
  size_t smem = 0;
  for (int d = 0; d < 3; ++d) T_out[d] = 0;
  for (int d = 0; d < p.ndim; ++d) {
    const int n = p.max_nx[d];
    int T = lines[d] > 0 ? lines[d] : auto_lines(n);
    int ntr_max = 1;
    for (const StepBlock &B : s->hblocks) {
      const int ntr = d == 0 ? B.nx[1] * B.nx[2] : d == 1 ? B.nx[0] * B.nx[2] : B.nx[0] * B.nx[1];
      ntr_max = std::max(ntr_max, ntr);
    }
    T = std::min(T, ntr_max);
    T_out[d] = T;
    const int ext = d == 0 ? s->hblocks[0].ni : d == 1 ? s->hblocks[0].nj : s->hblocks[0].nk;
    const int nv = p.nvar;
    const size_t need = tma ? (s->params.exact ? aph_exact::stage_smem_bytes_tma(recon, n, T, ext, nv)
                                               : aph_fast::stage_smem_bytes_tma(recon, n, T, ext, nv))
                            : (s->params.exact ? aph_exact::stage_smem_bytes(recon, n, T, nv)
                                               : aph_fast::stage_smem_bytes(recon, n, T, nv));
    smem = std::max(smem, need);
  }
  return smem;
}

// Resident stage CTAs per SM for a launch shape (the fewest over the kernels a step
// launches: VL2's first stage reconstructs donor-cell); 0 if it does not fit.
int stage_residency(aph_stepper s, int threads, int reg_cap, size_t smem) {
  std::vector<int> recons = {s->params.recon};
  if (s->integrator == APH_INTEGRATOR_VL2 && s->params.recon != APH_RECON_DC) recons.push_back(APH_RECON_DC);
  int per_sm = 1 << 30;
  for (int rc : recons) {
    int k = 0;
    cudaError_t e = s->params.exact
                        ? aph_exact::stage_occupancy(rc, s->params.rsolver, threads, smem, reg_cap, &k)
                        : aph_fast::stage_occupancy(rc, s->params.rsolver, threads, smem, reg_cap, &k);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return 0;
    }
    per_sm = std::min(per_sm, k);
  }
  return per_sm;
}

// Build work lists, shared-memory size and grid for the current configuration.
aph_status configure(aph_stepper s) {
  destroy_graph(s);
  const PackDev &p = s->dev;
  const int nb = p.nblocks;
  // lines per item and shared memory per direction
  const size_t smem = stage_lines(s, s->cfg.lines, s->cfg.tma != 0, s->T);
  auto smem_of = [&](int n, int T) {
    return s->params.exact ? aph_exact::stage_smem_bytes(s->params.recon, n, T, p.nvar)
                           : aph_fast::stage_smem_bytes(s->params.recon, n, T, p.nvar);
  };
  if (smem > 220 * 1024)
    return fail(APH_ERR_UNSUPPORTED, "stage needs %zu bytes of shared memory; use fewer lines", smem);
  const int threads = s->cfg.threads;
  int per_sm = stage_residency(s, threads, s->cfg.reg_cap, smem);
  if (per_sm < 1) return fail(APH_ERR_UNSUPPORTED, "stage kernel does not fit on an SM");
  if (s->cfg.ctas_per_sm > 0) per_sm = std::min(per_sm, s->cfg.ctas_per_sm);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  std::vector<int> order(nb);  // largest blocks first
  for (int b = 0; b < nb; ++b) order[b] = b;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
    return s->hblocks[x].nint > s->hblocks[y].nint;
  });
  for (int d = 0; d < p.ndim; ++d) {
    const int T = s->T[d];
    struct Item { int2 w; long long cost; };
    std::vector<Item> list;
    for (int b : order) {
      const StepBlock &B = s->hblocks[b];
      const int n = B.nx[d];
      const int ntr = d == 0 ? B.nx[1] * B.nx[2] : d == 1 ? B.nx[0] * B.nx[2] : B.nx[0] * B.nx[1];
      if (ntr >= (1 << (31 - kItemLineBits)) || T >= (1 << kItemLineBits))
        return fail(APH_ERR_UNSUPPORTED, "block %d: %d lines along x%d, %d per item: too many", b, ntr,
                    d + 1, T);
      auto add = [&](int first, int lines) {
        list.push_back(Item{make_int2(b, (first << kItemLineBits) | lines), (long long)lines * n});
      };
      if (s->cfg.tma) {  // the TMA box's T lines, the block's last item shorter
        for (int l = 0; l < ntr; l += T) add(l, std::min(T, ntr - l));
        continue;
      }
      // plain loads: a narrower block takes as many lines per item as the shared memory
      // sized for the widest holds, and its lines are spread evenly over the fewest items
      int Tb = std::min(T, ntr);
      while (Tb < ntr && Tb + 1 < (1 << kItemLineBits) && smem_of(n, Tb + 1) <= smem) ++Tb;
      const int k = (ntr + Tb - 1) / Tb, base = ntr / k, rem = ntr % k;
      for (int i = 0, l = 0; i < k; ++i) {
        const int lines = base + (i < rem ? 1 : 0);
        add(l, lines);
        l += lines;
      }
    }
    // schedule order: the costliest items first (longest-processing-time), so that the tail
    // of a pass holds the cheap ones
    std::stable_sort(list.begin(), list.end(), [](const Item &x, const Item &y) { return x.cost > y.cost; });
    std::vector<int2> items(list.size());
    for (size_t i = 0; i < list.size(); ++i) items[i] = list[i].w;
    s->nline_items[d] = (int)items.size();
    if (aph_status st = upload_items(s, &s->d_line_items[d], items)) return st;
  }
  if (s->cfg.tma) {
    if (const char *why = tma_unsupported(s, s->T))
      return fail(APH_ERR_UNSUPPORTED, "TMA windows need other lines per item or blocks: %s", why);
    if (aph_status st = encode_tmaps(s)) return st;
  }
  s->smem = smem;
  // entire-domain cell chunks
  std::vector<int2> cells;
  for (int b = 0; b < nb; ++b)
    for (long long c = 0; c < s->hblocks[b].ncell; c += threads) cells.push_back(make_int2(b, (int)c));
  s->ncell_items = (int)cells.size();
  // no more CTAs than the largest phase has work items: a small pack (one Sod block) then
  // waits at its grid barriers for a few CTAs instead of a full GPU's worth
  int most = std::max(s->ncell_items, s->nfix_items);
  for (int d = 0; d < p.ndim; ++d) most = std::max(most, s->nline_items[d]);
  s->grid = std::max(1, std::min(per_sm * sms, most));
  return upload_items(s, &s->d_cell_items, cells);
}

StageArgs stage_args(aph_stepper s, int stage_idx, const Stage &st, bool last, bool init) {
  StageArgs a;
  std::memset(&a, 0, sizeof(a));
  a.p = s->dev;
  a.blocks = s->d_blocks;
  a.ctl = s->d_ctl;
  a.block_flags = s->d_flags;
  a.cell_items = s->d_cell_items;
  a.ncell_items = s->ncell_items;
  for (int d = 0; d < 3; ++d) {
    a.line_items[d] = s->d_line_items[d];
    a.nline_items[d] = s->nline_items[d];
    a.T[d] = s->T[d];
    a.order[d] = s->cfg.order[d];
  }
  a.gam0 = st.gam0;
  a.gam1 = st.gam1;
  a.beta = st.beta;
  for (int d = 0; d < 3; ++d) a.grav[d] = s->grav[d];
  a.gravity = s->gravity;
  a.copy_u1 = stage_idx == 0;
  a.last = last;
  a.init = init;
  a.schedule = s->cfg.schedule;
  a.timeout_ns = 4000000000ULL;
  a.fix_items = s->d_fix_items;
  a.nfix_items = s->nfix_items;
  a.bflux_stride = s->bflux_stride;
  a.cf = s->nfix_items > 0;
  a.members = s->d_members;
  a.tmaps = s->cfg.tma ? s->d_tmaps : nullptr;
  a.ext[0] = s->hblocks[0].ni;
  a.ext[1] = s->hblocks[0].nj;
  a.ext[2] = s->hblocks[0].nk;
  return a;
}

// End-of-step (or initial) dt policy.
cudaError_t enqueue_policy(aph_stepper s, bool initial, cudaStream_t st) {
  if (s->d_members)
    k_members_policy<<<1, 256, 0, st>>>(s->d_ctl, s->d_members, s->nmembers, s->dev.cfl, initial);
  else if (initial)
    k_dt_initial<<<1, 1, 0, st>>>(s->d_ctl, s->dev.cfl);
  else
    k_dt_policy<<<1, 1, 0, st>>>(s->d_ctl, s->dev.cfl);
  return cudaGetLastError();
}

cudaError_t launch_one(aph_stepper s, const StageArgs &a, int recon, cudaStream_t st) {
  void *work = (char *)s->d_ctl + offsetof(StepCtl, work);
  cudaError_t e = cudaMemsetAsync(work, 0, sizeof(((StepCtl *)nullptr)->work), st);
  if (e != cudaSuccess) return e;
  if (s->params.exact)
    return aph_exact::launch_stage(a, recon, s->params.rsolver, s->grid, s->cfg.threads, s->smem,
                                   s->cooperative, s->cfg.reg_cap, st);
  return aph_fast::launch_stage(a, recon, s->params.rsolver, s->grid, s->cfg.threads, s->smem,
                                s->cooperative, s->cfg.reg_cap, st);
}

// Enqueue one full RK step (all stages + dt policy).
cudaError_t enqueue_step(aph_stepper s, cudaStream_t st) {
  const std::vector<Stage> stages = stages_of(s->integrator);
  for (size_t i = 0; i < stages.size(); ++i) {
    const bool last = i + 1 == stages.size();
    const int recon = (s->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : s->params.recon;
    StageArgs a = stage_args(s, (int)i, stages[i], last, false);
    cudaError_t e = launch_one(s, a, recon, st);
    if (e != cudaSuccess) return e;
  }
  return enqueue_policy(s, false, st);
}

aph_status build_graph(aph_stepper s) {
  destroy_graph(s);
  if (!s->cap) {
    cudaError_t e = cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "capture stream");
  }
  for (int attempt = 0;; ++attempt) {
    cudaError_t e = cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "begin capture");
    cudaError_t e2 = enqueue_step(s, s->cap);
    e = cudaStreamEndCapture(s->cap, &s->graph);
    if (e2 == cudaSuccess && e == cudaSuccess) break;
    if (s->graph) cudaGraphDestroy(s->graph);
    s->graph = nullptr;
    cudaGetLastError();
    // a cooperative launch that cannot be captured: capture a plain launch of the same
    // occupancy-sized grid (its barrier waits stay bounded)
    if (s->cooperative && attempt == 0) {
      s->cooperative = false;
      continue;
    }
    return cuda_fail(e2 != cudaSuccess ? e2 : e, "capture step");
  }
  cudaError_t e;
  e = cudaGraphInstantiate(&s->exec, s->graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(s->graph);
    s->graph = nullptr;
    return cuda_fail(e, "instantiate step graph");
  }
  return APH_OK;
}

aph_status initial_dt(aph_stepper s, cudaStream_t st) {
  StageArgs a = stage_args(s, 0, Stage{0, 1, 1}, false, true);
  cudaError_t e = launch_one(s, a, s->params.recon, st);
  if (e == cudaSuccess) e = enqueue_policy(s, true, st);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "initial dt");
}

aph_status read_ctl(aph_stepper s, StepCtl *out) {
  cudaError_t e = cudaMemcpy(out, s->d_ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "read stepper state");
  if (out->error) return fail(out->error, "device-side failure in the stage kernel (status %d)", out->error);
  if (out->nonfinite) return fail(APH_ERR_STATE, "an update produced a NaN or an infinity");
  return APH_OK;
}

void free_all(aph_stepper s) {
  destroy_graph(s);
  if (s->cap) cudaStreamDestroy(s->cap);
  cudaFree(s->d_blocks);
  cudaFree(s->d_u1);
  cudaFree(s->d_prim);
  cudaFree(s->d_gamma);
  cudaFree(s->d_du);
  cudaFree(s->d_eraw);
  cudaFree(s->d_efl);
  cudaFree(s->d_backup);
  cudaFree(s->d_flags);
  cudaFree(s->d_ctl);
  cudaFree(s->d_cell_items);
  for (int d = 0; d < 3; ++d) cudaFree(s->d_line_items[d]);
  cudaFree(s->d_fix_items);
  cudaFree(s->d_bflux);
  cudaFree(s->d_members);
  cudaFree(s->d_hist);
  cudaFree(s->d_tmaps);
}

// Packed interiors <-> the state: grid.y = block; element e of a block's nvar * nint
// interior values enumerates (var, k, j, i) in the packed order, so its packed index is
// nvar * ipre + e.  Host memory is read or written directly (pinned, mapped).
__global__ void k_interiors(const StepBlock *blocks, int ndim, int ng, int nvar, const double *src,
                            double *dst, int load) {
  const StepBlock &B = blocks[blockIdx.y];
  const int n0 = B.nx[0], n1 = B.nx[1], n2 = B.nx[2];
  const int sj = ndim >= 2 ? ng : 0, sk = ndim >= 3 ? ng : 0;
  const long long total = (long long)nvar * B.nint;
  const long long base = (long long)nvar * B.ipre;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long line = e / n0;
    const int i = (int)(e - line * n0);
    const int j = (int)(line % n1);
    const long long kv = line / n1;
    const int k = (int)(kv % n2), v = (int)(kv / n2);
    const long long g = (long long)v * B.ncell + ((long long)(k + sk) * B.nj + (j + sj)) * B.ni + (i + ng);
    if (load) B.u0[g] = src[base + e];
    else dst[base + e] = B.u0[g];
  }
}

__global__ void k_set_dt(StepCtl *c, MemberCtl *m, int n, const double *dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (!m) {
    if (i == 0) c->dt = dt[0];
    return;
  }
  if (i < n) {  // a member with dt 0 (past its end time) is skipped
    m[i].dt = dt[i];
    m[i].active = dt[i] > 0.0;
  }
}

// Whether the stage launch just run applied a floor in any block.
__global__ void k_or_flags(const unsigned long long *flags, int n, int *out) {
  const unsigned long long launch = flags[2 * n];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (launch != 0 && flags[2 * i] == launch) atomicOr(out, 1);
}

}  // namespace

__global__ void k_members_reset(MemberCtl *m, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    m[i].time = 0.0;
    m[i].dt = 0.0;
    m[i].ncycle = 0;
    m[i].active = 1;
    m[i].min_bits = ~0ULL;
  }
}

namespace aph {
size_t stepper_field_doubles(aph_stepper s) { return (size_t)s->dev.nvar * s->total_cells; }

// Forget the energies kept across the last step's floors: the state was replaced.
cudaError_t forget_floors(aph_stepper s, cudaStream_t st) {
  return cudaMemsetAsync(s->d_efl, 0xff, sizeof(double) * s->total_cells, st);
}

cudaError_t stepper_restart(aph_stepper s, cudaStream_t st) {
  k_ctl_init<<<1, 1, 0, st>>>(s->d_ctl, DBL_MAX, 0.0);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = forget_floors(s, st);
  if (e == cudaSuccess && s->d_members) {
    k_members_reset<<<(s->nmembers + 127) / 128, 128, 0, st>>>(s->d_members, s->nmembers);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && initial_dt(s, st) != APH_OK) e = cudaErrorUnknown;
  return e;
}

cudaError_t stepper_step_dt(aph_stepper s, const double *dt_dev, double *keep, int *floor_flag,
                            cudaStream_t st) {
  const std::vector<Stage> stages = stages_of(s->integrator);
  const int n = s->d_members ? s->nmembers : 1;
  k_set_dt<<<(n + 127) / 128, 128, 0, st>>>(s->d_ctl, s->d_members, n, dt_dev);
  cudaError_t e = cudaGetLastError();
  const size_t field = stepper_field_doubles(s);
  for (size_t i = 0; i < stages.size() && e == cudaSuccess; ++i) {
    const int recon = (s->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : s->params.recon;
    StageArgs a = stage_args(s, (int)i, stages[i], false, false);
    a.full_domain = keep ? 1 : 0;  // the kept primitives are read over the entire domain
    e = launch_one(s, a, recon, st);
    if (e == cudaSuccess && keep)
      e = cudaMemcpyAsync(keep + i * field, s->d_prim, field * sizeof(double), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && floor_flag) {
      k_or_flags<<<(s->dev.nblocks + 255) / 256, 256, 0, st>>>(s->d_flags, s->dev.nblocks, floor_flag);
      e = cudaGetLastError();
    }
  }
  return e;
}
}  // namespace aph

extern "C" {

aph_status aph_stepper_create(const aph_stepper_desc *desc, aph_stepper *out) {
  clear_error();
  if (!desc || !out) return fail(APH_ERR_INVALID, "NULL argument");
  *out = nullptr;
  if (aph_status st = validate_params(&desc->params)) return st;
  if (stages_of(desc->integrator).empty())
    return fail(APH_ERR_INVALID, "integrator %d not recognized", desc->integrator);
  if (desc->nblocks <= 0 || !desc->blocks) return fail(APH_ERR_INVALID, "no blocks");
  const int ndim = desc->params.ndim;
  const bool amr = desc->amr != nullptr;
  const int nvar = desc->params.nvar;
  if (amr) {
    if (ndim != 2) return fail(APH_ERR_UNSUPPORTED, "refined meshes are 2D");
    std::vector<AmrFaces> faces(desc->nblocks);
    std::vector<int> nxs(2 * desc->nblocks);
    for (int b = 0; b < desc->nblocks; ++b) {
      std::memcpy(&faces[b], &desc->amr[b], sizeof(AmrFaces));
      nxs[2 * b] = desc->blocks[b].nx[0];
      nxs[2 * b + 1] = desc->blocks[b].nx[1];
    }
    char msg[160];
    if (amr_check(desc->nblocks, faces.data(), (const int(*)[2])nxs.data(), desc->params.nghost,
                  msg, sizeof(msg)))
      return fail(APH_ERR_INVALID, "%s", msg);
    for (int f = 0; f < 4; ++f)
      if (desc->bc[f] < 0 || desc->bc[f] > 2)
        return fail(APH_ERR_INVALID, "boundary condition %d not recognized", desc->bc[f]);
  } else if ((long long)desc->nb[0] * desc->nb[1] * desc->nb[2] != desc->nblocks) {
    return fail(APH_ERR_INVALID, "nb product != nblocks");
  }
  const aph_ensemble *ens = desc->ensemble;
  std::vector<MemberCtl> members;
  if (ens) {
    if (!amr) return fail(APH_ERR_INVALID, "an ensemble needs face tables (desc.amr)");
    if (ens->nmembers < 1 || !ens->member || !ens->gm1)
      return fail(APH_ERR_INVALID, "ensemble: nmembers, member and gm1 are required");
    for (int b = 0; b < desc->nblocks; ++b) {
      const int m = ens->member[b];
      if (m < 0 || m >= ens->nmembers) return fail(APH_ERR_INVALID, "block %d: member %d out of range", b, m);
      for (int f = 0; f < 4; ++f) {
        if (desc->amr[b].face_kind[f] == APH_FACE_FINER || desc->amr[b].face_kind[f] == APH_FACE_COARSER)
          return fail(APH_ERR_UNSUPPORTED, "ensemble members are unrefined meshes");
        for (int n = 0; n < desc->amr[b].face_count[f]; ++n)
          if (ens->member[desc->amr[b].face_nbr[f][n]] != m)
            return fail(APH_ERR_INVALID, "block %d face %d: neighbour in another member", b, f);
      }
    }
    members.resize(ens->nmembers);
    for (int m = 0; m < ens->nmembers; ++m) {
      const double gm1 = ens->gm1[m];
      if (!(gm1 > 0.0) || !std::isfinite(gm1)) return fail(APH_ERR_INVALID, "member %d: gm1 must be > 0", m);
      PackDev g;
      std::memset(&g, 0, sizeof(g));
      g.gm1 = gm1;
      fill_gas_consts(g);
      MemberCtl &x = members[m];
      std::memset(&x, 0, sizeof(x));
      x.gm1 = g.gm1;
      x.igm1 = g.igm1;
      x.gamma = g.gamma;
      x.c2g = g.c2g;
      x.one_igm1 = g.one_igm1;
      x.hlle_k = g.hlle_k;
      x.hllc_k = g.hllc_k;
      const double t = ens->tlim && ens->tlim[m] > 0 ? ens->tlim[m] : desc->tlim;
      x.tlim = t > 0 ? t : DBL_MAX;
      x.min_bits = ~0ULL;
      x.active = 1;
    }
  }
  aph_stepper s = new aph_stepper_s();
  s->params = desc->params;
  s->integrator = desc->integrator;
  PackDev &p = s->dev;
  std::memset(&p, 0, sizeof(p));
  p.nblocks = desc->nblocks;
  p.ndim = ndim;
  p.ng = desc->params.nghost;
  p.nvar = nvar;
  p.gm1 = desc->params.gm1;
  p.dfloor = desc->params.dfloor;
  p.pfloor = desc->params.pfloor;
  p.cfl = desc->params.cfl;
  fill_gas_consts(p);
  p.amr = amr ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    if (!amr && d >= ndim && desc->nb[d] != 1) {
      delete s;
      return fail(APH_ERR_INVALID, "nb%d must be 1", d + 1);
    }
    p.nb[d] = desc->nb[d];
    p.bc[d][0] = desc->bc[2 * d];
    p.bc[d][1] = desc->bc[2 * d + 1];
    for (int k = 0; k < 2; ++k)
      if (p.bc[d][k] < APH_BC_PERIODIC || p.bc[d][k] > APH_BC_REFLECT) {
        delete s;
        return fail(APH_ERR_INVALID, "bc not recognized");
      }
  }
  s->hblocks.resize(p.nblocks);
  long long cells = 0, inter = 0;
  for (int b = 0; b < p.nblocks; ++b) {
    const aph_block &a = desc->blocks[b];
    StepBlock &B = s->hblocks[b];
    std::memset(&B, 0, sizeof(B));
    for (int d = 0; d < 3; ++d) {
      if (d < ndim ? a.nx[d] < 1 : a.nx[d] != 1) {
        delete s;
        return fail(APH_ERR_INVALID, "block %d: nx%d invalid", b, d + 1);
      }
      if (!amr && a.nx[d] != desc->blocks[0].nx[d]) {
        delete s;
        return fail(APH_ERR_UNSUPPORTED, "a block grid with ghost exchange needs equal blocks");
      }
      if (!(a.dx[d] > 0.0)) {
        delete s;
        return fail(APH_ERR_INVALID, "block %d: dx%d must be positive", b, d + 1);
      }
      B.nx[d] = a.nx[d];
      B.dx[d] = a.dx[d];
      p.max_nx[d] = std::max(p.max_nx[d], a.nx[d]);
    }
    if (!a.cons) {
      delete s;
      return fail(APH_ERR_INVALID, "block %d: cons is NULL", b);
    }
    B.u0 = a.cons;
    B.ni = a.nx[0] + 2 * p.ng;
    B.nj = ndim >= 2 ? a.nx[1] + 2 * p.ng : 1;
    B.nk = ndim >= 3 ? a.nx[2] + 2 * p.ng : 1;
    B.ncell = (long long)B.ni * B.nj * B.nk;
    B.nint = (long long)a.nx[0] * a.nx[1] * a.nx[2];
    if (ens) B.member = ens->member[b];
    if (amr) {
      static_assert(sizeof(AmrFaces) == sizeof(aph_amr_block), "face table layout");
      std::memcpy(&B.amr, &desc->amr[b], sizeof(AmrFaces));
    } else {
      B.loc[0] = b % p.nb[0];
      B.loc[1] = (b / p.nb[0]) % p.nb[1];
      B.loc[2] = b / (p.nb[0] * p.nb[1]);
    }
    cells += B.ncell;
    inter += B.nint;
  }
  if (!amr)
    for (int d = 0; d < 3; ++d) p.mesh_nx[d] = p.nb[d] * s->hblocks[0].nx[d];
  s->total_cells = cells;
  s->total_interior = inter;
  s->gravity = desc->use_gravity != 0;
  for (int d = 0; d < 3; ++d) s->grav[d] = desc->gravity[d];
  s->cfg.threads = 256;
  s->cfg.ctas_per_sm = 0;
  for (int d = 0; d < 3; ++d) {
    s->cfg.lines[d] = 0;
    s->cfg.order[d] = d + 1;
  }
  s->cfg.schedule = 0;
  s->cfg.use_graph = 1;
  s->cfg.reg_cap = 0;
  s->cfg.tma = 0;
  cudaError_t e = cudaSuccess;
  auto ck = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  ck(cudaMalloc(&s->d_u1, sizeof(double) * nvar * cells));
  ck(cudaMalloc(&s->d_prim, sizeof(double) * nvar * cells));
  ck(cudaMalloc(&s->d_gamma, sizeof(double) * 2 * cells));
  ck(cudaMalloc(&s->d_du, sizeof(double) * nvar * inter));
  ck(cudaMalloc(&s->d_eraw, sizeof(double) * cells));
  ck(cudaMalloc(&s->d_efl, sizeof(double) * cells));
  ck(cudaMalloc(&s->d_flags, sizeof(unsigned long long) * (2 * (size_t)p.nblocks + 1)));
  ck(cudaMalloc(&s->d_ctl, sizeof(StepCtl)));
  ck(cudaMalloc(&s->d_blocks, sizeof(StepBlock) * p.nblocks));
  if (ens) {
    s->nmembers = ens->nmembers;
    ck(cudaMalloc(&s->d_members, sizeof(MemberCtl) * members.size()));
    if (e == cudaSuccess)
      e = cudaMemcpy(s->d_members, members.data(), sizeof(MemberCtl) * members.size(), cudaMemcpyHostToDevice);
  }
  if (amr) {
    s->bflux_stride = nvar * std::max(p.max_nx[0], p.max_nx[1]);
    ck(cudaMalloc(&s->d_bflux, sizeof(double) * 4 * s->bflux_stride * p.nblocks));
    std::vector<int> fix;
    for (int b = 0; b < p.nblocks; ++b)
      for (int f = 0; f < 4; ++f)
        if (desc->amr[b].face_kind[f] == APH_FACE_FINER) {
          fix.push_back(b);
          break;
        }
    s->nfix_items = (int)fix.size();
    if (!fix.empty()) {
      ck(cudaMalloc(&s->d_fix_items, sizeof(int) * fix.size()));
      if (e == cudaSuccess)
        e = cudaMemcpy(s->d_fix_items, fix.data(), sizeof(int) * fix.size(), cudaMemcpyHostToDevice);
    }
  }
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    return cuda_fail(e, "stepper allocation");
  }
  long long oc = 0, oi = 0;
  for (int b = 0; b < p.nblocks; ++b) {
    StepBlock &B = s->hblocks[b];
    B.u1 = s->d_u1 + (size_t)nvar * oc;
    B.prim = s->d_prim + (size_t)nvar * oc;
    B.gamma = s->d_gamma + 2 * oc;
    B.du = s->d_du + (size_t)nvar * oi;
    B.eraw = s->d_eraw + oc;
    B.efl = s->d_efl + oc;
    B.ipre = oi;
    if (amr) B.bflux = s->d_bflux + (size_t)4 * s->bflux_stride * b;
    oc += B.ncell;
    oi += B.nint;
  }
  ck(cudaMemcpy(s->d_blocks, s->hblocks.data(), sizeof(StepBlock) * p.nblocks, cudaMemcpyHostToDevice));
  ck(cudaMemset(s->d_flags, 0, sizeof(unsigned long long) * (2 * (size_t)p.nblocks + 1)));
  ck(cudaMemset(s->d_efl, 0xff, sizeof(double) * cells));
  k_ctl_init<<<1, 1>>>(s->d_ctl, desc->tlim > 0 ? desc->tlim : DBL_MAX, desc->fixed_dt);
  ck(cudaGetLastError());
  if (e != cudaSuccess) {
    free_all(s);
    delete s;
    return cuda_fail(e, "stepper setup");
  }
  if (aph_status st = configure(s)) {
    free_all(s);
    delete s;
    return st;
  }
  aph_status st = initial_dt(s, 0);
  if (st == APH_OK) {
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) st = cuda_fail(e, "initial dt");
  }
  if (st == APH_OK) {
    StepCtl c;
    st = read_ctl(s, &c);
  }
  if (st) {
    free_all(s);
    delete s;
    return st;
  }
  *out = s;
  return APH_OK;
}

aph_status aph_stepper_destroy(aph_stepper s) {
  if (!s) return APH_OK;
  free_all(s);
  delete s;
  return APH_OK;
}

aph_status aph_stepper_step(aph_stepper s, int nsteps, void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "stepper is NULL");
  if (nsteps < 0) return fail(APH_ERR_INVALID, "nsteps < 0");
  cudaStream_t st = (cudaStream_t)stream;
  if (s->cfg.use_graph) {
    if (!s->exec) {
      if (aph_status r = build_graph(s)) return r;
    }
    for (int i = 0; i < nsteps; ++i) {
      cudaError_t e = cudaGraphLaunch(s->exec, st);
      if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    }
    return APH_OK;
  }
  for (int i = 0; i < nsteps; ++i) {
    cudaError_t e = enqueue_step(s, st);
    if (e != cudaSuccess) return cuda_fail(e, "stage launch");
  }
  return APH_OK;
}

static aph_status interiors(aph_stepper s, const double *src, double *dst, bool load, void *stream) {
  clear_error();
  if (!s || !(load ? (const void *)src : (const void *)dst)) return fail(APH_ERR_INVALID, "NULL argument");
  cudaStream_t st = (cudaStream_t)stream;
  const void *ptr = load ? (const void *)src : (const void *)dst;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, ptr);
  if (e != cudaSuccess) {
    cudaGetLastError();
    at.type = cudaMemoryTypeUnregistered;
  }
  const PackDev &p = s->dev;
  const int nv = p.nvar;
  if (at.type != cudaMemoryTypeUnregistered) {  // device, managed or pinned host memory
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (p.nblocks > 65535) return fail(APH_ERR_UNSUPPORTED, "more than 65535 blocks");
    const dim3 grid(std::max(1, (4 * sms + p.nblocks - 1) / p.nblocks), p.nblocks);
    k_interiors<<<grid, 256, 0, st>>>(s->d_blocks, p.ndim, p.ng, nv, src, dst, load ? 1 : 0);
    e = cudaGetLastError();
    return e == cudaSuccess ? APH_OK : cuda_fail(e, "interiors");
  }
  // pageable host memory: one 3D copy per block and variable
  for (const StepBlock &B : s->hblocks) {
    const int sj = p.ndim >= 2 ? p.ng : 0, sk = p.ndim >= 3 ? p.ng : 0;
    for (int v = 0; v < nv && e == cudaSuccess; ++v) {
      double *packed = const_cast<double *>(load ? src : dst) + (size_t)nv * B.ipre + (size_t)v * B.nint;
      double *state = B.u0 + (size_t)v * B.ncell;
      cudaMemcpy3DParms c;
      std::memset(&c, 0, sizeof(c));
      const cudaPitchedPtr pk = make_cudaPitchedPtr(packed, sizeof(double) * B.nx[0], B.nx[0], B.nx[1]);
      const cudaPitchedPtr sp = make_cudaPitchedPtr(state, sizeof(double) * B.ni, B.ni, B.nj);
      const cudaPos at_state = make_cudaPos(sizeof(double) * p.ng, sj, sk);
      c.extent = make_cudaExtent(sizeof(double) * B.nx[0], B.nx[1], B.nx[2]);
      if (load) {
        c.srcPtr = pk;
        c.dstPtr = sp;
        c.dstPos = at_state;
        c.kind = cudaMemcpyHostToDevice;
      } else {
        c.srcPtr = sp;
        c.srcPos = at_state;
        c.dstPtr = pk;
        c.kind = cudaMemcpyDeviceToHost;
      }
      e = cudaMemcpy3DAsync(&c, st);
    }
  }
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "interiors");
}

aph_status aph_stepper_load_interiors(aph_stepper s, const double *src, void *stream) {
  return interiors(s, src, nullptr, true, stream);
}

aph_status aph_stepper_store_interiors(aph_stepper s, double *dst, void *stream) {
  return interiors(s, nullptr, dst, false, stream);
}

aph_status aph_stepper_status(aph_stepper s, double *time, double *dt, int *ncycle, void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "stepper is NULL");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "stepper status");
  StepCtl c;
  aph_status st = read_ctl(s, &c);
  if (time) *time = c.time;
  if (dt) *dt = c.dt;
  if (ncycle) *ncycle = c.ncycle;
  return st;
}

aph_status aph_stepper_member_status(aph_stepper s, double *time, double *dt, int *ncycle,
                                     void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "stepper is NULL");
  if (!s->d_members) return fail(APH_ERR_INVALID, "the stepper has no ensemble");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  std::vector<MemberCtl> m(s->nmembers);
  if (e == cudaSuccess)
    e = cudaMemcpy(m.data(), s->d_members, sizeof(MemberCtl) * m.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "member status");
  for (int i = 0; i < s->nmembers; ++i) {
    if (time) time[i] = m[i].time;
    if (dt) dt[i] = m[i].dt;
    if (ncycle) ncycle[i] = m[i].ncycle;
  }
  StepCtl c;
  return read_ctl(s, &c);
}

aph_status aph_stepper_history(aph_stepper s, double out[2], void *stream) {
  clear_error();
  if (!s || !out) return fail(APH_ERR_INVALID, "NULL argument");
  int max_int = 0;
  for (const StepBlock &B : s->hblocks) max_int = std::max<int>(max_int, (int)B.nint);
  const size_t need = history_scratch_doubles(max_int, s->dev.nblocks);
  if (s->hist_len < need) {
    cudaFree(s->d_hist);
    s->d_hist = nullptr;
    s->hist_len = 0;
    cudaError_t e = cudaMalloc(&s->d_hist, need * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "history scratch");
    s->hist_len = need;
  }
  cudaStream_t st = (cudaStream_t)stream;
  double *res = s->d_hist + need - 2;
  cudaError_t e = launch_history_steps(s->dev, s->d_blocks, max_int, s->d_hist, need - 2, res, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, res, 2 * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "stepper history");
}

aph_status aph_stepper_set_clock(aph_stepper s, double time, double dt, int ncycle, void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "stepper is NULL");
  if (s->d_members) return fail(APH_ERR_UNSUPPORTED, "an ensemble keeps one clock per member");
  if (!(dt >= 0.0) || ncycle < 0) return fail(APH_ERR_INVALID, "dt and ncycle must be >= 0");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(st);
  StepCtl c;
  if (e == cudaSuccess) e = cudaMemcpy(&c, s->d_ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "set clock");
  c.time = time;
  c.dt = dt;
  c.ncycle = ncycle;
  c.min_bits = ~0ULL;
  e = cudaMemcpy(s->d_ctl, &c, sizeof(StepCtl), cudaMemcpyHostToDevice);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "set clock");
}

aph_status aph_stepper_get_config(aph_stepper s, aph_stepper_config *cfg) {
  clear_error();
  if (!s || !cfg) return fail(APH_ERR_INVALID, "NULL argument");
  *cfg = s->cfg;
  for (int d = 0; d < 3; ++d) cfg->lines[d] = d < s->dev.ndim ? s->T[d] : 0;
  return APH_OK;
}

aph_status aph_stepper_set_config(aph_stepper s, const aph_stepper_config *cfg) {
  clear_error();
  if (!s || !cfg) return fail(APH_ERR_INVALID, "NULL argument");
  if (cfg->threads < 64 || cfg->threads > 1024 || cfg->threads % 32)
    return fail(APH_ERR_INVALID, "threads must be a multiple of 32 in 64..1024");
  if (cfg->threads > 256) return fail(APH_ERR_UNSUPPORTED, "stage kernel is built for <= 256 threads");
  if (cfg->schedule < 0 || cfg->schedule > 2) return fail(APH_ERR_INVALID, "schedule not in 0..2");
  if (cfg->reg_cap < 0 || cfg->reg_cap > 1) return fail(APH_ERR_INVALID, "reg_cap not in 0..1");
  if (cfg->tma < 0 || cfg->tma > 1) return fail(APH_ERR_INVALID, "tma not in 0..1");
  int seen = 0;
  for (int d = 0; d < s->dev.ndim; ++d) {
    if (cfg->order[d] < 1 || cfg->order[d] > s->dev.ndim) return fail(APH_ERR_INVALID, "bad sweep order");
    seen |= 1 << cfg->order[d];
  }
  if (seen != ((1 << (s->dev.ndim + 1)) - 2)) return fail(APH_ERR_INVALID, "sweep order is not a permutation");
  if (s->params.exact)
    for (int d = 0; d < s->dev.ndim; ++d)
      if (cfg->order[d] != d + 1)
        return fail(APH_ERR_INVALID, "exact mode sums the directions in x, y, z order");
  aph_stepper_config old = s->cfg;
  s->cfg = *cfg;
  for (int d = s->dev.ndim; d < 3; ++d) s->cfg.order[d] = d + 1;
  if (aph_status st = configure(s)) {
    s->cfg = old;
    configure(s);
    return st;
  }
  return APH_OK;
}

// Run nsteps steps without the graph, timing every stage launch with CUDA events on the
// launching stream; stage_ms[i] gets the mean duration of stage i.
aph_status aph_stepper_profile(aph_stepper s, int nsteps, double *stage_ms, void *stream) {
  clear_error();
  if (!s || !stage_ms || nsteps < 1) return fail(APH_ERR_INVALID, "bad argument");
  cudaStream_t st = (cudaStream_t)stream;
  const std::vector<Stage> stages = stages_of(s->integrator);
  const int ns = (int)stages.size();
  std::vector<cudaEvent_t> ev(2 * ns * nsteps);
  for (auto &e : ev) cudaEventCreate(&e);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < nsteps && e == cudaSuccess; ++k) {
    for (int i = 0; i < ns && e == cudaSuccess; ++i) {
      const bool last = i + 1 == ns;
      const int recon = (s->integrator == APH_INTEGRATOR_VL2 && i == 0) ? APH_RECON_DC : s->params.recon;
      StageArgs a = stage_args(s, i, stages[i], last, false);
      void *work = (char *)s->d_ctl + offsetof(StepCtl, work);
      e = cudaMemsetAsync(work, 0, sizeof(((StepCtl *)nullptr)->work), st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2 * (k * ns + i)], st);
      if (e == cudaSuccess)
        e = s->params.exact ? aph_exact::launch_stage(a, recon, s->params.rsolver, s->grid, s->cfg.threads,
                                                      s->smem, s->cooperative, s->cfg.reg_cap, st)
                            : aph_fast::launch_stage(a, recon, s->params.rsolver, s->grid, s->cfg.threads,
                                                     s->smem, s->cooperative, s->cfg.reg_cap, st);
      if (e == cudaSuccess) e = cudaEventRecord(ev[2 * (k * ns + i) + 1], st);
    }
    if (e == cudaSuccess) e = enqueue_policy(s, false, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  for (int i = 0; i < ns; ++i) stage_ms[i] = 0.0;
  if (e == cudaSuccess)
    for (int k = 0; k < nsteps; ++k)
      for (int i = 0; i < ns; ++i) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev[2 * (k * ns + i)], ev[2 * (k * ns + i) + 1]);
        stage_ms[i] += ms / nsteps;
      }
  for (auto &x : ev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "stepper profile");
  StepCtl c;
  return read_ctl(s, &c);
}

// Time candidate configurations on a scratch copy of the state and keep the fastest.
aph_status aph_stepper_autotune(aph_stepper s, int trial_steps, aph_stepper_config *best,
                                double *best_ms) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "stepper is NULL");
  if (trial_steps < 1) trial_steps = 2;
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  // back up u0 of every block and the control block
  const int nv = s->dev.nvar;
  const size_t nbv = sizeof(double) * nv;
  const size_t ncells = (size_t)s->total_cells;
  if (!s->d_backup) {  // u0 of every block, then the energies kept across the step-end floors
    e = cudaMalloc(&s->d_backup, (nbv + 2 * sizeof(double)) * ncells);
    if (e != cudaSuccess) return cuda_fail(e, "autotune backup");
  }
  double *bk_eraw = s->d_backup + nv * ncells, *bk_efl = bk_eraw + ncells;
  StepCtl ctl_saved;
  e = cudaMemcpy(&ctl_saved, s->d_ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost);
  std::vector<MemberCtl> members_saved(s->nmembers);
  if (e == cudaSuccess && s->nmembers)
    e = cudaMemcpy(members_saved.data(), s->d_members, sizeof(MemberCtl) * s->nmembers,
                   cudaMemcpyDeviceToHost);
  long long off = 0;
  for (const StepBlock &B : s->hblocks) {
    if (e == cudaSuccess) e = cudaMemcpy(s->d_backup + nv * off, B.u0, nbv * B.ncell, cudaMemcpyDeviceToDevice);
    off += B.ncell;
  }
  if (e == cudaSuccess) e = cudaMemcpy(bk_eraw, s->d_eraw, sizeof(double) * ncells, cudaMemcpyDeviceToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(bk_efl, s->d_efl, sizeof(double) * ncells, cudaMemcpyDeviceToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "autotune backup");
  auto restore = [&]() {
    long long o = 0;
    for (const StepBlock &B : s->hblocks) {
      cudaMemcpy(B.u0, s->d_backup + nv * o, nbv * B.ncell, cudaMemcpyDeviceToDevice);
      o += B.ncell;
    }
    cudaMemcpy(s->d_eraw, bk_eraw, sizeof(double) * ncells, cudaMemcpyDeviceToDevice);
    cudaMemcpy(s->d_efl, bk_efl, sizeof(double) * ncells, cudaMemcpyDeviceToDevice);
    cudaMemcpy(s->d_ctl, &ctl_saved, sizeof(StepCtl), cudaMemcpyHostToDevice);
    if (s->nmembers)
      cudaMemcpy(s->d_members, members_saved.data(), sizeof(MemberCtl) * s->nmembers,
                 cudaMemcpyHostToDevice);
  };
  const aph_stepper_config base = s->cfg;
  const int ndim = s->dev.ndim;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best_t = 1e300;
  aph_stepper_config best_c = base;
  std::vector<std::pair<double, aph_stepper_config>> timed;  // every candidate that ran
  auto time_one = [&](const aph_stepper_config &c, int steps, double &per) {
    if (aph_stepper_set_config(s, &c) != APH_OK) return false;
    restore();
    if (aph_stepper_step(s, 1, 0) != APH_OK) return false;  // warm-up (and graph build)
    cudaEventRecord(e0, 0);
    if (aph_stepper_step(s, steps, 0) != APH_OK) return false;
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    StepCtl c2;
    if (read_ctl(s, &c2) != APH_OK) return false;
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    per = ms / steps;
    return true;
  };
  auto trial = [&](const std::vector<aph_stepper_config> &cands) {
    for (const aph_stepper_config &c : cands) {
      double per;
      if (!time_one(c, trial_steps, per)) continue;
      timed.emplace_back(per, c);
      if (per < best_t) {
        best_t = per;
        best_c = c;
      }
    }
  };
  // Launch shapes: for each CTA size, register budget and window staging, the line counts at
  // the upper edge of each residency level (the most lines per item that still fit that many
  // CTAs on an SM: more lines amortise a window's halo cells, more resident warps hide each
  // other's barriers and loop tails), keeping levels of at least 8 warps per SM.
  auto shapes = [&](int threads, int reg_cap, int tma, const aph_stepper_config &from) {
    std::vector<aph_stepper_config> out;
    int most = 1;
    for (int d = 0; d < ndim; ++d)
      for (const StepBlock &B : s->hblocks)
        most = std::max(most, d == 0 ? B.nx[1] * B.nx[2] : d == 1 ? B.nx[0] * B.nx[2] : B.nx[0] * B.nx[1]);
    most = std::min(most, 64);
    int prev_occ = 0, prev_T = 0, T_low_edge = 0;
    for (int T = tma ? 2 : 1; T <= most + 1; T += tma ? 2 : 1) {
      int occ = 0;
      if (T <= most) {
        const int lines[3] = {T, T, T};
        int Ts[3];
        const size_t smem = stage_lines(s, lines, tma != 0, Ts);
        if (smem <= 220 * 1024 && !(tma && tma_unsupported(s, Ts)))
          occ = stage_residency(s, threads, reg_cap, smem);
      }
      if (occ != prev_occ && prev_occ > 0 && prev_occ * threads >= 256) {
        // the edge, and the count below it (a pass item's loops end in a partly filled round
        // of warps, which a smaller count at the same residency may fill better)
        for (int Tc : {prev_T, prev_T - (tma ? 2 : 1)}) {
          if (Tc < 1 || (Tc != prev_T && Tc == T_low_edge)) continue;
          aph_stepper_config c = from;
          c.threads = threads;
          c.reg_cap = reg_cap;
          c.tma = tma;
          c.ctas_per_sm = 0;
          for (int d = 0; d < 3; ++d) c.lines[d] = d < ndim ? Tc : 0;
          out.push_back(c);
        }
        T_low_edge = prev_T;
      }
      if (occ == 0 && prev_occ > 0) break;
      prev_occ = occ;
      prev_T = T;
    }
    return out;
  };
  // first candidate set: launch shapes with plain loads, strided schedule, x-y-z order
  {
    aph_stepper_config c0 = base;
    c0.schedule = 0;
    c0.use_graph = 1;
    c0.tma = 0;
    for (int d = 0; d < 3; ++d) c0.order[d] = d + 1;
    std::vector<aph_stepper_config> cands;
    for (int threads : {128, 256})
      for (int rc : {0, 1})
        for (aph_stepper_config c : shapes(threads, rc, 0, c0)) {
          cands.push_back(c);  // strided, and the dynamic work counter (the pick can differ)
          c.schedule = 2;
          cands.push_back(c);
        }
    if (cands.empty()) cands.push_back(c0);
    trial(cands);
  }
  // second set: schedules and sweep orders (any order only in fast mode: exact mode keeps the
  // reference's x, y, z summation) around the best shape
  {
    std::vector<std::vector<int>> orders = {{1, 2, 3}};
    if (!s->params.exact && ndim == 2) orders.push_back({2, 1, 3});
    if (!s->params.exact && ndim == 3) {
      orders.push_back({3, 2, 1});
      orders.push_back({2, 3, 1});
    }
    const aph_stepper_config b = best_c;
    std::vector<aph_stepper_config> cands;
    for (int sched : {0, 1, 2})
      for (const auto &o : orders) {
        aph_stepper_config c = b;
        c.schedule = sched;
        for (int d = 0; d < 3; ++d) c.order[d] = o[d];
        if (sched != b.schedule || c.order[0] != b.order[0] || c.order[1] != b.order[1]) cands.push_back(c);
      }
    trial(cands);
  }
  // third set: TMA-staged windows (even line counts) with the best schedule and order; fast
  // mode only (exact mode reconstructs the gamma field, which the windows do not carry)
  if (!s->params.exact) {
    const aph_stepper_config b = best_c;
    std::vector<aph_stepper_config> cands;
    for (int threads : {128, 256})
      for (int rc : {0, 1}) {
        const auto v = shapes(threads, rc, 1, b);
        cands.insert(cands.end(), v.begin(), v.end());
      }
    trial(cands);
  }
  // the three fastest candidates timed again over twice the steps (candidates within a few
  // per cent of each other are otherwise picked by the noise of a short trial)
  std::stable_sort(timed.begin(), timed.end(),
                   [](const std::pair<double, aph_stepper_config> &x,
                      const std::pair<double, aph_stepper_config> &y) { return x.first < y.first; });
  if (timed.size() > 1) {
    best_t = 1e300;
    for (size_t i = 0; i < timed.size() && i < 3; ++i) {
      double per;
      if (!time_one(timed[i].second, 2 * trial_steps, per)) continue;
      if (per < best_t) {
        best_t = per;
        best_c = timed[i].second;
      }
    }
    if (best_t == 1e300) {  // none ran again: the first round's best
      best_t = timed[0].first;
      best_c = timed[0].second;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  aph_status st = aph_stepper_set_config(s, &best_c);
  restore();
  e = cudaDeviceSynchronize();
  if (e != cudaSuccess) return cuda_fail(e, "autotune");
  if (best) aph_stepper_get_config(s, best);
  if (best_ms) *best_ms = best_t;
  return st;
}

aph_status aph_stepper_stage(aph_stepper s, int stage, int flags, void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "NULL stepper");
  const std::vector<Stage> stages = stages_of(s->integrator);
  if (stage < 0 || stage >= (int)stages.size())
    return fail(APH_ERR_INVALID, "stage %d not in 0..%d", stage, (int)stages.size() - 1);
  if (flags & ~APH_STAGE_GHOSTS_GIVEN) return fail(APH_ERR_INVALID, "unknown flags 0x%x", flags);
  if ((flags & APH_STAGE_GHOSTS_GIVEN) && (s->d_members || s->dev.amr))
    return fail(APH_ERR_UNSUPPORTED, "caller-filled ghost cells need a uniform block grid");
  const bool last = stage + 1 == (int)stages.size();
  const int recon = (s->integrator == APH_INTEGRATOR_VL2 && stage == 0) ? APH_RECON_DC : s->params.recon;
  StageArgs a = stage_args(s, stage, stages[stage], last, false);
  a.ghosts_given = (flags & APH_STAGE_GHOSTS_GIVEN) ? 1 : 0;
  const cudaError_t e = launch_one(s, a, recon, (cudaStream_t)stream);
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "stepper stage");
}

aph_status aph_stepper_local_dt(aph_stepper s, double *estimate, void *stream) {
  clear_error();
  if (!s || !estimate) return fail(APH_ERR_INVALID, "NULL argument");
  if (s->d_members) return fail(APH_ERR_UNSUPPORTED, "ensembles keep a dt per member");
  StepCtl c;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaMemcpy(&c, s->d_ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "stepper local dt");
  if (c.error) return fail(c.error, "a stage's grid barrier gave up");
  const double m = c.min_bits == ~0ULL ? DBL_MAX : [&] {
    double x;
    std::memcpy(&x, &c.min_bits, sizeof(x));
    return x;
  }();
  *estimate = s->dev.cfl * m;
  return APH_OK;
}

aph_status aph_stepper_end_step(aph_stepper s, double estimate, void *stream) {
  clear_error();
  if (!s) return fail(APH_ERR_INVALID, "NULL stepper");
  if (s->d_members) return fail(APH_ERR_UNSUPPORTED, "ensembles keep a dt per member");
  if (!(estimate > 0.0)) return fail(APH_ERR_INVALID, "the dt estimate must be positive");
  k_dt_policy<<<1, 1, 0, (cudaStream_t)stream>>>(s->d_ctl, s->dev.cfl, estimate);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? APH_OK : cuda_fail(e, "stepper end step");
}

aph_status aph_diag_barrier_timeout(double timeout_s, void *stream) {
  clear_error();
  if (!(timeout_s > 0.0) || timeout_s > 10.0) return fail(APH_ERR_INVALID, "timeout must be in (0, 10] s");
  StepCtl *ctl = nullptr;
  cudaError_t e = cudaMalloc(&ctl, sizeof(StepCtl));
  if (e != cudaSuccess) return cuda_fail(e, "barrier probe");
  cudaStream_t st = (cudaStream_t)stream;
  k_ctl_init<<<1, 1, 0, st>>>(ctl, DBL_MAX, 0.0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = aph_fast::launch_barrier_probe(ctl, (unsigned long long)(timeout_s * 1e9), st);
  StepCtl c;
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemcpy(&c, ctl, sizeof(StepCtl), cudaMemcpyDeviceToHost);
  cudaFree(ctl);
  if (e != cudaSuccess) return cuda_fail(e, "barrier probe");
  if (c.error) return fail(c.error, "the probe's grid barrier gave up after %.3f s", timeout_s);
  return APH_OK;
}

}  // extern "C"
