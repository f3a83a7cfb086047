/* aph_hydro.h -- C ABI of the GB300-native hydro flux path.
 *
 * The entry points replace the hydro package's device work in apophis: the
 * "prim"/"gamma" FillDerived callback, the CalculateFluxes task, Parthenon's
 * UpdateWithFluxDivergence and ApplyBoundaryConditions steps, the constant-g source
 * and the EstimateTimestep callback.  Memory is owned by the caller (device
 * pointers in plain structs), every call returns an aph_status, nothing throws,
 * and each call is asynchronous on the given CUDA stream unless stated otherwise.
 * Field layout is Parthenon's VariablePack: a meshblock field with nvar components
 * is (nvar, nk, nj, ni) doubles, i fastest, with nghost ghost cells on both sides
 * of every active dimension (nj = nk = 1 in 1D, nk = 1 in 2D).
 */
#ifndef APH_HYDRO_H_
#define APH_HYDRO_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int aph_status;
#define APH_OK 0
#define APH_ERR_INVALID 1      /* bad argument: null pointer, size, enum, ghost width */
#define APH_ERR_UNSUPPORTED 2  /* valid combination this build does not implement */
#define APH_ERR_CUDA 3         /* a CUDA runtime call failed */
#define APH_ERR_TIMEOUT 4      /* a bounded device-side wait gave up */
#define APH_ERR_STATE 5        /* non-finite or non-positive density/pressure detected */

/* Enumerations, numbered as src/main.hpp:32-53 */
#define APH_RECON_DC 1
#define APH_RECON_PLM 2
#define APH_RECON_PPM 3
#define APH_RSOLVER_NONE 1
#define APH_RSOLVER_HLLE 2
#define APH_RSOLVER_HLLC 3
#define APH_RSOLVER_LHLLC 4
#define APH_INTEGRATOR_RK1 1
#define APH_INTEGRATOR_RK2 2
#define APH_INTEGRATOR_RK3 3
#define APH_INTEGRATOR_VL2 4
/* Physical boundaries: Parthenon "periodic", "outflow" and apophis "reflecting"
 * (src/boundaries/apophis_boundaries.cpp:257-272) */
#define APH_BC_PERIODIC 0
#define APH_BC_OUTFLOW 1
#define APH_BC_REFLECT 2

/* One meshblock (Parthenon MeshBlockData of the "base" and "u1" registers). */
typedef struct aph_block {
  double *cons;    /* "cons" (hydro.cpp:199-202), nvar components */
  double *prim;    /* "prim" (hydro.cpp:223-225), nvar components */
  double *gamma;   /* "gamma" (hydro.cpp:251-257): gamma_c, gamma_e */
  double *u1;      /* "cons" of the u1 register (apophis_driver.cpp:45-54); may be NULL
                      for calls that do not read it */
  double *flux[3]; /* cons.flux(X1DIR..X3DIR), nvar components each, same shape as cons;
                      flux[d] at (n,k,j,i) is the face on the low side of cell (k,j,i) */
  int nx[3];       /* interior cells per dimension (1 for an unused dimension) */
  double dx[3];    /* cell widths; for an unused dimension the mesh extent along it */
  long long flux_stride[3][3]; /* strides in doubles of flux[d] over (n, k, j), i being
                      contiguous; all three 0: the shape of cons.  A flux array of its own
                      shape, e.g. Parthenon's face-centred (nvar, nk, nj, ni + 1) along x1,
                      passes its strides (element (n, k, j, i) at n*s[0] + k*s[1] + j*s[2] + i,
                      face i on the low side of cell i); each row must hold the faces of the
                      cons row (plus one along d), each plane its rows, each component its
                      planes */
  double *eos_lambda; /* "eos_lambda" (hydro.cpp:241-249), 3 components, the shape of cons;
                      may be NULL.  Only ConsToPrim touches it, as the reference's does for
                      the ideal gas: lT (component 2) becomes 7 where it is 0
                      (hydro.cpp:491-493) */
} aph_block;

/* Hydro package parameters (InitializeHydro, src/hydro/hydro.cpp:33-349). */
typedef struct aph_hydro_params {
  int ndim;        /* 1, 2 or 3 */
  int nghost;      /* parthenon/mesh/nghost */
  int nvar;        /* 5 + number of passive scalars */
  int recon;       /* hydro/reconstruction */
  int rsolver;     /* hydro/riemann */
  double gm1;      /* eos/gm1 of the ideal gas */
  double dfloor;   /* hydro/dfloor */
  double pfloor;   /* hydro/pfloor */
  double cfl;      /* parthenon/time/cfl */
  int exact;       /* 1: the reference's operation order, one rounding per operation
                      (bit-identical to its FP64 CPU path); 0: fused multiply-adds and
                      shared reciprocals (about 1e-15 relative per operation) */
} aph_hydro_params;

/* Neighbours of one meshblock of a statically refined 2D mesh.  Levels differ by at most
 * one across a face; periodic faces name the wrapped neighbour.  The Parthenon counterpart
 * is the mesh's neighbour-block list used by its boundary communication. */
#define APH_FACE_SAME 0      /* one neighbour on the same level */
#define APH_FACE_COARSER 1   /* one neighbour one level coarser */
#define APH_FACE_FINER 2     /* the neighbours one level finer that cover the face */
#define APH_FACE_BOUNDARY 3  /* physical outflow / reflecting boundary */
typedef struct aph_amr_block {
  int level;           /* 0 = base level; cell width is the base width / 2^level */
  int origin[2];       /* global index of the first interior cell, in cells of this level */
  int face_kind[4];    /* faces x-, x+, y-, y+ */
  int face_count[4];   /* neighbours across each face (up to 4 for APH_FACE_FINER) */
  int face_nbr[4][4];  /* neighbour block indices, in transverse order */
} aph_amr_block;

/* A pack: the device-resident descriptor of a list of meshblocks (MeshData). */
typedef struct aph_pack_s *aph_pack;

/* Text of the last error on the calling thread ("" when none). */
const char *aph_last_error(void);
int aph_version(void);

/* Describe nblocks meshblocks as one pack.  Uploads the descriptors to the device.
 * Blocks may differ in nx; ndim, nghost and nvar are shared. */
aph_status aph_pack_create(const aph_hydro_params *params, const aph_block *blocks, int nblocks,
                           aph_pack *out);
/* Blocks form a uniform nb[0] x nb[1] x nb[2] grid, numbered x-fastest, with the
 * physical boundaries bc[2*d + side] (side 0 inner, 1 outer); needed by
 * aph_hydro_fill_ghosts. */
aph_status aph_pack_set_topology(aph_pack pack, const int nb[3], const int bc[6]);
/* Blocks form a statically refined 2D mesh (ndim 2; passive scalars allowed): ghost fill uses
 * the face tables (copy, 2x2 restriction, minmod-linear prolongation) and the flux-divergence
 * update corrects coarse cells at coarse-fine faces to the mean of the fine face fluxes (the
 * flux-correction tasks of apophis_driver.cpp:68, 74-76). bc as in aph_pack_set_topology. */
aph_status aph_pack_set_amr(aph_pack pack, const aph_amr_block *amr, const int bc[6]);
/* Host-only check of a refined mesh's face tables against the blocks' interior sizes
 * nx[2*b], nx[2*b+1] (the check aph_pack_set_amr and aph_stepper_create run): kinds and
 * counts in range, neighbours on the stated level and covering the whole face, coarse-fine
 * faces on even cell boundaries, at least 2*nghost cells per side.  No device work. */
aph_status aph_amr_check(const aph_amr_block *amr, const int *nx, int nblocks, int nghost);
/* A partition of a pack: blocks first..first+count-1, sharing the parent's descriptors (and
 * so its neighbours), for launches over part of a pack (one meshblock at a time, or one of
 * Parthenon's pack partitions).  Destroy it before the parent. */
aph_status aph_pack_partition(aph_pack parent, int first, int count, aph_pack *out);
aph_status aph_pack_destroy(aph_pack pack);

/* ConsToPrim<EOS_t> (src/hydro/hydro.cpp:422-533), the FillDerivedMesh callback:
 * over the entire domain of each block, apply the density and pressure floors to
 * cons in place and write prim and gamma. */
aph_status aph_hydro_cons_to_prim(aph_pack pack, void *stream);

/* CalculateFluxes<euler, recon, rsolver> (src/hydro/hydro.cpp:535-744), the
 * flux_first_stage / flux_other_stage task (apophis_driver.cpp:70-72): reconstruct
 * prim and gamma, solve the Riemann problem on every face of the interior and write
 * cons.flux.  recon and rsolver are the template arguments of the FluxFun_t. */
aph_status aph_hydro_calculate_fluxes(aph_pack pack, int recon, int rsolver, void *stream);

/* Parthenon Update::UpdateWithFluxDivergence (called at apophis_driver.cpp:79-82):
 * cons = gam0*cons + gam1*u1 + beta_dt*(-div F) on the interior.  The _dev variant
 * takes beta_dt = beta * (*dt_dev) from device memory (for graph replay). */
aph_status aph_hydro_update_with_flux_divergence(aph_pack pack, double gam0, double gam1,
                                                 double beta_dt, void *stream);
aph_status aph_hydro_update_with_flux_divergence_dev(aph_pack pack, double gam0, double gam1,
                                                     double beta, const double *dt_dev,
                                                     void *stream);

/* EstimateTimestep<euler> (src/hydro/hydro.cpp:351-420), the EstimateTimestepMesh
 * callback: cfl * min over interior cells of dx_d / (|v_d| + lambda).  The blocking
 * form returns the value on the host; the _async form writes it to *dt_dev. */
aph_status aph_hydro_estimate_timestep(aph_pack pack, double *dt_host, void *stream);
aph_status aph_hydro_estimate_timestep_async(aph_pack pack, double *dt_dev, void *stream);

/* EstimateTimestep of one meshblock that allocates no memory at all.  This entry point
 * has no counterpart in the reference.  It is for callers that must not allocate device
 * memory when they ask for a timestep: a host code whose pool allocator has taken the
 * device memory up front (a Kokkos or Parthenon application sized to the GPU) has none
 * left for cudaMalloc, and cudaMalloc / cudaFree inside its step would synchronise the
 * device.  prim and cons are the block's fields as above; the result, cfl * min, goes to
 * *dt_dev, asynchronously on stream.  Its scratch is a fixed device array inside the
 * library, one per GPU for the life of the process, sized for at most
 * APH_NOALLOC_MAX_CELLS interior cells; larger blocks are rejected with APH_ERR_INVALID.
 * The first call on a device looks up that array's device address (again after the
 * device's context was replaced, e.g. by cudaDeviceReset), so make the first call before
 * any stream capture.  Every call overwrites the array, which keeps the last call's
 * partial minima; two calls that overlap on the GPU (different streams, no ordering
 * between them) race and must not be issued. */
#define APH_NOALLOC_MAX_CELLS 1048576
aph_status aph_hydro_estimate_timestep_noalloc(const double *prim, const double *cons,
                                               const int nx[3], int nghost, int ndim,
                                               const double dx[3], double gm1, double cfl,
                                               double *dt_dev, void *stream);

/* ApplyGravity for a constant field g (src/gravity/gravity.cpp:374-410) with the
 * stage's beta*dt; uses prim of the previous FillDerived as the reference does. */
/* History sums GlobalQuantHst<Sum, IDN> and <Sum, IEN> (src/hydro/hydro.cpp:336-346,
 * 754-771), the hydro package's history outputs total_mass and total_energy: the sum over
 * interior cells of cons * CellVolume; out[0] mass, out[1] energy (blocking).  Reduced in a
 * fixed order, so repeated calls on the same state agree bit for bit. */
aph_status aph_hydro_history(aph_pack pack, double out[2], void *stream);

aph_status aph_hydro_apply_gravity(aph_pack pack, const double g[3], double beta_dt,
                                   void *stream);

/* Boundary exchange plus ApplyBoundaryConditions (apophis_driver.cpp:94-104) on a
 * uniform block grid (aph_pack_set_topology): every ghost cell of cons takes the value
 * of the interior cell its periodic / outflow / reflecting image points to; the
 * reflecting image negates the normal momentum (apophis_boundaries.cpp:210-221). */
aph_status aph_hydro_fill_ghosts(aph_pack pack, void *stream);

/* ---- batched path ----------------------------------------------------------------
 * A stepper advances a whole pack by full RK steps (the MultiStageDriver cycle with the
 * stage order of ApophisDriver::MakeTaskCollection, apophis_driver.cpp:27-129): each
 * stage is one persistent launch over every meshblock (ghost fill, ConsToPrim, the
 * x/y/z flux passes, the update, gravity and, at the last stage, the dt reduction);
 * dt and time stay on the device; a step is captured once as a CUDA graph and replayed.
 * The state is the caller's cons (u0): its interior cells; the stepper owns u1 and its
 * scratch.  Ghost cells of cons are scratch too: a stage forms the ghost values it reads (a
 * ghost that copies an interior cell is read at that cell and not written), so between steps
 * they hold no defined values.  The floors of the last FillDerived of a step are applied at
 * the start of the next stage, so cons between steps holds the update's raw values. */
typedef struct aph_stepper_s *aph_stepper;

/* A batch of independent problems (an ensemble) stepped together in one pack: block b belongs
 * to member member[b]; each member has its own adiabatic index (gm1) and advances with its
 * own CFL dt and clock to its own end time.  Members must not neighbour one another in the
 * face tables (aph_stepper_desc.amr, required: each member is its own mesh, e.g. a periodic
 * box).  No counterpart in the reference, which runs one problem per executable. */
typedef struct aph_ensemble {
  int nmembers;
  const int *member;   /* per block, 0..nmembers-1 */
  const double *gm1;   /* per member: gamma - 1 (> 0) */
  const double *tlim;  /* per member: end time; NULL or <= 0: the desc's tlim */
} aph_ensemble;

typedef struct aph_stepper_desc {
  aph_hydro_params params;   /* nvar must be 5 */
  int integrator;            /* APH_INTEGRATOR_* (parthenon/time/integrator) */
  int nblocks;
  const aph_block *blocks;   /* cons (state, ghosts included), nx, dx; other fields unused */
  int nb[3];                 /* uniform block grid, blocks numbered x-fastest */
  int bc[6];                 /* physical boundaries, as in aph_pack_set_topology */
  int use_gravity;           /* 1: constant-g source after each update */
  double gravity[3];
  double tlim;               /* parthenon/time/tlim; <= 0: none */
  double fixed_dt;           /* > 0: every step uses this dt instead of the CFL policy */
  const aph_amr_block *amr;  /* NULL: uniform block grid (nb); else the refined 2D mesh */
  const aph_ensemble *ensemble;  /* NULL: one problem; else the batch (needs amr face tables) */
} aph_stepper_desc;

/* Launch configuration, chosen by aph_stepper_autotune or set by hand. */
typedef struct aph_stepper_config {
  int threads;      /* CTA size (64..256, multiple of 32) */
  int ctas_per_sm;  /* resident CTAs per SM; 0: as many as fit */
  int lines[3];     /* lines per work item of each direction's pass; 0: automatic */
  int order[3];     /* sweep order (1-based directions); x, y, z in exact mode */
  int schedule;     /* 0 strided, 1 contiguous ranges, 2 dynamic work counter */
  int use_graph;    /* 1: replay the captured step graph */
  int reg_cap;      /* 1: the stage kernel built for three 256-thread CTAs per SM (about 80
                       registers per thread); 0: registers as needed (two CTAs) */
  int tma;          /* 1: stage each pass item's prim window with one tensor copy (TMA) when
                       the blocks are equal, rows even, nghost even and the lines per item
                       even and dividing a plane; 0: plain loads */
} aph_stepper_config;

/* Allocate the stepper's scratch, run the initial FillDerived + EstimateTimestep
 * (blocking) and set dt_0. */
aph_status aph_stepper_create(const aph_stepper_desc *desc, aph_stepper *out);
aph_status aph_stepper_destroy(aph_stepper stepper);
/* Enqueue nsteps full RK steps on stream (asynchronous). */
aph_status aph_stepper_step(aph_stepper stepper, int nsteps, void *stream);
/* Synchronise stream and report time, the dt of the next step and the cycle count;
 * returns APH_ERR_TIMEOUT if a stage's grid barrier gave up. */
aph_status aph_stepper_status(aph_stepper stepper, double *time, double *dt, int *ncycle,
                              void *stream);
/* Ensembles: per member (arrays of nmembers) time, the dt of its next step (0 once it has
 * reached its end time) and cycle count.  aph_stepper_status then reports the earliest
 * member time, the largest next dt and the largest cycle count. */
aph_status aph_stepper_member_status(aph_stepper stepper, double *time, double *dt, int *ncycle,
                                     void *stream);
/* Resume: set the clock (time, dt of the next step, cycle count) of a stepper created from a
 * saved state (no ensemble). */
aph_status aph_stepper_set_clock(aph_stepper stepper, double time, double dt, int ncycle,
                                 void *stream);
/* The history sums of the stepper's state (as aph_hydro_history, over all blocks). */
aph_status aph_stepper_history(aph_stepper stepper, double out[2], void *stream);
/* The interiors of the stepper's state as one packed array: block after block, each block's
 * (nvar, nx3, nx2, nx1) interior cells (no ghost cells: a step refills them).  The array may
 * be device memory or pinned host memory (cudaHostAlloc / cudaHostRegister), which one kernel
 * reads or writes across the host link directly; other host memory is copied with one 3D copy
 * per block and variable.  Asynchronous on stream.  No counterpart in the reference, whose
 * state stays in Parthenon's per-block arrays; this is the host interface of a resident pack
 * (a host code that keeps its state in host memory loads it before and stores it after each
 * step or run). */
aph_status aph_stepper_load_interiors(aph_stepper stepper, const double *src, void *stream);
aph_status aph_stepper_store_interiors(aph_stepper stepper, double *dst, void *stream);
/* Sharded packs (one rank's blocks of a larger uniform grid; the reference's MPI driver,
 * apophis_driver.cpp:68-104, exchanges their ghost zones and reduces dt across ranks):
 * a step driven stage by stage.  aph_stepper_stage enqueues stage `stage` (0-based) of the
 * current step with the stepper's dt; with APH_STAGE_GHOSTS_GIVEN the caller has filled every
 * ghost cell of the state (a halo exchange) and the stage's own ghost fill is skipped (uniform
 * block grids only).  After the last stage, aph_stepper_local_dt returns (blocking) this
 * pack's estimate cfl * min over its interior cells of the new state, and
 * aph_stepper_end_step applies the dt policy (time += dt; dt = min(2 dt, estimate), clipped at
 * tlim) with the caller's estimate, the minimum over all ranks.  Stage by stage without the
 * flag and with this pack's own estimate is exactly aph_stepper_step. */
#define APH_STAGE_GHOSTS_GIVEN 1
aph_status aph_stepper_stage(aph_stepper stepper, int stage, int flags, void *stream);
aph_status aph_stepper_local_dt(aph_stepper stepper, double *estimate, void *stream);
aph_status aph_stepper_end_step(aph_stepper stepper, double estimate, void *stream);
aph_status aph_stepper_get_config(aph_stepper stepper, aph_stepper_config *cfg);
aph_status aph_stepper_set_config(aph_stepper stepper, const aph_stepper_config *cfg);
/* Advance nsteps steps without the graph, timing each stage launch with CUDA events on
 * stream; stage_ms[i] receives the mean duration of stage i (blocking). */
aph_status aph_stepper_profile(aph_stepper stepper, int nsteps, double *stage_ms, void *stream);
/* Time a built-in candidate set of configurations for trial_steps steps each on a copy
 * of the state (the state and clock are restored) and keep the fastest. */
aph_status aph_stepper_autotune(aph_stepper stepper, int trial_steps, aph_stepper_config *best,
                                double *best_ms);

/* Failure-path probe (no counterpart in the reference): a one-CTA launch whose grid barrier
 * waits for a CTA that does not exist.  The wait gives up after timeout_s (<= 10) and the call
 * returns APH_ERR_TIMEOUT, the status every persistent stage launch reports when a barrier
 * runs out; the context stays usable.  Stepper status calls also return APH_ERR_STATE once an
 * update has produced a NaN or an infinity. */
aph_status aph_diag_barrier_timeout(double timeout_s, void *stream);

/* Test probe (no counterpart in the reference): evaluates on the device, for the n device
 * values x, the integer-pipe operations the exact arithmetic mode uses on tame operands
 * (op 0: x / 6.0 by the exact remainder, 1: 0.5 * x, 2: 2.0 * x as exponent steps, 3: 1.0 if
 * x is tame, else 0.0) into out, so that tests can compare them bit for bit with the IEEE
 * operations they stand for.  Asynchronous on stream. */
aph_status aph_diag_exact_ops(int op, const double *x, double *out, long long n, void *stream);
/* The same for the integer-pipe IEEE additions and small multiplications: op 0: x + y,
 * 1: x - y, 2: 3 * x, 3: 6 * x, 4: 1.25 * x (y unused by ops 2-4), for operands zero or normal
 * with 2^-900 < |x| < 2^900; and for the FP64 pipe's operations they are weighed against:
 * 5: x / y, 6: the reciprocal 1 / y, 7: sqrt(x), 8: x / y from the reciprocal of y (Markstein's
 * correction, for x and y tame). */
aph_status aph_diag_exact_ops2(int op, const double *x, const double *y, double *out, long long n,
                               void *stream);

/* ---- adjoint of the step --------------------------------------------------------------
 * Hand-written reverse mode of the full fixed-dt step: ConsToPrim, the PPM, PLM or
 * donor-cell limiters (each branch's transposed linear map; the quotient rule for PPM's
 * extremum ratio), the HLLE / HLLC fluxes with their wave-speed and contact branches, the
 * flux divergence, the RK stage combination and the ghost map.  No counterpart in the
 * reference (which has no derivatives); it differentiates the step the batched stepper
 * takes (its forward runs on an internal stepper).  All state arguments are device arrays
 * in pack layout: nblocks consecutive meshblocks of (5, nk, nj, ni) doubles (blocks of equal
 * size), ghost entries ignored on input and zero in adjoint outputs.  The pack is described
 * by an aph_stepper_desc (its cons pointers are not used: the adjoint owns its buffers),
 * uniform grids or face tables without coarse-fine faces, ensembles included; hlle or hllc,
 * no gravity, nvar 5, fast arithmetic. */
typedef struct aph_adjoint_s *aph_adjoint;
aph_status aph_adjoint_create(const aph_stepper_desc *desc, aph_adjoint *out);
aph_status aph_adjoint_destroy(aph_adjoint adjoint);
/* One RK step with fixed dt: u_next = step(u_n) (the forward the adjoint linearises). */
aph_status aph_adjoint_step(aph_adjoint adjoint, const double *u_n, double dt, double *u_next,
                            void *stream);
/* Vector-Jacobian product of one step: lam_n = (dU^{n+1}/dU^n)^T lam_next (lam_n may alias
 * lam_next).  Returns APH_ERR_STATE if a floor fired in the step. */
aph_status aph_adjoint_step_vjp(aph_adjoint adjoint, const double *u_n, double dt,
                                const double *lam_next, double *lam_n, void *stream);
/* Rollout of nsteps steps with the fixed dt schedule dts[] (host array) from u0, keeping a
 * checkpoint every checkpoint_every steps on the device; writes the final state.  Also sizes
 * the reverse sweep's segment storage (checkpoint_every steps of stage-input primitives),
 * so that aph_adjoint_backward allocates nothing. */
aph_status aph_adjoint_forward(aph_adjoint adjoint, const double *u0, int nsteps, const double *dts,
                               int checkpoint_every, double *u_final, void *stream);
/* The same with a dt per member and step: dts[k * nmembers + m] (one member without an
 * ensemble); aph_adjoint_forward uses dts[k] for every member. */
aph_status aph_adjoint_forward_members(aph_adjoint adjoint, const double *u0, int nsteps,
                                       const double *dts, int checkpoint_every, double *u_final,
                                       void *stream);
/* Pick the launch configuration of the adjoint's forward (its internal stepper) by timing
 * it on the state u (as aph_stepper_autotune; blocking). */
aph_status aph_adjoint_autotune(aph_adjoint adjoint, const double *u, void *stream);
/* Reverse sweep of the last rollout: recompute each segment from its checkpoint, then the
 * step VJPs backwards; lam_initial = (dU^N/dU^0)^T lam_final (blocking). */
aph_status aph_adjoint_backward(aph_adjoint adjoint, const double *lam_final, double *lam_initial,
                                void *stream);

#ifdef __cplusplus
}
#endif

#endif /* APH_HYDRO_H_ */
