// aph_capi_internal.h -- helpers shared by the C-ABI translation units.
#pragma once
#include <cstdarg>
#include <vector>

#include "../../include/aph_hydro.h"
#include "aph_internal.h"

namespace aph {
aph_status fail(aph_status code, const char *fmt, ...);
aph_status cuda_fail(cudaError_t e, const char *where);
void clear_error();
const char *last_error();
void fill_gas_consts(PackDev &p);
aph_status validate_params(const aph_hydro_params *params);

const BlockDev *pack_blocks(aph_pack p);
const PackDev &pack_dev(aph_pack p);
int pack_max_interior(aph_pack p);
int pack_max_ncell(aph_pack p);
const aph_hydro_params &pack_params(aph_pack p);
const std::vector<BlockDev> &pack_host_blocks(aph_pack p);
bool pack_has_topology(aph_pack p);

// Adjoint support (aph_stepper.cu).  One RK step of the stepper's state with the per-member
// dt dt_dev (a device array of nmembers doubles, or of one without an ensemble), without the
// graph and without advancing the clock.  keep (if non-null) receives the primitives of
// every stage input over the entire domain, stepper_field_doubles(s) doubles per stage, in
// block order; a floor fired in any stage is OR-ed into *floor_flag (if non-null).
cudaError_t stepper_step_dt(aph_stepper s, const double *dt_dev, double *keep, int *floor_flag,
                            cudaStream_t st);
size_t stepper_field_doubles(aph_stepper s);
// Clock back to zero (no end time, CFL dt policy) and the initial dt of the current state.
cudaError_t stepper_restart(aph_stepper s, cudaStream_t st);

// History sums (aph_history.cu): out_dev[0] total mass, out_dev[1] total energy; scratch
// needs history_scratch_doubles(max_interior, nblocks) doubles (the last two hold the result).
size_t history_scratch_doubles(int max_interior, int nblocks);
cudaError_t launch_history(const PackDev &p, const BlockDev *blocks, int max_interior, double *scratch,
                           size_t scratch_len, double *out_dev, cudaStream_t s);
cudaError_t launch_history_steps(const PackDev &p, const StepBlock *blocks, int max_interior,
                                 double *scratch, size_t scratch_len, double *out_dev, cudaStream_t s);

// field: 0 cons, 1 u1
cudaError_t launch_fill_ghosts(const PackDev &p, const BlockDev *blocks, int max_ncell, int field,
                               cudaStream_t s);
}  // namespace aph
