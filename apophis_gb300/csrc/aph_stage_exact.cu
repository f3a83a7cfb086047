// Batched stage kernel, exact arithmetic mode (built with --fmad=false).
#define APH_EXACT 1
#define APH_NS aph_exact
#include "aph_stage.cuh"
