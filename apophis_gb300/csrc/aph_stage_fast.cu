// Batched stage kernel, fast arithmetic mode.
#define APH_EXACT 0
#define APH_NS aph_fast
#include "aph_stage.cuh"
