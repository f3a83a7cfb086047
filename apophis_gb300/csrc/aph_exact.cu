// Exact arithmetic mode: the reference's operation order with one rounding per operation.
// Built with --fmad=false so that no multiply and add are fused.
#define APH_EXACT 1
#define APH_NS aph_exact
#include "aph_kernels.cuh"
