// Fast arithmetic mode: fused multiply-adds, shared reciprocals, rsqrt-based sound speed.
#define APH_EXACT 0
#define APH_NS aph_fast
#include "aph_kernels.cuh"
