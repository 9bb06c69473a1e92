// The fused mixed kernel of cross-sections from 33 to 48 (tiles of 64,
// S = 2; blocks up to 32 take the warp engine of negf_mixed.cu): its own
// translation unit so that it compiles in parallel with the rest.
#define PF_FUSED_S 2
#include "negf_fused.cuh"
