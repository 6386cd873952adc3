// Mixed-precision instantiation of the force kernels (FP32 pair and three-body
// arithmetic; FP64 accumulation, reductions and normal-derivative assembly).
#define LMFF_REAL float
#define LMFF_NS f32
#define LMFF_PACKED_X2 1   // the FP32 unit: packed pair body, j records
#include "forces_impl.cuh"
