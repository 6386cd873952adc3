// FP64 instantiation of the force kernels (the all-FP64 drop-in).
#define LMFF_REAL double
#define LMFF_NS f64
#include "forces_impl.cuh"
