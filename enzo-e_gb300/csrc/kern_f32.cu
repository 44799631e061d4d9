// FP32 instantiation of the VL+CT kernels (bulk arithmetic in float with FMA
// contraction; FP64 only in the energy recovery, the energy floor / sync and
// the timestep division).
#define VLCT_REAL float
#include "vlct_kern_impl.cuh"
