// FP32 instantiation of the VL+CT kernels: storage and bulk arithmetic in
// float with FMA contraction; the internal-energy recovery and the energy
// floor / dual-energy sync in float-float (vlct_energy.cuh); FP64 only in the
// per-block timestep division and minimum and the conserved-total sums.
#define VLCT_REAL float
#include "vlct_kern_impl.cuh"
