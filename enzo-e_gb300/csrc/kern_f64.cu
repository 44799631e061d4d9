// FP64 instantiation of the VL+CT kernels.  Built with --fmad=false so that
// every multiply and add rounds separately, as in the reference's CPU build.
#define VLCT_REAL double
#include "vlct_kern_impl.cuh"

namespace vlct {
cudaError_t launch_set_scalar(double* p, double v, cudaStream_t st) {
  set_scalar_kernel<<<1, 1, 0, st>>>(p, v);
  return cudaGetLastError();
}
}  // namespace vlct
