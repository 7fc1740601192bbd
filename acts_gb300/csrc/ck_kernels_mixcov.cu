// ck_kernels_mixcov.cu — instantiations of the mixed-precision fit kernel
// with an FP64 covariance: stepper, Jacobian transport and field
// interpolation in FP32; covariance transport, Kalman update, inverses and
// chi2 in FP64.
#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {

cudaError_t launchFitMixedCov64(const FitParams& fp, int variant, int grid, int block,
                                cudaStream_t st) {
  switch (variant) {
    case 0:
      fitKernel<float, double, 128, 1><<<grid, block, 0, st>>>(fp);
      break;
    case 1:
      fitKernel<float, double, 128, 3><<<grid, block, 0, st>>>(fp);
      break;
    default:
      fitKernel<float, double, 128, 4><<<grid, block, 0, st>>>(fp);
      break;
  }
  return cudaGetLastError();
}

int occupancyMixedCov64(int variant, int tpb) {
  int n = 0;
  switch (variant) {
    case 0:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, double, 128, 1>, tpb, 0);
      break;
    case 1:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, double, 128, 3>, tpb, 0);
      break;
    default:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, double, 128, 4>, tpb, 0);
      break;
  }
  return n;
}

}  // namespace ck
