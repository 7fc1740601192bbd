// ck_reverse_fp64.cu — reverse filtering in the plain FP64 form: the
// reversed filter pass (the 256-slot compaction kernel with reversed lanes,
// with and without the free-to-bound correction) and the output kernel that
// follows it (KalmanFitter::fit_impl, KalmanFitter.hpp:897-945).
#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {

cudaError_t launchReverseFP64(const FitParams& fp, int grid, cudaStream_t st) {
  if (fp.opt.freeToBoundCorrection)
    fitKernelCompact<double, double, 256, true, true>
        <<<grid, 256, compactSmemBytes<double, double, 256>(), st>>>(fp);
  else
    fitKernelCompact<double, double, 256, false, true>
        <<<grid, 256, compactSmemBytes<double, double, 256>(), st>>>(fp);
  return cudaGetLastError();
}

cudaError_t launchReverseOutputFP64(const FitParams& fp, cudaStream_t st) {
  const int grid = (fp.n_queue + kSmoothBlock - 1) / kSmoothBlock;
  reverseOutputKernel<double, kSmoothBlock><<<grid, kSmoothBlock, 0, st>>>(fp);
  return cudaGetLastError();
}

cudaError_t configureReverseFP64() {
  cudaError_t e = cudaFuncSetAttribute(fitKernelCompact<double, double, 256, true, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<double, double, 256>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fitKernelCompact<double, double, 256, false, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)compactSmemBytes<double, double, 256>());
}

}  // namespace ck
