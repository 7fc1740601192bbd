// ck_reverse_mixed.cu — reverse filtering in the mixed-precision form: the
// reversed filter pass (the 256-slot compaction kernel with reversed lanes,
// with and without the free-to-bound correction) and the output kernel that
// follows it (KalmanFitter::fit_impl, KalmanFitter.hpp:897-945).
#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {

cudaError_t launchReverseMixed(const FitParams& fp, int grid, cudaStream_t st) {
  if (fp.opt.freeToBoundCorrection)
    fitKernelCompact<float, float, 256, true, true>
        <<<grid, 256, compactSmemBytes<float, float, 256>(), st>>>(fp);
  else
    fitKernelCompact<float, float, 256, false, true>
        <<<grid, 256, compactSmemBytes<float, float, 256>(), st>>>(fp);
  return cudaGetLastError();
}

cudaError_t launchReverseOutputMixed(const FitParams& fp, cudaStream_t st) {
  const int grid = (fp.n_queue + kSmoothBlock - 1) / kSmoothBlock;
  reverseOutputKernel<float, kSmoothBlock><<<grid, kSmoothBlock, 0, st>>>(fp);
  return cudaGetLastError();
}

cudaError_t configureReverseMixed() {
  cudaError_t e = cudaFuncSetAttribute(fitKernelCompact<float, float, 256, true, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<float, float, 256>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fitKernelCompact<float, float, 256, false, true>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)compactSmemBytes<float, float, 256>());
}

}  // namespace ck
