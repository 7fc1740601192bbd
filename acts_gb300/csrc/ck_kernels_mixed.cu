// ck_kernels_mixed.cu — instantiations of the mixed-precision fit kernel:
// Runge-Kutta stages, Jacobian transport, field interpolation and covariance
// transport in FP32, with the free parameters accumulated in FP64 from the
// FP32 stage increments; the Kalman update (gain, 2x2 inverse, covariance
// update, chi2) in FP32 on FP64 residuals; smoother-gain inverse and
// bound-parameter conversion in FP64.
#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {

cudaError_t launchFitMixed(const FitParams& fp, int variant, int grid, int block,
                           cudaStream_t st) {
  if (fp.opt.freeToBoundCorrection) {
    // the free-to-bound correction runs in its own instantiation of the
    // 256-slot compaction kernel (the caller sizes the grid for it)
    fitKernelCompact<float, float, 256, true>
        <<<grid, 256, compactSmemBytes<float, float, 256>(), st>>>(fp);
    return cudaGetLastError();
  }
  switch (variant) {
    case 0:
      fitKernel<float, float, 128, 1><<<grid, block, 0, st>>>(fp);
      break;
    case 1:
      fitKernel<float, float, 128, 3><<<grid, block, 0, st>>>(fp);
      break;
    case 2:
      fitKernel<float, float, 128, 4><<<grid, block, 0, st>>>(fp);
      break;
    case 3:
      fitKernelCompact<float, float, 256><<<grid, 256, compactSmemBytes<float, float, 256>(), st>>>(fp);
      break;
    case 5:
      fitKernelPool<float, float, 384, 256><<<grid, 256, poolSmemBytes<float, float, 384>(), st>>>(fp);
      break;
    case 6:
      fitKernelPool<float, float, 448, 256><<<grid, 256, poolSmemBytes<float, float, 448>(), st>>>(fp);
      break;
    default:
      fitKernelCompact<float, float, 128><<<grid, 128, compactSmemBytes<float, float, 128>(), st>>>(fp);
      break;
  }
  return cudaGetLastError();
}

cudaError_t configureMixed() {
  cudaError_t e = cudaFuncSetAttribute(smoothKernelStaged<float, kSmoothBlock>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)stagedSmoothSmemBytes<float, kSmoothBlock>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelPool<float, float, 384, 256>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)poolSmemBytes<float, float, 384>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelPool<float, float, 448, 256>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)poolSmemBytes<float, float, 448>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelCompact<float, float, 256, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<float, float, 256>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelCompact<float, float, 256>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<float, float, 256>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fitKernelCompact<float, float, 128>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)compactSmemBytes<float, float, 128>());
}

cudaError_t launchSmoothMixed(const FitParams& fp, cudaStream_t st) {
  const int grid = (fp.n_queue + kSmoothBlock - 1) / kSmoothBlock;
  if (fp.smooth_staged && fp.opt.smoother == CK_SMOOTHER_GAIN_MATRIX)
    smoothKernelStaged<float, kSmoothBlock>
        <<<grid, kSmoothBlock, stagedSmoothSmemBytes<float, kSmoothBlock>(), st>>>(fp);
  else
    smoothKernel<float, kSmoothBlock><<<grid, kSmoothBlock, 0, st>>>(fp);
  return cudaGetLastError();
}

int occupancyMixed(int variant, int tpb) {
  int n = 0;
  switch (variant) {
    case 0:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, float, 128, 1>, tpb, 0);
      break;
    case 1:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, float, 128, 3>, tpb, 0);
      break;
    case 2:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<float, float, 128, 4>, tpb, 0);
      break;
    case 3:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelCompact<float, float, 256>, 256,
                                                    compactSmemBytes<float, float, 256>());
      break;
    case 5:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelPool<float, float, 384, 256>, 256,
                                                    poolSmemBytes<float, float, 384>());
      break;
    case 6:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelPool<float, float, 448, 256>, 256,
                                                    poolSmemBytes<float, float, 448>());
      break;
    default:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelCompact<float, float, 128>, 128,
                                                    compactSmemBytes<float, float, 128>());
      break;
  }
  return n;
}

}  // namespace ck
