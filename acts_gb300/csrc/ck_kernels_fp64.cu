// ck_kernels_fp64.cu — instantiations of the plain FP64 fit kernel.
#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {

// Register-cap variants of the persistent kernel (launch bounds 128 threads,
// 1 / 3 / 4 resident blocks per SM -> 255 / 168 / 128 registers per thread).
cudaError_t launchFitFP64(const FitParams& fp, int variant, int grid, int block,
                          cudaStream_t st) {
  if (fp.opt.freeToBoundCorrection) {
    // the free-to-bound correction runs in its own instantiation of the
    // 256-slot compaction kernel (the caller sizes the grid for it)
    fitKernelCompact<double, double, 256, true>
        <<<grid, 256, compactSmemBytes<double, double, 256>(), st>>>(fp);
    return cudaGetLastError();
  }
  switch (variant) {
    case 0:
      fitKernel<double, double, 128, 1><<<grid, block, 0, st>>>(fp);
      break;
    case 1:
      fitKernel<double, double, 128, 3><<<grid, block, 0, st>>>(fp);
      break;
    case 2:
      fitKernel<double, double, 128, 4><<<grid, block, 0, st>>>(fp);
      break;
    case 3:
      fitKernelCompact<double, double, 256><<<grid, 256, compactSmemBytes<double, double, 256>(), st>>>(fp);
      break;
    case 5:
      fitKernelPool<double, double, 320, 256><<<grid, 256, poolSmemBytes<double, double, 320>(), st>>>(fp);
      break;
    case 6:
      fitKernelPool<double, double, 256, 256><<<grid, 256, poolSmemBytes<double, double, 256>(), st>>>(fp);
      break;
    default:
      fitKernelCompact<double, double, 128><<<grid, 128, compactSmemBytes<double, double, 128>(), st>>>(fp);
      break;
  }
  return cudaGetLastError();
}

int occupancyFP64(int variant, int tpb) {
  int n = 0;
  switch (variant) {
    case 0:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<double, double, 128, 1>, tpb, 0);
      break;
    case 1:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<double, double, 128, 3>, tpb, 0);
      break;
    case 2:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernel<double, double, 128, 4>, tpb, 0);
      break;
    case 3:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelCompact<double, double, 256>, 256,
                                                    compactSmemBytes<double, double, 256>());
      break;
    case 5:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelPool<double, double, 320, 256>, 256,
                                                    poolSmemBytes<double, double, 320>());
      break;
    case 6:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelPool<double, double, 256, 256>, 256,
                                                    poolSmemBytes<double, double, 256>());
      break;
    default:
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fitKernelCompact<double, double, 128>, 128,
                                                    compactSmemBytes<double, double, 128>());
      break;
  }
  return n;
}

cudaError_t configureFP64() {
  cudaError_t e = cudaFuncSetAttribute(smoothKernelStaged<double, kSmoothBlock>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)stagedSmoothSmemBytes<double, kSmoothBlock>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelPool<double, double, 320, 256>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)poolSmemBytes<double, double, 320>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelPool<double, double, 256, 256>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)poolSmemBytes<double, double, 256>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelCompact<double, double, 256, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<double, double, 256>());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(fitKernelCompact<double, double, 256>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)compactSmemBytes<double, double, 256>());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(fitKernelCompact<double, double, 128>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)compactSmemBytes<double, double, 128>());
}

cudaError_t launchSmoothFP64(const FitParams& fp, cudaStream_t st) {
  const int grid = (fp.n_queue + kSmoothBlock - 1) / kSmoothBlock;
  if (fp.smooth_staged && fp.opt.smoother == CK_SMOOTHER_GAIN_MATRIX)
    smoothKernelStaged<double, kSmoothBlock>
        <<<grid, kSmoothBlock, stagedSmoothSmemBytes<double, kSmoothBlock>(), st>>>(fp);
  else
    smoothKernel<double, kSmoothBlock><<<grid, kSmoothBlock, 0, st>>>(fp);
  return cudaGetLastError();
}

cudaError_t configureMixed();

cudaError_t configureFitKernels() {
  cudaError_t e = configureFP64();
  if (e == cudaSuccess) e = configureMixed();
  if (e == cudaSuccess) e = configureReverseFP64();
  return e != cudaSuccess ? e : configureReverseMixed();
}

int occupancyBlocks(int precision, int variant, int tpb) {
  switch (precision) {
    case CK_PRECISION_MIXED: return occupancyMixed(variant, tpb);
    default: return occupancyFP64(variant, tpb);
  }
}

}  // namespace ck
