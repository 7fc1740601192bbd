// ck_launch.h — host-side launchers of the fit kernels.
#pragma once

#include <cuda_runtime.h>

#include "ck_internal.h"

namespace ck {

constexpr int kNumFitVariants = 3;
constexpr int kFitMaxBlock = 128;

cudaError_t launchFitFP64(const FitParams& fp, int variant, int grid, int block,
                          cudaStream_t st);
cudaError_t launchFitMixed(const FitParams& fp, int variant, int grid, int block,
                           cudaStream_t st);
int occupancyFP64(int variant, int tpb);
int occupancyMixed(int variant, int tpb);
int occupancyBlocks(int precision, int variant, int tpb);
cudaError_t launchSmoothFP64(const FitParams& fp, cudaStream_t st);
cudaError_t launchSmoothMixed(const FitParams& fp, cudaStream_t st);
inline cudaError_t launchSmooth(const FitParams& fp, int precision, cudaStream_t st) {
  return precision == CK_PRECISION_MIXED ? launchSmoothMixed(fp, st) : launchSmoothFP64(fp, st);
}
constexpr int kSmoothBlock = 128;

}  // namespace ck
