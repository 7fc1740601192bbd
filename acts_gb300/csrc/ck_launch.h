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
cudaError_t launchFitMixedCov64(const FitParams& fp, int variant, int grid, int block,
                                cudaStream_t st);
int occupancyFP64(int variant, int tpb);
int occupancyMixed(int variant, int tpb);
int occupancyMixedCov64(int variant, int tpb);
int occupancyBlocks(int precision, int variant, int tpb);

}  // namespace ck
