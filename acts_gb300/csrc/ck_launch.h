// ck_launch.h — host-side launchers of the fit kernels.
#pragma once

#include <cuda_runtime.h>

#include "ck_internal.h"

namespace ck {

// Forward-filter kernel variants: 0-2 per-warp phase scheduling with
// register caps of 255 / 168 / 128 (1 / 3 / 4 resident 128-thread blocks);
// 3-4 block-level phase compaction with 256 / 128 slots per block; 5-6
// warp-autonomous phase pools, 256 threads with more slots (5: 384 mixed /
// 320 FP64; 6: 448 mixed / 256 FP64).
constexpr int kNumFitVariants = 7;
constexpr int kFitMaxBlock = 128;
constexpr int kDefaultVariant = 3;
// Runge-Kutta trials per round of the compaction kernels by precision
// (FP64, mixed): measured best on the barrel and uneven workloads
constexpr int kDefaultStepsPerRound[2] = {2, 3};
// the RTS smoother reads its records through warp-cooperative staging
constexpr int kDefaultSmootherStaged = 0;
// block size a variant requires (0: any multiple of 32 up to kFitMaxBlock)
inline int variantBlock(int variant) {
  return (variant == 3 || variant >= 5) ? 256 : (variant == 4 ? 128 : 0);
}
inline bool validLaunch(int variant, int tpb) {
  if (variant < 0 || variant >= kNumFitVariants) return false;
  const int vb = variantBlock(variant);
  return vb ? tpb == vb : (tpb > 0 && tpb <= kFitMaxBlock && tpb % 32 == 0);
}

cudaError_t launchFitFP64(const FitParams& fp, int variant, int grid, int block,
                          cudaStream_t st);
cudaError_t launchFitMixed(const FitParams& fp, int variant, int grid, int block,
                           cudaStream_t st);
int occupancyFP64(int variant, int tpb);
int occupancyMixed(int variant, int tpb);
int occupancyBlocks(int precision, int variant, int tpb);
// one-time per-device set-up of the kernels (shared-memory limits)
cudaError_t configureFitKernels();
cudaError_t launchSmoothFP64(const FitParams& fp, cudaStream_t st);
cudaError_t launchSmoothMixed(const FitParams& fp, cudaStream_t st);
inline cudaError_t launchSmooth(const FitParams& fp, int precision, cudaStream_t st) {
  return precision == CK_PRECISION_MIXED ? launchSmoothMixed(fp, st) : launchSmoothFP64(fp, st);
}
constexpr int kSmoothBlock = 128;
// reverse filtering (ck_reverse_*.cu): the reversed filter pass, then the
// output kernel in place of the smoother; the pass needs the queue ticket
// cleared and the extrapolation start slots
cudaError_t launchReverseFP64(const FitParams& fp, int grid, cudaStream_t st);
cudaError_t launchReverseMixed(const FitParams& fp, int grid, cudaStream_t st);
cudaError_t launchReverseOutputFP64(const FitParams& fp, cudaStream_t st);
cudaError_t launchReverseOutputMixed(const FitParams& fp, cudaStream_t st);
cudaError_t configureReverseFP64();
cudaError_t configureReverseMixed();
inline cudaError_t launchReverse(const FitParams& fp, int precision, int grid, cudaStream_t st) {
  return precision == CK_PRECISION_MIXED ? launchReverseMixed(fp, grid, st)
                                         : launchReverseFP64(fp, grid, st);
}
inline cudaError_t launchReverseOutput(const FitParams& fp, int precision, cudaStream_t st) {
  return precision == CK_PRECISION_MIXED ? launchReverseOutputMixed(fp, st)
                                         : launchReverseOutputFP64(fp, st);
}
// extrapolation of every successfully smoothed track to the reference
// surface (with the form's stepper; ck_extrapolate.cu)
cudaError_t launchExtrapolate(const FitParams& fp, int precision, cudaStream_t st);
constexpr int kExtrapolateBlock = 64;

}  // namespace ck
