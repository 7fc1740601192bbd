// ck_extrapolate.cu — extrapolation of the fitted tracks to the reference
// surface (KalmanFitter::fit_impl, KalmanFitter.hpp:959-972, with
// extrapolateTrackToReferenceSurface, Core/include/Acts/Utilities/
// TrackHelpers.hpp:175-381). Runs after the smoother, one thread per queue
// position, with the stepper of the form (FP64; FP32 stages with FP64
// positions in the mixed form): a track takes one to three Runge-Kutta steps
// from its first (or last) measurement state to the line. The kernel's time
// is set by the rare track that never reaches the line and runs into the
// step limit (1000 steps, alone on its SM; measured 18 ms of FP64 steps on
// 200k barrel tracks, where the others take 1.8 ms): the FP32 stages of the
// mixed form shorten that tail.
#include <cuda_runtime.h>

#include "ck_fitter.cuh"
#include "ck_launch.h"

namespace ck {
namespace {

// the straight-line distance from a candidate start state to the reference
// surface (findTrackStateForExtrapolation's intersect); false when the state
// is missing or the line is parallel to the track
__device__ bool startDistance(const FitParams& fp, const ExtStart& es, double& dist) {
  if (es.surface < 0) return false;
  Surf<double> sf;
  sf.load(fp.surfaces + es.surface);
  double f[8];
  boundToFree(sf, es.par, f);
  Surf<double> ts;
  ts.load(fp.surfaces + fp.ref_surface);
  const double p[3] = {f[0], f[1], f[2]}, d[3] = {f[4], f[5], f[6]};
  return Lane<double, double>::lineIntersect(ts, p, d, kOnSurfaceTolerance, dist);
}

template <typename P, typename CV>
__global__ void __launch_bounds__(kExtrapolateBlock) extrapolateKernel(FitParams fp) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < fp.n_queue;
       q += gridDim.x * blockDim.x) {
    if (fp.tip[q] < 0) continue;  // the fit failed
    const int t = fp.perm ? __ldg(&fp.perm[q]) : q;
    if (fp.out.status[t] != CK_TRACK_OK) continue;  // the smoother failed
    const ExtStart& first = fp.ext[2 * (size_t)q];
    const ExtStart& last = fp.ext[2 * (size_t)q + 1];
    // the reversed pass reached the reference surface: the track has its
    // parameters (KalmanFitter.hpp:938-943, :949)
    if (first.fitted) continue;
    Lane<P, CV> L;
    L.t = t;
    L.q = q;
    if (first.surface < 0) {
      L.fail(fp, CK_TRACK_NO_COMPATIBLE_STATE);
      continue;
    }
    // TrackExtrapolationStrategy (TrackHelpers.hpp:214-300)
    const ExtStart* from = nullptr;
    double dist = 0.0;
    if (fp.ref_strategy == CK_EXTRAPOLATE_FIRST || fp.ref_strategy == CK_EXTRAPOLATE_LAST) {
      from = fp.ref_strategy == CK_EXTRAPOLATE_FIRST ? &first : &last;
      if (!startDistance(fp, *from, dist)) from = nullptr;
    } else {
      double df = 0.0, dl = 0.0;
      const bool vf = startDistance(fp, first, df), vl = startDistance(fp, last, dl);
      const double af = vf ? fabs(df) : CUDART_INF, al = vl ? fabs(dl) : CUDART_INF;
      if (vf && af <= al) {
        from = &first;
        dist = df;
      } else if (vl && al <= af) {
        from = &last;
        dist = dl;
      }
    }
    if (!from) {
      L.fail(fp, CK_TRACK_REFERENCE_UNREACHABLE);
      continue;
    }
    L.startExtrapolation(fp, q, t, *from, dist);
    // bounded: every step either ends the lane or counts towards maxSteps
    while (L.phase == PH_STEP) L.template step<kStepExtrapolate>(fp, q);
  }
}

}  // namespace

cudaError_t launchExtrapolate(const FitParams& fp, int precision, cudaStream_t st) {
  FitParams e = fp;
  e.opt = fp.extOpt;  // the reference's default propagator options
  const int grid = (fp.n_queue + kExtrapolateBlock - 1) / kExtrapolateBlock;
  if (precision == CK_PRECISION_MIXED)
    extrapolateKernel<float, float><<<grid, kExtrapolateBlock, 0, st>>>(e);
  else
    extrapolateKernel<double, double><<<grid, kExtrapolateBlock, 0, st>>>(e);
  return cudaGetLastError();
}

}  // namespace ck
