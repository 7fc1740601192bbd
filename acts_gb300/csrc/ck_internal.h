// ck_internal.h — host/device structures private to libcudakalman.so.
#pragma once

#include <cstdint>

#include "cudakalman.h"

namespace ck {

// Surface as the kernels see it: the ck_surface fields plus the material
// slab precomputed as the MaterialSlab constructor does
// (Core/include/Acts/Material/MaterialSlab.hpp:119-128).
struct DevSurface {
  double R[9];  // row-major, columns = local axes
  double c[3];
  double radius;
  int type;
  int flags;
  float matI, matNe;                 // mean excitation, molar electron density
  float thickness, tX0, tL0;         // slab thickness and thickness / X0, / L0
  float split;                       // split factor
  int vacuum;                        // Material::isVacuum() (Ar <= 0)
  int pad;
  float Rf[9], cf[3], radiusf;        // FP32 copies for the mixed form
  int pad2;
};

// Reference angles of the mixed form's FP64 atan2: entry k + 64 holds
// (cos, sin) of k * kTrigStep, k = -64..64.
constexpr int kTrigEntries = 129;
constexpr double kTrigStep = 3.14159265358979323846 / 64;

// Field as the kernels see it. Grid nodes are float4 (Bx, By, Bz, 0) in
// Tesla, layout [ix][iy][iz]; the axis arithmetic follows the reference's
// equidistant Axis built by fieldMapXYZ.
struct DevField {
  int kind;
  int n[3];
  double b[3];      // constant field, GeV/(e mm)
  double mn[3];     // first grid point
  double width[3];  // bin width of the reference axis
  double upper[3];  // lower edge of the last bin (end of the valid range)
  // the same constants rounded to float (host conversion, round to
  // nearest) for the mixed form's FP32 lookups
  float bf[3], mnf[3], widthf[3], upperf[3];
  const float4* nodes;
};

// float / double constants of Interactions.cpp, evaluated on the host with
// the reference's literal arithmetic.
struct MatConst {
  float Me, K, plasmaScale, invCm3;
  double highland, rossi;
  float log10f;  // ck_logf(10)
  float pad;
};

struct DevOptions {
  double stepTolerance, stepSizeCutOff, initialStepSize, maxStepSize;
  double pathLimit, loopFraction, surfaceTolerance, nearLimit, outlierChi2Cut;
  uint32_t maxRkTrials, maxSteps, maxTargetSkipping;
  int loopProtection, multipleScattering, energyLoss, joseph;
  int useOutlierCut, earlyTermination;
  int smoother;  // CK_SMOOTHER_*
  int freeToBoundCorrection;
  int reverseFiltering;
  double reverseCovScaling, reverseMomThreshold;
};

// Record of one forward track state kept for the smoother (scratch), one
// contiguous block per (track, state): the bound parameters in FP64
// (predicted 6, filtered 6), path length, chi2, surface id, type flags and
// the matrices in the covariance type CV of the form (predicted cov 21 and
// filtered cov 21, packed upper; jacobian 36). A lane writes its state's
// block as a whole, so DRAM sees full sectors.
// The record's flags word holds the CK_FLAG_* type flags in its low 16 bits
// and, for measurement states, the measurement's subspace (CK_MEAS_*) from
// bit 16.
constexpr int kRecSubShift = 16;
constexpr uint32_t kRecFlagMask = 0xffffu;
constexpr int kRecPred = 0;
constexpr int kRecFilt = 6;
constexpr int kRecParams = 12;
constexpr int kRecPredCov = 0;
constexpr int kRecFiltCov = 21;
constexpr int kRecJac = 42;
constexpr int kRecMatrix = 78;

template <typename CV>
struct RecState {
  double par[kRecParams];
  double pathLength, chi2;
  int32_t surface, flags;
  CV mat[kRecMatrix];
};
static_assert(sizeof(RecState<float>) == 432, "record layout");
static_assert(sizeof(RecState<double>) == 744, "record layout");

// A track state the extrapolation to the reference surface may start from
// (the first and the last state with a non-outlier measurement, slots 0 and
// 1 of each queue position): its surface and smoothed parameters and
// covariance (packed upper) in FP64. Written by the smoother; with reverse
// filtering, slot 0 holds the reversed pass's last filtered state (written by
// that pass) and is also the first measurement state's smoothed output.
struct ExtStart {
  double par[6];
  double cov[21];
  int32_t surface;  // -1: no such state
  // slot 0 with reverse filtering: 1 when the reversed pass reached the
  // reference surface and wrote the track parameters itself
  int32_t fitted;
};
static_assert(sizeof(ExtStart) == 224, "extrapolation start layout");

// The propagation entry's per-track targets and path limits (inputs) and its
// outputs (ck_propagate_out; end parameters and covariance go through
// FitParams::out.track_params / track_cov). Unused (NULL) in the fit.
struct PropIO {
  const int32_t* target;
  const double* path_limit;
  double* jac;     // [36][n] transport Jacobian, or NULL
  double* frames;  // [n*12] end plane without a target, or NULL
  double* path;    // [n], or NULL
  int32_t* steps;  // [n], or NULL
};

struct FitParams {
  int n_tracks;
  int n_queue;  // number of slots in the work queue (= n_tracks)
  // inputs
  const int32_t* seq_off;
  const int32_t* seq_surf;
  const int32_t* meas_off;
  const int32_t* meas_surf;
  const double* meas_val;
  const double* meas_cov;
  const int32_t* meas_sub;  // CK_MEAS_* per measurement, or NULL (all 2D)
  const double* start_params;
  const double* start_cov;
  const double* start_frames;
  const float* particle;
  const int32_t* pdg;
  // queue: slot -> track index (descending sequence length) and ticket
  const int32_t* perm;
  int32_t* ticket;
  // track-state records of the forward filter, read back by the smoother
  // kernel: RecState<CV> of state k of queue position q at
  // rec[q * max_states + k];
  //   tip [q]: index of the last measurement state, -1 when the forward
  //            filter failed (its status is then already written)
  void* rec;
  int32_t* tip;
  const double2* trig;  // kTrigEntries reference angles (mixed form)
  // lanes of each warp that take tracks: all 32 for large batches; fewer
  // when the batch is small, so that its tracks spread over all warps
  int lanes_per_warp;
  // Runge-Kutta trials a STEP item of the compaction kernels may take in one
  // round (>= 1)
  int steps_per_round;
  // the RTS smoother reads its records through warp-cooperative staging in
  // shared memory (smoothKernelStaged) instead of per lane
  int smooth_staged;
  int max_states;
  // outputs (device memory, ck_batch_out layout)
  ck_batch_out out;
  // detector
  const DevSurface* surfaces;
  int n_surfaces;
  DevField field;
  MatConst mc;
  DevOptions opt;
  // extrapolation to the reference surface: its table index (-1: none), the
  // strategy (CK_EXTRAPOLATE_*), two start states per queue position, and
  // the propagator options it runs with (the reference's defaults)
  int ref_surface;
  int ref_strategy;
  ExtStart* ext;
  DevOptions extOpt;
  PropIO prop;
  // Smoothing in the forward filter's tail (compaction kernels): a block
  // whose slots are all done smooths finished tracks, claimed in queue order
  // by the ticket smooth_ticket; smoothed[q] = 1 marks them for the smoother
  // kernel, which takes the rest. NULL: the smoother kernel smooths all.
  uint8_t* smoothed;
  int32_t* smooth_ticket;
};

}  // namespace ck
