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
};

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
};

// Record of one forward track state kept for the smoother (scratch).
// Doubles per record: predicted 6, predicted cov 21 (packed upper),
// filtered 6, filtered cov 21, jacobian 36.
constexpr int kRecPred = 0;
constexpr int kRecPredCov = 6;
constexpr int kRecFilt = 27;
constexpr int kRecFiltCov = 33;
constexpr int kRecJac = 54;
constexpr int kRecDoubles = 90;

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
  const double* start_params;
  const double* start_cov;
  const double* start_frames;
  const float* particle;
  const int32_t* pdg;
  // queue: slot -> track index (descending sequence length) and ticket
  const int32_t* perm;
  int32_t* ticket;
  // scratch records of the tracks in flight, indexed by the resident thread
  // slot (blockIdx.x * blockDim.x + threadIdx.x < n_slots):
  //   rec        [(k * kRecDoubles + f) * n_slots + slot]
  //   rec_meta   [(k * 2 + {surface, flags}) * n_slots + slot]
  //   rec_meta_d [(k * 2 + {pathLength, chi2}) * n_slots + slot]
  double* rec;
  int32_t* rec_meta;
  double* rec_meta_d;
  int n_slots;
  int max_states;
  // outputs (device memory, ck_batch_out layout)
  ck_batch_out out;
  // detector
  const DevSurface* surfaces;
  int n_surfaces;
  DevField field;
  MatConst mc;
  DevOptions opt;
};

}  // namespace ck
