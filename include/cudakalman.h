/*
 * cudakalman.h — C ABI of ActsPlugins::CudaKalman, a batched Kalman track
 * fitter for one NVIDIA GB300 (sm_103a).
 *
 * The ABI is the drop-in boundary for the reference call
 *
 *   Acts::KalmanFitter<Propagator<EigenStepper<>, DirectNavigator>,
 *                      VectorMultiTrajectory>::fit(begin, end, startParameters,
 *                                                  kfOptions, sSequence,
 *                                                  trackContainer)
 *   (Core/include/Acts/TrackFitting/KalmanFitter.hpp:719-731, the
 *    DirectNavigator overload; fit_impl at :859-984)
 *
 * A foreign caller (ctypes, cgo, JNI, the C++ facade in
 * acts_gb300/host/ActsPlugins/CudaKalman.hpp) binds these symbols. Every
 * signature uses plain C types: pointers, sizes and POD structs. No C++, no
 * torch and no CUDA types appear here; CUDA streams are passed as void*.
 *
 * Units are the reference's native units (Core/include/Acts/Definitions/
 * Units.hpp:85-174): length mm, momentum/energy/mass GeV, time mm/c
 * (1 ns = 299.792458 mm), magnetic field in GeV/(e*mm) (1 T = 0.000299792458).
 *
 * Parameter order follows Core/include/Acts/Definitions/TrackParametrization.hpp:
 *   bound: loc0, loc1, phi, theta, q/p, t        (6)
 *   free : x, y, z, t, dx, dy, dz, q/p           (8)
 *
 * Output arrays are structure-of-arrays with the track index innermost:
 *   element c of state k of track t lives at  [(k * C + c) * n_tracks + t]
 *   (C = 6 for parameter vectors, 36 for covariance / Jacobian matrices in
 *   row-major order, 1 for scalars). Per-track scalars live at [t].
 * States are stored in propagation order: k = 0 is the first track state and
 * k = n_states[t]-1 is the tip (the last state that carries a source link),
 * i.e. the order of Acts::TrackProxy::trackStates() after linkForward().
 */
#ifndef CUDAKALMAN_H
#define CUDAKALMAN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CK_API_VERSION 1

/* ---------------------------------------------------------------- status */

/* Call-level status. */
typedef enum ck_status {
  CK_OK = 0,
  CK_ERR_INVALID_ARGUMENT = 1, /* bad pointer, size or option */
  CK_ERR_CUDA = 2,             /* a CUDA runtime call failed */
  CK_ERR_NO_DEVICE = 3,        /* no CUDA device visible */
  CK_ERR_OUT_OF_MEMORY = 4,    /* device allocation failed */
  CK_ERR_UNSUPPORTED = 5,      /* a requested feature is outside the declared set */
  CK_ERR_BUDGET = 6,           /* serving: request larger than the memory budget */
  CK_ERR_TIMEOUT = 7,          /* a bounded wait ran out */
  CK_ERR_NOT_READY = 8,        /* serving: nothing finished yet */
  CK_ERR_SCRATCH_LIMIT = 9     /* request exceeds a fixed scratch capacity */
} ck_status;

/* Per-track status, one int32 per track. Mirrors the error enums the
 * reference fit returns through Result<...>:
 *   KalmanFitterError (Core/include/Acts/TrackFitting/KalmanFitterError.hpp:20-31)
 *   PropagatorError::StepCountLimitReached / NextTargetLimitReached
 *   EigenStepperError::StepSizeStalled / StepSizeAdjustmentFailed
 *   SurfaceError::GlobalPositionNotOnSurface
 *   MagneticFieldError::OutOfBounds                                       */
enum {
  CK_TRACK_OK = 0,
  CK_TRACK_UPDATE_FAILED = 1,         /* NaN in the Kalman gain            */
  CK_TRACK_SMOOTH_FAILED = 2,         /* NaN in the smoother gain          */
  CK_TRACK_NO_MEASUREMENT_FOUND = 3,  /* forward filter produced no measurement */
  CK_TRACK_STEP_COUNT_LIMIT = 4,      /* propagation exceeded maxSteps     */
  CK_TRACK_NEXT_TARGET_LIMIT = 5,     /* maxTargetSkipping exceeded        */
  CK_TRACK_STEP_SIZE_STALLED = 6,     /* |h| fell below stepSizeCutOff     */
  CK_TRACK_STEP_ADJUST_FAILED = 7,    /* more than maxRungeKuttaStepTrials */
  CK_TRACK_NOT_ON_SURFACE = 8,        /* globalToLocal failed              */
  CK_TRACK_FIELD_OUT_OF_BOUNDS = 9,   /* grid field lookup outside the map */
  CK_TRACK_TOO_MANY_STATES = 10,      /* more states than out->max_states  */
  CK_TRACK_NOT_PROCESSED = 11,        /* the kernel did not reach the track */
  CK_TRACK_INVALID_INPUT = 12,        /* a surface id outside the table    */
  /* extrapolation to the reference surface (TrackExtrapolationError,
   * Core/include/Acts/Utilities/TrackHelpers.hpp:48-53) */
  CK_TRACK_NO_COMPATIBLE_STATE = 13,  /* CompatibleTrackStateNotFound      */
  CK_TRACK_REFERENCE_UNREACHABLE = 14, /* ReferenceSurfaceUnreachable      */
  /* KalmanFitterError::InconsistentTrackStates: the reversed filter's last
   * measurement state is not on the forward filter's first one's surface */
  CK_TRACK_INCONSISTENT_STATES = 15
};

/* Track-state type flags, bit positions of Acts::TrackStateFlag
 * (Core/include/Acts/EventData/TrackStateType.hpp:30-48). */
enum {
  CK_FLAG_HAS_MEASUREMENT = 1u << 0,
  CK_FLAG_HAS_PARAMETERS = 1u << 1,
  CK_FLAG_IS_OUTLIER = 1u << 2,
  CK_FLAG_IS_HOLE = 1u << 3,
  CK_FLAG_HAS_MATERIAL = 1u << 4
};

/* ------------------------------------------------------------- geometry */

enum { CK_SURFACE_PLANE = 0, CK_SURFACE_CYLINDER = 1, CK_SURFACE_LINE = 2 };
enum { CK_SURF_SENSITIVE = 1, CK_SURF_MATERIAL = 2 };

/* A surface of the flat surface table (the DirectNavigator sequence refers to
 * surfaces by their index in this table).
 *   Plane   : PlaneSurface (Core/src/Surfaces/PlaneSurface.cpp:60-191),
 *             local frame = rotation columns, normal = column 2.
 *   Cylinder: CylinderSurface (Core/src/Surfaces/CylinderSurface.cpp:90-277),
 *             symmetry axis = rotation column 2, radius `radius`.
 *   Line    : LineSurface without bounds (Core/src/Surfaces/LineSurface.cpp
 *             :57-251), line = rotation column 2 through `center`; a
 *             PerigeeSurface (PerigeeSurface.cpp) is the line along global z
 *             (identity rotation). Only as the reference surface of the
 *             extrapolation (ck_options.reference_surface); a sequence or a
 *             measurement on a line surface is invalid input.
 * Material is a homogeneous slab (HomogeneousSurfaceMaterial) with the
 * reference's float Material fields (Core/include/Acts/Material/Material.hpp
 * :135-145) and split factor (Core/src/Material/ISurfaceMaterial.cpp:18-46). */
typedef struct ck_surface {
  int32_t type;          /* CK_SURFACE_PLANE / _CYLINDER / _LINE             */
  int32_t flags;         /* CK_SURF_SENSITIVE | CK_SURF_MATERIAL            */
  double rotation[9];    /* row-major 3x3, columns = local x, y, z axes     */
  double center[3];
  double radius;         /* cylinder radius (mm)                            */
  double half_length_z;  /* cylinder bounds (0: unbounded)                  */
  double half_x, half_y; /* plane rectangle bounds (0: unbounded); bounds
                            apply to the target of ck_find_tracks only      */
  float mat_thickness;   /* slab thickness (mm)                             */
  float mat_x0, mat_l0;  /* radiation / nuclear interaction length (mm)     */
  float mat_ar, mat_z;   /* relative atomic mass, nuclear charge            */
  float mat_molar_rho;   /* molar density (mol / mm^3)                      */
  float mat_molar_electron_rho; /* molar electron density = Z * molarRho    */
  float mat_mean_excitation;    /* I (GeV)                                  */
  float split_factor;    /* ISurfaceMaterial split factor (default 1)       */
  float reserved;
} ck_surface;

/* ---------------------------------------------------------------- field */

enum { CK_FIELD_CONSTANT = 0, CK_FIELD_GRID_XYZ = 1 };

/* Magnetic field.
 *   constant: ConstantBField (Core/include/Acts/MagneticField/ConstantBField.hpp:21-45)
 *   grid    : InterpolatedBFieldMap built by fieldMapXYZ
 *             (Core/src/MagneticField/BFieldMapUtils.cpp:106-186): grid
 *             points at x = min[0] + i * (max[0]-min[0])/(n[0]-1), same for
 *             y and z; trilinear interpolation (Core/include/Acts/Utilities/
 *             Interpolation.hpp:96-120); lookups outside
 *             [min, max) fail with CK_TRACK_FIELD_OUT_OF_BOUNDS.
 * values: n[0]*n[1]*n[2]*3 floats in Tesla, layout [ix][iy][iz][3]. Host
 * memory; the library copies it to the device at ck_create(). */
typedef struct ck_field {
  int32_t kind;
  int32_t n[3];
  double constant_tesla[3];
  double min[3];
  double max[3];
  const float* values_tesla;
} ck_field;

/* ------------------------------------------------------------- options */

/* FP64: everything in double (the reference's arithmetic).
 * MIXED: Runge-Kutta stages, field interpolation, Jacobian transport and
 *   covariance transport in FP32; the free parameters (position, direction,
 *   q/p, time) are accumulated in FP64 from the FP32 stage increments;
 *   Kalman update (Joseph form when selected), 2x2 inverse, smoother-gain
 *   inverse, bound-parameter conversion and chi2 in FP64. */
enum { CK_PRECISION_FP64 = 0, CK_PRECISION_MIXED = 1 };

/* Smoother extension (KalmanFitterExtensions::smoother):
 * GAIN_MATRIX: GainMatrixSmoother (Core/src/TrackFitting/GainMatrixSmoother.cpp:18-97),
 * MBF: MbfSmoother, the modified Bryson-Frazier smoother
 *   (Core/include/Acts/TrackFitting/MbfSmoother.hpp:48-90, MbfSmoother.cpp:17-48,
 *    detail/MbfSmootherImpl.hpp:17-58), which the reference's example
 *   KalmanFitterFunction connects (KalmanFitterFunction.cpp:77,102). */
enum { CK_SMOOTHER_GAIN_MATRIX = 0, CK_SMOOTHER_MBF = 1 };
#define CK_NUM_PRECISIONS 2

/* Fit options. ck_options_default() fills the reference defaults:
 *   StepperPlainOptions (Core/include/Acts/Propagator/StepperOptions.hpp:36-49)
 *   PropagatorPlainOptions (Core/include/Acts/Propagator/PropagatorOptions.hpp:28-51)
 *   DirectNavigator::Options (Core/include/Acts/Propagator/DirectNavigator.hpp:34-48)
 *   KalmanFitterOptions (Core/include/Acts/TrackFitting/KalmanFitter.hpp:108-186)
 *   GainMatrixUpdater (Joseph off) and a predicted-chi2 outlier cut
 *   (Examples/Algorithms/TrackFitting/src/KalmanFitterFunction.cpp:60-68;
 *    +inf = no outlier finder, the void outlier finder of the reference). */
typedef struct ck_options {
  double step_tolerance;        /* 1e-4                                    */
  double step_size_cutoff;      /* 0                                       */
  double initial_step_size;     /* 10 m                                    */
  double max_step_size;         /* DBL_MAX                                 */
  uint32_t max_rk_step_trials;  /* 10000                                   */
  uint32_t max_steps;           /* 1000                                    */
  uint32_t max_target_skipping; /* 100                                     */
  int32_t loop_protection;      /* 1                                       */
  double path_limit;            /* DBL_MAX                                 */
  double loop_fraction;         /* 0.5                                     */
  double surface_tolerance;     /* s_onSurfaceTolerance = 1e-4 mm          */
  double near_limit;            /* DirectNavigator nearLimit = -100 um     */
  int32_t multiple_scattering;  /* 1                                       */
  int32_t energy_loss;          /* 1                                       */
  int32_t use_joseph;           /* 0 (GainMatrixUpdater default)           */
  int32_t precision;            /* CK_PRECISION_*                          */
  double outlier_chi2_cut;      /* +inf                                    */
  /* KalmanFitterOptions::reverseFiltering (KalmanFitter.hpp:897-945): 1
   * (for every track; see also reverse_filtering_mom_threshold) replaces the
   * smoother by a second filter pass backwards along the
   * sequence, started from the last measurement state with its covariance
   * scaled by reverse_filtering_cov_scaling and aimed at reference_surface.
   * Only the first measurement state receives smoothed parameters (the
   * reversed pass's last filtered ones) and the last one its own filtered
   * parameters; every other state's smoothed parameters are NaN. The track
   * parameters come from the reversed pass when it reached the reference
   * surface, else from the extrapolation. Default 0. */
  int32_t reverse_filtering;
  /* KalmanFitterOptions::freeToBoundCorrection (FreeToBoundCorrection with
   * its defaults: alpha 0.1, beta 2, incidence window [1e-5, 0.99500417]):
   * the covariance transport to each state's surface goes through the
   * unscented transform of CorrectedFreeToBoundTransformer
   * (Core/src/EventData/CorrectedTransformationFreeToBound.cpp:51-183,
   * Core/src/Propagator/detail/CovarianceEngine.cpp:120-144). 0 (default)
   * or 1. Computed in FP64 in both forms. */
  int32_t free_to_bound_correction;
  /* KalmanFitterOptions::referenceSurface: -1 (none) or the index of a
   * CK_SURFACE_LINE surface of the table. After smoothing, each track is
   * extrapolated to it (extrapolateTrackToReferenceSurface,
   * Core/include/Acts/Utilities/TrackHelpers.hpp:175-381) with the
   * reference's default propagator options, and its parameters and
   * covariance there are written to ck_batch_out.track_params/track_cov. */
  int32_t reference_surface;
  /* 0 (default, the reference's behaviour): when outliers keep the track
   * incomplete, propagation continues after the last surface that carries a
   * source link until the loop-protection path limit, and any propagation
   * error on the way (e.g. leaving the field map) fails the fit. 1: stop
   * after the last such surface (states beyond it are never part of the
   * track), which turns those failures into successful fits. */
  int32_t early_termination;
  int32_t smoother;             /* CK_SMOOTHER_*, default GAIN_MATRIX       */
  /* KalmanFitterOptions::referenceSurfaceStrategy (TrackExtrapolationStrategy):
   * the track state the extrapolation starts from; default FIRST_OR_LAST. */
  int32_t reference_strategy;
  /* KalmanFitterOptions::reverseFilteringCovarianceScaling: 100 */
  double reverse_filtering_cov_scaling;
  /* KalmanFitterExtensions::reverseFilteringLogic as the examples' fitter
   * function connects it (SimpleReverseFilteringLogic,
   * Examples/Algorithms/TrackFitting/src/KalmanFitterFunction.cpp:50-58):
   * with reverse_filtering 0, a track is reverse-filtered when its last
   * measurement state's filtered momentum 1/|q/p| is at most this threshold
   * (GeV). Default 0: no track. */
  double reverse_filtering_mom_threshold;
} ck_options;

enum { CK_EXTRAPOLATE_FIRST = 0, CK_EXTRAPOLATE_LAST = 1, CK_EXTRAPOLATE_FIRST_OR_LAST = 2 };

/* --------------------------------------------------------------- handle */

/* Static configuration of a fitter handle: the surface table and the field
 * (both copied to the device and kept resident), tuning knobs and the device
 * ordinal. */
typedef struct ck_config {
  int32_t device;              /* CUDA device ordinal                       */
  int32_t n_surfaces;
  const ck_surface* surfaces;  /* host pointer, copied                      */
  ck_field field;              /* field values copied                       */
  int32_t threads_per_block;   /* 0 = autotuned / default                   */
  int32_t blocks_per_sm;       /* 0 = autotuned / default                   */
  int32_t use_graph;           /* capture the batch pipeline in a CUDA graph */
  int32_t reserved;
  const char* autotune_cache;  /* path of the autotuner cache file or NULL  */
} ck_config;

typedef struct ck_handle ck_handle;

/* Where the pointers of a batch live. */
enum { CK_MEM_HOST = 0, CK_MEM_DEVICE = 1 };

/* One batch of independent track fits: for every track the source links
 * (calibrated 2D measurements on loc0/loc1, the pass-through calibrator of
 * the reference tests), the start parameters with covariance on a per-track
 * start plane, the particle hypothesis and the DirectNavigator surface
 * sequence. CSR offsets have n_tracks+1 entries. */
typedef struct ck_batch_in {
  int32_t n_tracks;
  int32_t memory;                /* CK_MEM_HOST or CK_MEM_DEVICE            */
  const int32_t* seq_offsets;    /* [n_tracks+1]                            */
  const int32_t* seq_surfaces;   /* [seq_offsets[n_tracks]] surface ids     */
  const int32_t* meas_offsets;   /* [n_tracks+1]                            */
  const int32_t* meas_surfaces;  /* [n_meas] surface id of each source link */
  const double* meas_values;     /* [n_meas*2] (loc0, loc1); 1D: see below  */
  const double* meas_cov;        /* [n_meas*4] row-major 2x2; 1D: see below */
  const double* start_params;    /* [n_tracks*6] bound parameters           */
  const double* start_cov;       /* [n_tracks*36] row-major                 */
  const double* start_frames;    /* [n_tracks*12] start plane: rotation (9,
                                    row-major, columns = local axes) + center */
  const float* particle;         /* [n_tracks*2] (mass GeV, |q|)            */
  const int32_t* particle_pdg;   /* [n_tracks] absolute PDG id              */
  /* [n_meas] measured bound parameters of each source link, the projector's
   * subspace (BoundSubspaceIndices; MeasurementsCreator's eLoc0 / eLoc1 /
   * eLoc01): CK_MEAS_LOC0 or CK_MEAS_LOC1 for a 1D (strip) measurement,
   * whose value is meas_values[2m] and variance meas_cov[4m] (the other
   * slots are ignored), CK_MEAS_LOC01 for a 2D one. NULL: every source link
   * is 2D. The updater, outlier chi2, ndf and MbfSmoother use the subspace
   * (GainMatrixUpdaterImpl.hpp:95-104 instantiates N = 1..6; N = 1, 2 with
   * local-coordinate projectors here). */
  const int32_t* meas_subspace;
} ck_batch_in;

/* Measurement subspaces (bit i: bound parameter i is measured). */
enum { CK_MEAS_LOC0 = 1, CK_MEAS_LOC1 = 2, CK_MEAS_LOC01 = 3 };

/* Which per-state components to write (TrackStatePropMask analogue). */
enum {
  CK_OUT_PREDICTED = 1u << 0,
  CK_OUT_FILTERED = 1u << 1,
  CK_OUT_SMOOTHED = 1u << 2,
  CK_OUT_JACOBIAN = 1u << 3,
  CK_OUT_REFERENCE = 1u << 4,  /* track parameters at the reference surface */
  /* The per-state covariance arrays (predicted_cov, filtered_cov,
   * smoothed_cov) hold each symmetric matrix once, as its upper triangle
   * row by row ((0,0), (0,1), ..., (0,5), (1,1), ..., (5,5)): C = 21 instead
   * of 36, the same values, 42 % fewer bytes to move. The Jacobian and
   * track_cov keep C = 36. */
  CK_OUT_PACKED_COV = 1u << 5
};

/* Results of a batch. Arrays the component mask does not select may be NULL.
 * Layout: see the header comment (SoA, track index innermost). */
typedef struct ck_batch_out {
  int32_t max_states;        /* capacity per track                          */
  uint32_t components;       /* CK_OUT_* mask                               */
  int32_t memory;            /* CK_MEM_HOST or CK_MEM_DEVICE                */
  int32_t reserved;
  /* per track [n_tracks] */
  int32_t* status;
  int32_t* n_states;
  int32_t* n_measurements;
  int32_t* n_holes;
  int32_t* n_outliers;
  int32_t* ndf;
  double* chi2_sum;          /* sum of measurement-state chi2                */
  /* per state [max_states * C * n_tracks]; slots k >= n_states[t] are
   * unspecified */
  int32_t* state_surface;    /* surface id (C = 1)                           */
  uint32_t* state_flags;     /* CK_FLAG_* (C = 1)                            */
  double* state_path_length; /* accumulated path at the state (C = 1)        */
  double* state_chi2;        /* filtered chi2 of measurement states (C = 1)  */
  double* predicted;         /* C = 6  */
  double* predicted_cov;     /* C = 36 (21 with CK_OUT_PACKED_COV) */
  double* filtered;          /* C = 6  */
  double* filtered_cov;      /* C = 36 (21 with CK_OUT_PACKED_COV) */
  double* smoothed;          /* C = 6  */
  double* smoothed_cov;      /* C = 36 (21 with CK_OUT_PACKED_COV) */
  double* jacobian;          /* C = 36, transport from the previous state   */
  /* per track [C * n_tracks], element c of track t at [c * n_tracks + t]:
   * the track's parameters and covariance at the reference surface
   * (TrackProxy::parameters / covariance after the extrapolation); written
   * when options.reference_surface >= 0 */
  double* track_params;      /* C = 6  */
  double* track_cov;         /* C = 36 */
} ck_batch_out;

/* Fills the reference defaults (see ck_options). Replaces the default member
 * initialisers of the reference option structs. */
void ck_options_default(ck_options* opt);

/* Library and device information. */
int32_t ck_api_version(void);
const char* ck_status_string(ck_status s);
const char* ck_last_error(void); /* thread-local message of the last failure */

/* Creates a fitter handle: uploads the surface table and the field, creates
 * the handle's stream and loads (or runs) the autotuner. Replaces the
 * construction of KalmanFitter<Propagator<EigenStepper, DirectNavigator>>
 * with its field provider (KalmanFitter.hpp:264-269, EigenStepper.ipp:20-22). */
ck_status ck_create(const ck_config* cfg, ck_handle** out);
ck_status ck_destroy(ck_handle* h);

/* Fits every track of the batch: forward Kalman filter, then the RTS
 * gain-matrix smoother (KalmanFitter::fit_impl, KalmanFitter.hpp:859-984),
 * for the declared extension set (pass-through calibrator, GainMatrixUpdater,
 * GainMatrixSmoother, predicted-chi2 outlier finder). Asynchronous on
 * `stream` (NULL = the handle's stream); host-memory batches are staged
 * through the handle's device buffers, and successive calls of one handle
 * run on the device in call order, whatever their streams. Call ck_sync()
 * (or synchronize `stream`) before reading host outputs, and keep host
 * inputs unchanged until then. */
ck_status ck_fit_batch(ck_handle* h, const ck_options* opt,
                       const ck_batch_in* in, ck_batch_out* out, void* stream);
ck_status ck_sync(ck_handle* h);

/* ck_fit_batch for a device-resident batch (in->memory and out->memory both
 * CK_MEM_DEVICE) that allocates nothing: the pipeline scratch is one
 * statically sized device array (ck_static_scratch_capacity() bytes, 32 MiB)
 * per device, shared by all handles. For callers that must not call the
 * device allocator once running (cudaMalloc/cudaFree can synchronise the
 * device; ck_fit_batch grows its buffers on demand). A batch needing more
 * than the array (ck_static_scratch_bytes_for) fails with CK_ERR_SCRATCH_LIMIT.
 * Nothing in the array has to start at zero. Calls whose device work
 * overlaps (other streams or handles on the same device, unordered) race on
 * the array. Make the first call before capturing the stream: it resolves
 * the array's address. No counterpart in the reference. */
ck_status ck_fit_batch_static(ck_handle* h, const ck_options* opt,
                              const ck_batch_in* in, ck_batch_out* out, void* stream);
/* Scratch bytes ck_fit_batch_static needs for a batch (-1 on bad sizes), and
 * the size of the static array. No counterpart in the reference.
 * ck_static_scratch_bytes counts the records, queue and tips only: a call
 * with a reference surface (options.reference_surface >= 0), reverse
 * filtering or a reverse-filtering momentum threshold also holds two
 * extrapolation start states per track (448 bytes), and every area is
 * rounded up to 256 bytes. ck_static_scratch_bytes_for gives the exact
 * figure a call with these options checks against the capacity (-1 on bad
 * sizes or invalid options). */
int64_t ck_static_scratch_bytes(int32_t n_tracks, int32_t max_states, int32_t precision);
int64_t ck_static_scratch_bytes_for(const ck_options* options, int32_t n_tracks,
                                    int32_t max_states);
int64_t ck_static_scratch_capacity(void);

/* Kernel-only timing of the most recent batch (CUDA events recorded on the
 * launching stream around the fit kernel): milliseconds. */
ck_status ck_last_kernel_ms(ck_handle* h, double* ms);

/* The same split into the forward-filter kernel and the smoother kernel
 * (milliseconds each). */
ck_status ck_last_kernel_split_ms(ck_handle* h, double* filter_ms, double* smoother_ms);

/* Number of kernels launched by the most recent ck_fit_batch call. */
ck_status ck_last_launch_count(ck_handle* h, int32_t* n);

/* Host<->device bytes moved by the most recent ck_fit_batch call (0 for
 * device-resident batches). */
ck_status ck_last_transfer_bytes(ck_handle* h, int64_t* h2d_bytes,
                                 int64_t* d2h_bytes);

/* Launch shape of the fit kernel (after autotuning). */
ck_status ck_get_launch_config(ck_handle* h, int32_t precision,
                               int32_t* threads_per_block,
                               int32_t* blocks_per_sm);
/* The RTS smoother kernel of a precision form: 0 reads each state's record
 * per lane from global memory, 1 stages the records of a warp's 32 tracks in
 * shared memory with coalesced warp-wide copies first (gain-matrix smoother;
 * the MbfSmoother always reads per lane). Results are identical. */
ck_status ck_set_smoother_staging(ck_handle* h, int32_t precision, int32_t enable);
/* The forward-filter kernel variant of a precision form (see
 * ck_set_launch_config) and its Runge-Kutta trials per scheduling round. */
ck_status ck_get_launch_variant(ck_handle* h, int32_t precision, int32_t* variant,
                                int32_t* steps_per_round);

/* Pins the launch shape of the forward-filter kernel: variant (0-2
 * per-warp phase scheduling with register caps of 255 / 168 / 128 per
 * thread and any multiple of 32 up to 128 threads per block; 3 and 4
 * block-level phase compaction with 256 and 128 threads per block; 5-6
 * warp-autonomous phase pools with 256 threads per block and more track
 * slots than threads),
 * threads per block and resident blocks per SM. */
ck_status ck_set_launch_config(ck_handle* h, int32_t precision, int32_t variant,
                               int32_t threads_per_block, int32_t blocks_per_sm);

/* Runge-Kutta trials a track may take per scheduling round of the
 * block-compaction kernels, for one precision (1..64; defaults 2 for FP64,
 * 3 for mixed; the autotuner also sweeps it). Results do not depend on it.
 * No counterpart in the reference (a scheduling knob of this implementation). */
ck_status ck_set_steps_per_round(ck_handle* h, int32_t precision, int32_t steps);

/* Grid of the forward-filter kernel in blocks for one precision (0, the
 * default: SMs x resident blocks per SM, the whole GPU). A smaller grid
 * leaves SMs free for fits launched at the same time on other streams (the
 * serving loop's concurrent co-batches). Results do not depend on it.
 * No counterpart in the reference (a scheduling knob of this implementation). */
ck_status ck_set_grid_blocks(ck_handle* h, int32_t precision, int32_t blocks);

/* Chunking of host-memory batches (both sides in host memory): a batch of at
 * least two chunks is fitted chunk by chunk while the inputs of the next
 * chunk and the outputs of the previous one travel on copy streams. `tracks`:
 * tracks per chunk (0: the default, 500000; a negative value: never chunk).
 * Results do not depend on it. */
ck_status ck_set_host_chunk_tracks(ck_handle* h, int32_t tracks);

/* Enables (default) or disables ordering the work queue by descending
 * surface-sequence length before the fit. */
ck_status ck_sort_queue(ck_handle* h, int32_t enable);

/* Enables (default) or disables smoothing in the forward filter's tail: in
 * the compaction kernels, a block whose tracks have all ended smooths
 * finished tracks of the batch while the last tracks are still propagating;
 * the smoother kernel takes the rest. Results do not depend on it. Not with
 * reverse filtering. No counterpart in the reference (a scheduling knob). */
ck_status ck_set_tail_smoothing(ck_handle* h, int32_t enable);

/* Text log of the last autotuner sweep (variant, block, blocks/SM, ms). */
const char* ck_autotune_log(ck_handle* h);

/* Measured peak of the FP64 (precision = CK_PRECISION_FP64) or FP32 FMA
 * pipe on the handle's device, in GFLOP/s (FMA = 2 flops), from a
 * dependent-chain-free FMA loop timed with CUDA events. */
ck_status ck_fp_peak_gflops(ck_handle* h, int32_t precision, double* gflops);

/* sizeof() of ck_surface, ck_field, ck_options, ck_config, ck_batch_in,
 * ck_batch_out, ck_server_config, ck_propagate_in, ck_propagate_out,
 * ck_ckf_options, ck_ckf_in, ck_ckf_out (in that order; the first n), for
 * binding checks. */
void ck_abi_struct_sizes(int64_t* out, int32_t n);

/* Runs the autotuner for `precision` on the given device-resident batch:
 * sweeps threads per block and resident blocks per SM, times each variant
 * with CUDA events and stores the fastest in the handle (and the cache file
 * given at creation). */
ck_status ck_autotune(ck_handle* h, const ck_options* opt,
                      const ck_batch_in* in_device, ck_batch_out* out_device);

/* ---------------------------------------------- unit operators (batched) */

/* GainMatrixUpdater::operator() on a batch of track states
 * (Core/include/Acts/TrackFitting/detail/GainMatrixUpdaterImpl.hpp:21-91):
 * N = 2 (loc0, loc1), or N = 1 where subspace[i] (CK_MEAS_*, NULL = all
 * 2D) selects one local coordinate. Arrays are AoS per state:
 * predicted[6], predicted_cov[36], meas[2], meas_cov[4] (1D: meas[0],
 * meas_cov[0]); outputs filtered[6], filtered_cov[36], chi2[1], status[1]
 * (CK_TRACK_OK or CK_TRACK_UPDATE_FAILED). Host pointers; synchronous. */
ck_status ck_gain_matrix_update(ck_handle* h, int32_t n, int32_t use_joseph,
                                const double* predicted,
                                const double* predicted_cov,
                                const double* meas, const double* meas_cov,
                                const int32_t* subspace,
                                double* filtered, double* filtered_cov,
                                double* chi2, int32_t* status);

/* GainMatrixSmoother::operator() (Core/include/Acts/TrackFitting/
 * GainMatrixSmoother.hpp:43-99, Core/src/TrackFitting/GainMatrixSmoother.cpp
 * :18-97) on n_traj independent trajectories of n_states each, in forward
 * order; AoS per state: predicted[6], predicted_cov[36], filtered[6],
 * filtered_cov[36], jacobian[36]; outputs smoothed[6], smoothed_cov[36];
 * status per trajectory. Host pointers; synchronous. */
ck_status ck_gain_matrix_smooth(ck_handle* h, int32_t n_traj, int32_t n_states,
                                const double* predicted,
                                const double* predicted_cov,
                                const double* filtered,
                                const double* filtered_cov,
                                const double* jacobian, double* smoothed,
                                double* smoothed_cov, int32_t* status);

/* MbfSmoother::operator() (Core/include/Acts/TrackFitting/MbfSmoother.hpp
 * :48-90, Core/src/TrackFitting/MbfSmoother.cpp:17-48,
 * detail/MbfSmootherImpl.hpp:17-58) on n_traj independent trajectories of
 * n_states each, in forward order, smoothed backwards from the last state:
 * flags[k] (CK_FLAG_*; a state with a measurement that is not an outlier is
 * visited as a measurement with the (loc0, loc1) projector), AoS per state:
 * predicted[6], predicted_cov[36], filtered[6], filtered_cov[36],
 * jacobian[36] (transport from the previous state), measurement[2],
 * measurement_cov[4]; outputs smoothed[6], smoothed_cov[36]. FP64. Host
 * pointers; synchronous. */
ck_status ck_mbf_smooth(ck_handle* h, int32_t n_traj, int32_t n_states,
                        const uint32_t* flags, const double* predicted,
                        const double* predicted_cov, const double* filtered,
                        const double* filtered_cov, const double* jacobian,
                        const double* measurement, const double* measurement_cov,
                        double* smoothed, double* smoothed_cov);

/* The mixed form's FP64 atan2 (table-driven argument reduction; used for
 * the bound angles and the cylinder loc0) on a batch: out[i] = atan2(y[i],
 * x[i]). Host pointers; synchronous. No counterpart in the reference (it
 * stands for std::atan2 in transformFreeToBoundParameters,
 * TransformationHelpers.cpp:41-63). */
ck_status ck_atan2_mixed(ck_handle* h, int32_t n, const double* y, const double* x,
                         double* out);

/* Pointwise material effects (computeMaterialEffects,
 * Core/src/Propagator/detail/PointwiseMaterialInteraction.cpp:49-90) for a
 * batch of (slab, direction, q/p) inputs on the device: per input the
 * surface id (its slab, scaled by `thickness_scale`), direction[3], q/p,
 * mass, |q|, pdg; outputs eLoss, variancePhi, varianceTheta, varianceQOverP
 * as double[4]. Host pointers; synchronous. */
ck_status ck_material_effects(ck_handle* h, int32_t n, const int32_t* surface,
                              const float* thickness_scale,
                              const double* direction, const double* qop,
                              const float* mass, const float* abs_q,
                              const int32_t* pdg, int32_t multiple_scattering,
                              int32_t energy_loss, double* effects);

/* Field lookup on the device for n positions (getField of the handle's
 * field); out[3*n] in GeV/(e*mm); status per point. Host pointers. */
ck_status ck_field_lookup(ck_handle* h, int32_t n, const double* pos,
                          double* out, int32_t* status);
/* The same lookup in a precision form's stepper arithmetic: FP64, or the
 * mixed form's FP32 lookup (positions rounded to float, trilinear weights
 * and interpolation in float) that its Runge-Kutta stages evaluate. */
ck_status ck_field_lookup_precision(ck_handle* h, int32_t precision, int32_t n,
                                    const double* pos, double* out, int32_t* status);

/* ------------------------------------------------------- propagation */
/* A batch of independent propagations of bound track parameters with the
 * fitter's stepper (the same Runge-Kutta, transport and intersection code as
 * the fit, in the options' precision form):
 *   Propagator<EigenStepper<>, VoidNavigator>::propagate(start, options) and
 *   ::propagate(start, target, options)
 *   (Core/include/Acts/Propagator/Propagator.ipp:25-260) with the
 *   SurfaceReached aborter on the target (StandardAborters.hpp:66-155) and
 *   PathLimitReached with loop protection (StandardAborters.hpp:24-62,
 *   detail/LoopProtection.hpp:19-72); no actors, no material.
 * Each propagation runs in the direction of the sign of its path limit (a
 * target is reached forward with a positive limit). With a target its end
 * parameters are bound on the target (Propagator::makeResult's boundState);
 * without one they are curvilinear at the end point (loc0 = loc1 = 0 on the
 * plane through the end point normal to the direction, its frame the
 * curvilinear unit vectors of UnitVectors.hpp:94-150), and the frame is
 * returned in end_frames, so that the result can start another propagation.
 * Options used: precision, step_tolerance, step_size_cutoff,
 * initial_step_size, max_step_size, max_rk_step_trials, max_steps,
 * loop_protection, loop_fraction, surface_tolerance. Per-track status as the
 * fit's (CK_TRACK_*). Inputs use the per-track layout of ck_batch_in,
 * outputs the structure-of-arrays layout of ck_batch_out's track_params
 * (element c of track t at [c * n + t]). */
typedef struct ck_propagate_in {
  int32_t n;
  int32_t memory;              /* CK_MEM_HOST or CK_MEM_DEVICE (inputs and outputs) */
  const double* start_params;  /* [n*6] bound parameters on the start plane  */
  const double* start_cov;     /* [n*36] row-major, or NULL: no covariance   */
  const double* start_frames;  /* [n*12] start plane as in ck_batch_in        */
  const float* particle;       /* [n*2] (mass GeV, |q|)                       */
  const int32_t* target;       /* [n] surface-table index of the target
                                  (plane, cylinder or line), -1: none; NULL:
                                  no targets                                  */
  const double* path_limit;    /* [n] signed path limit (mm)                  */
} ck_propagate_in;

typedef struct ck_propagate_out {
  int32_t* status;       /* [n] CK_TRACK_*                                     */
  double* end_params;    /* [6][n] bound parameters at the end                 */
  double* end_cov;       /* [36][n] transported covariance, or NULL            */
  double* jacobian;      /* [36][n] bound-to-bound transport Jacobian from the
                            start surface to the end surface, or NULL          */
  double* end_frames;    /* [n*12] the end plane of a propagation without a
                            target (ck_batch_in layout), or NULL               */
  double* path_length;   /* [n] signed path length, or NULL                    */
  int32_t* steps;        /* [n] accepted Runge-Kutta steps, or NULL            */
} ck_propagate_out;

ck_status ck_propagate(ck_handle* h, const ck_options* options, const ck_propagate_in* in,
                       ck_propagate_out* out, void* stream);

/* ------------------------------------------- combinatorial track finding */
/* Combinatorial Kalman filter track finding from seeds:
 *   CombinatorialKalmanFilter<Propagator<EigenStepper<>, DirectNavigator>,
 *       TrackContainer>::findTracks(initialParameters, options, tracks)
 *   (Core/include/Acts/TrackFinding/CombinatorialKalmanFilter.hpp:1191-1335,
 *    Actor::act / filter / reset / processNewTrackStates :250-900)
 * with the default TrackStateCreator and MeasurementSelector
 * (TrackStateCreator.hpp:60-310, MeasurementSelector.ipp:19-124) and the
 * examples' branch stopper (Examples/Algorithms/TrackFinding/src/
 * TrackFindingAlgorithm.cpp:185-261), on the fitter's stepper, navigator and
 * updater in the options' precision form. Each seed follows its surface
 * sequence (the DirectNavigator's); on a sensitive surface the measurements
 * of that surface are the candidates: their predicted chi2 against the cut
 * selects up to max_candidates (ascending chi2), each opening a branch
 * (depth-first, the best first); none selected: the best becomes an outlier
 * when its chi2 is below chi2_cut_outlier, else a hole. A branch ends on the
 * target surface (its bound parameters become the track's), at the
 * loop-protection path limit, or when the branch stopper stops it (kept
 * with enough measurements); every branch that ends kept is a found track.
 * Material-only surfaces in a sequence are not supported (the track fails
 * with CK_TRACK_INVALID_INPUT). Errors of a seed's search (stepper, field,
 * the propagator's step limit over all its branches, a capacity below)
 * fail the seed: status set, no tracks. */
typedef struct ck_ckf_options {
  double chi2_cut;           /* MeasurementSelectorCuts::chi2CutOff (15)          */
  double chi2_cut_outlier;   /* chi2CutOffOutlier (+inf: always an outlier)       */
  int32_t max_candidates;    /* numMeasurementsCutOff (1)                         */
  int32_t min_measurements;  /* branch stopper: TrackSelector cuts (0, and       */
  int32_t max_holes;         /*   INT32_MAX for the maxima: no stopping)          */
  int32_t max_outliers;
  int32_t max_holes_and_outliers;
  int32_t target_surface;    /* CombinatorialKalmanFilterOptions::targetSurface:
                                a plane or cylinder of the table; -1: none     */
  int32_t max_states;        /* track-state capacity per seed (64)               */
  int32_t max_tracks;        /* found-track capacity per seed (16)               */
  int32_t max_branches;      /* active-branch capacity per seed (16)             */
  int32_t end_of_world;      /* 1: a branch ends (kept) as soon as the navigator
                                has no surface of the seed's sequence left
                                ahead, before a further step, as the end of
                                the world ends it with the reference's
                                geometry Navigator; 0 (default): the
                                DirectNavigator's behaviour, where only the
                                loop protection, the target or the stopper end
                                a branch (without a field and a target the
                                seed runs into the step limit; on a field map
                                it may leave the map)                          */
  int32_t lanes_per_seed;    /* GPU lanes that share a seed's search: 0 or 1
                                (default): one lane, whose candidate search
                                walks outward from the prediction over the
                                surface's candidates sorted along a measured
                                axis; 2, 4, 8, 16 or 32: the lanes split a full
                                scan of every surface (for few seeds on
                                surfaces with many candidates). The selection
                                is the same; floating-point values agree to
                                the parity tolerance (each kernel instance
                                contracts multiply-adds its own way). No
                                counterpart in the reference (a scheduling
                                knob)                                          */
  int32_t reserved;
} ck_ckf_options;

void ck_ckf_options_default(ck_ckf_options* options);

/* Seeds (start parameters on a plane, as ck_batch_in) with their surface
 * sequences, and the events' measurements grouped by event and surface: the
 * candidates of seed i on surface s are the measurements
 * [surf_meas_offsets[e*n_surfaces + s], surf_meas_offsets[e*n_surfaces + s + 1])
 * of its event e = seed_event[i], in the caller's order (the candidate
 * order). One call searches the seeds of many events; each seed sees only
 * its event's measurements. */
typedef struct ck_ckf_in {
  int32_t n_seeds;
  int32_t memory;                    /* CK_MEM_HOST or CK_MEM_DEVICE (in and out) */
  const int32_t* seq_offsets;        /* [n_seeds+1]                            */
  const int32_t* seq_surfaces;
  const double* start_params;        /* [n_seeds*6]                            */
  const double* start_cov;           /* [n_seeds*36]                           */
  const double* start_frames;        /* [n_seeds*12]                           */
  const float* particle;             /* [n_seeds*2] (mass GeV, |q|)            */
  const int32_t* particle_pdg;       /* [n_seeds] or NULL (211)                */
  int32_t n_meas;
  int32_t n_surfaces;                /* the handle's table size                */
  const int32_t* surf_meas_offsets;  /* [n_events*n_surfaces+1]                 */
  const double* meas_values;         /* [n_meas*2] (1D: first slot)            */
  const double* meas_cov;            /* [n_meas*4]                             */
  const int32_t* meas_subspace;      /* [n_meas] CK_MEAS_*, or NULL (all 2D)   */
  int32_t n_events;                  /* events in the call (0 counts as 1)     */
  const int32_t* seed_event;         /* [n_seeds] event of each seed, or NULL
                                        (all in event 0)                       */
} ck_ckf_in;

/* Results (entries beyond a seed's n_tracks / n_states are unspecified).
 * Per seed s: its found tracks k < n_tracks[s] at [s*max_tracks + k]
 * (the order the search keeps them in) and its track states i < n_states[s]
 * at [s*max_states + i] (creation order; a track is the chain of states from
 * its tip back along state_prev). Vector and matrix arrays hold C values per
 * element: element c of state i of seed s at [(s*max_states + i)*C + c];
 * covariances packed as upper triangles (C = 21), Jacobians C = 36. */
typedef struct ck_ckf_out {
  int32_t* status;                /* [n_seeds] CK_TRACK_*                      */
  int32_t* n_tracks;              /* [n_seeds]                                 */
  int32_t* n_states;              /* [n_seeds]                                 */
  int32_t* track_tip;             /* state index of the track's last state     */
  int32_t* track_n_measurements;
  int32_t* track_n_holes;
  int32_t* track_n_outliers;
  int32_t* track_ndf;
  double* track_chi2;
  double* track_params;           /* C = 6 on the target surface (NaN: none)   */
  double* track_cov;              /* C = 21                                    */
  int32_t* state_prev;            /* previous state of the branch, -1: first   */
  int32_t* state_surface;
  uint32_t* state_flags;          /* CK_FLAG_*                                 */
  int32_t* state_measurement;     /* measurement index, -1 for holes            */
  double* state_chi2;             /* measurement states: the filtered chi2;
                                     outliers: the predicted chi2              */
  double* state_path_length;
  double* predicted;              /* C = 6 */
  double* predicted_cov;          /* C = 21 */
  double* filtered;               /* C = 6 (outliers and holes: predicted)     */
  double* filtered_cov;           /* C = 21 */
  double* jacobian;               /* C = 36, transport from the previous state */
} ck_ckf_out;

ck_status ck_find_tracks(ck_handle* h, const ck_options* options,
                         const ck_ckf_options* ckf, const ck_ckf_in* in,
                         ck_ckf_out* out, void* stream);

/* Lanes per seed of the handle's last ck_find_tracks launch (0: none yet). */
int32_t ck_last_ckf_lanes(ck_handle* h);

/* ------------------------------------------- event generation on device */
/* Truth simulation and digitisation of tracks [first_track, first_track +
 * n_tracks) of a generator preset (ckgen.h: CKG_*) through the handle's
 * surface table and field, on the GPU: the Fatras-like simulation of the
 * host generator ckg_generate (a fixed-step RK4 truth trajectory, Highland
 * kicks and Bethe loss at the material layers, smeared measurements, holes
 * and outliers as the preset asks), from the same source, one thread per
 * track. `out` holds DEVICE pointers in ckg_out's layout (struct ckg_out,
 * ckgen.h; compact CSR rows with their offsets, at most max_per_track rows
 * per track); asynchronous on `stream` (NULL: the handle's). Results are
 * the host generator's up to floating-point rounding: the device's own
 * libm and multiply-add contraction. */
struct ckg_out;
ck_status ck_simulate(ck_handle* h, int32_t preset, uint64_t seed, int64_t first_track,
                      int32_t n_tracks, struct ckg_out* out, void* stream);

/* ------------------------------------------------------------- serving */

/* Continuous-batching serving loop (host request thread + device-resident
 * slot pool). Events are admitted against `memory_budget_bytes` as slots and
 * memory free up; admitted events are co-batched and their fits overlap on
 * the device across `n_streams` streams. */
typedef struct ck_server ck_server;

typedef struct ck_server_config {
  int64_t memory_budget_bytes; /* device memory the pool may hold           */
  int32_t n_streams;           /* concurrent batches in flight              */
  int32_t max_states;          /* per-track state capacity                  */
  int32_t max_batch_tracks;    /* largest co-batch                          */
  uint32_t components;         /* CK_OUT_* written back to the host         */
  /* Launch shape of the co-batches (0: automatic). grid_blocks: blocks of
   * each co-batch's forward-filter grid; automatic = the whole GPU divided by
   * (n_streams - 1), so that a co-batch admitted while others run starts on
   * free SMs at once instead of behind their blocks. steps_per_round:
   * Runge-Kutta trials per scheduling round; automatic = 6, the measured
   * best for 10k-track events (latency), where large offline batches prefer
   * 2-3 (throughput). Neither changes results. */
  int32_t grid_blocks;
  int32_t steps_per_round;
} ck_server_config;

ck_status ck_server_create(ck_handle* h, const ck_options* opt,
                           const ck_server_config* cfg, ck_server** out);
/* Queues one event. `event` (its inputs) and `results` (its output arrays,
 * laid out as ck_batch_out for event->n_tracks tracks with the server's
 * max_states; only components the server computes) stay owned by the
 * caller and must stay valid until ck_server_poll has returned the event;
 * nothing is copied at submission. Either may be in host memory (pageable
 * or page-locked) or device memory: results are copied straight into
 * `results` (pageable host results through a page-locked staging buffer).
 * Returns CK_ERR_BUDGET when the event alone exceeds a stream's capacity. */
ck_status ck_server_submit(ck_server* s, int64_t event_id,
                           const ck_batch_in* event, const ck_batch_out* results);
/* Pops one finished event: its id and latency in ms (submit until its
 * results are in place). CK_ERR_NOT_READY when none has finished within
 * timeout_ms; another status when the event's batch failed (its results are
 * then not written). */
ck_status ck_server_poll(ck_server* s, int64_t* event_id, double* latency_ms,
                         int32_t timeout_ms);
/* Counters: events submitted, completed, tracks completed, bytes in use. */
ck_status ck_server_stats(ck_server* s, int64_t* submitted, int64_t* completed,
                          int64_t* tracks, int64_t* bytes_in_use);
/* Tracks one stream slot can hold (the largest event accepted). */
int32_t ck_server_capacity(ck_server* s);
ck_status ck_server_destroy(ck_server* s);

#ifdef __cplusplus
}
#endif

#endif /* CUDAKALMAN_H */
