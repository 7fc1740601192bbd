// ActsPlugins/CudaKalman.hpp — C++ facade of the CudaKalman fitter.
//
// Header-only host code over the C ABI (include/cudakalman.h). It mirrors
// the call a reference user makes,
//
//   Acts::KalmanFitter<Propagator<EigenStepper<>, DirectNavigator>,
//                      VectorMultiTrajectory>::fit(begin, end, startParameters,
//                                                  kfOptions, sSequence,
//                                                  trackContainer)
//   (Core/include/Acts/TrackFitting/KalmanFitter.hpp:719-731)
//
// with the same argument meaning: an iterator range of source links, bound
// start parameters, the fit options, the DirectNavigator surface sequence and
// a track container the fitted track and its states are appended to; it
// returns a Result that holds either the new track's index or the error the
// reference would return. fitBatch() takes many tracks at once (the per-track
// loop of TrackFittingAlgorithm::execute,
// Examples/Algorithms/TrackFitting/src/TrackFittingAlgorithm.cpp:117-170).
// findTracks() is CombinatorialKalmanFilter::findTracks
// (Core/include/Acts/TrackFinding/CombinatorialKalmanFilter.hpp:1191-1335)
// for many seeds of one or more events at once, with the default
// MeasurementSelector and the examples' branch stopper.
//
// The ACTS types this build cannot include (Eigen/Boost are not available)
// are represented by small structs with the same fields; a build against a
// real ACTS installation maps Acts::BoundTrackParameters, SourceLink and
// VectorMultiTrajectory onto them one to one.
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <system_error>
#include <vector>

#include "cudakalman.h"

namespace ActsPlugins {

// Track-level errors, mirroring Acts::KalmanFitterError / PropagatorError /
// EigenStepperError / SurfaceError / MagneticFieldError by name.
enum class CudaKalmanError : int {
  UpdateFailed = CK_TRACK_UPDATE_FAILED,
  SmoothFailed = CK_TRACK_SMOOTH_FAILED,
  NoMeasurementFound = CK_TRACK_NO_MEASUREMENT_FOUND,
  StepCountLimitReached = CK_TRACK_STEP_COUNT_LIMIT,
  NextTargetLimitReached = CK_TRACK_NEXT_TARGET_LIMIT,
  StepSizeStalled = CK_TRACK_STEP_SIZE_STALLED,
  StepSizeAdjustmentFailed = CK_TRACK_STEP_ADJUST_FAILED,
  GlobalPositionNotOnSurface = CK_TRACK_NOT_ON_SURFACE,
  MagneticFieldOutOfBounds = CK_TRACK_FIELD_OUT_OF_BOUNDS,
  TooManyStates = CK_TRACK_TOO_MANY_STATES,
  NotProcessed = CK_TRACK_NOT_PROCESSED,
  InvalidInput = CK_TRACK_INVALID_INPUT,
};

inline const char* errorName(int code) {
  switch (code) {
    case CK_TRACK_UPDATE_FAILED: return "UpdateFailed";
    case CK_TRACK_SMOOTH_FAILED: return "SmoothFailed";
    case CK_TRACK_NO_MEASUREMENT_FOUND: return "NoMeasurementFound";
    case CK_TRACK_STEP_COUNT_LIMIT: return "StepCountLimitReached";
    case CK_TRACK_NEXT_TARGET_LIMIT: return "NextTargetLimitReached";
    case CK_TRACK_STEP_SIZE_STALLED: return "StepSizeStalled";
    case CK_TRACK_STEP_ADJUST_FAILED: return "StepSizeAdjustmentFailed";
    case CK_TRACK_NOT_ON_SURFACE: return "GlobalPositionNotOnSurface";
    case CK_TRACK_FIELD_OUT_OF_BOUNDS: return "MagneticFieldOutOfBounds";
    case CK_TRACK_TOO_MANY_STATES: return "TooManyStates";
    case CK_TRACK_NOT_PROCESSED: return "NotProcessed";
    case CK_TRACK_INVALID_INPUT: return "InvalidInput";
    case CK_TRACK_NO_COMPATIBLE_STATE: return "CompatibleTrackStateNotFound";
    case CK_TRACK_REFERENCE_UNREACHABLE: return "ReferenceSurfaceUnreachable";
    case CK_TRACK_INCONSISTENT_STATES: return "InconsistentTrackStates";
    default: return "ok";
  }
}

// Acts::Result<T> analogue: a value or an error code.
template <typename T>
class Result {
 public:
  static Result success(T v) { return Result(std::move(v), 0); }
  static Result failure(int e) { return Result(T{}, e); }
  bool ok() const { return m_error == 0; }
  const T& value() const {
    if (!ok())
      throw std::runtime_error(std::string("Result has error ") + ActsPlugins::errorName(m_error));
    return m_value;
  }
  int error() const { return m_error; }
  const char* errorName() const { return ActsPlugins::errorName(m_error); }

 private:
  Result(T v, int e) : m_value(std::move(v)), m_error(e) {}
  T m_value;
  int m_error;
};

using BoundVector = std::array<double, 6>;
using BoundMatrix = std::array<double, 36>;  // row-major

// Acts::BoundTrackParameters on a plane surface, with its particle
// hypothesis (EventData/BoundTrackParameters.hpp, ParticleHypothesis.hpp).
struct BoundTrackParameters {
  BoundVector parameters{};      // loc0, loc1, phi, theta, q/p, t
  BoundMatrix covariance{};      // row-major
  std::array<double, 9> planeRotation{1, 0, 0, 0, 1, 0, 0, 0, 1};  // columns = local axes
  std::array<double, 3> planeCenter{0, 0, 0};
  float mass = 0.13957039f;      // GeV (float, as ParticleHypothesis stores it)
  float absCharge = 1.0f;
  int absPdg = 211;
};

// A source link after the pass-through calibrator: a 2D measurement on
// (loc0, loc1) of a surface (TestSourceLink + testSourceLinkCalibrator).
struct SourceLink {
  int surface = -1;
  std::array<double, 2> value{};       // 1D: value[0]
  std::array<double, 4> covariance{};  // row-major 2x2; 1D: covariance[0]
  // measured local coordinates (the calibrator's projector subspace):
  // CK_MEAS_LOC01 (pixel), CK_MEAS_LOC0 or CK_MEAS_LOC1 (strip)
  int32_t subspace = CK_MEAS_LOC01;
};

// KalmanFitterOptions + plain stepper / propagator options.
struct KalmanFitterOptions {
  ck_options options;
  KalmanFitterOptions() { ck_options_default(&options); }
};

// One track state as VectorMultiTrajectory stores it
// (EventData/VectorMultiTrajectory.hpp:187-200).
struct TrackState {
  int surface = -1;
  int sourceLink = -1;  // findTracks: index of the state's measurement in the input (-1: none)
  uint32_t typeFlags = 0;
  double pathLength = 0;
  double chi2 = 0;
  BoundVector predicted{}, filtered{}, smoothed{};
  BoundMatrix predictedCovariance{}, filteredCovariance{}, smoothedCovariance{}, jacobian{};
  bool isMeasurement() const {
    return (typeFlags & CK_FLAG_HAS_MEASUREMENT) && !(typeFlags & CK_FLAG_IS_OUTLIER);
  }
  bool isOutlier() const { return typeFlags & CK_FLAG_IS_OUTLIER; }
  bool isHole() const { return typeFlags & CK_FLAG_IS_HOLE; }
  // TrackStateProxy::hasSmoothed: with reverse filtering only the first and
  // the last measurement state carry smoothed parameters (NaN elsewhere)
  bool hasSmoothed() const { return smoothed[0] == smoothed[0]; }
};

// Minimal TrackContainer: tracks own a contiguous range of states in
// propagation order (trackStates() after linkForward()).
struct Track {
  size_t firstState = 0;
  size_t nStates = 0;
  size_t nMeasurements = 0, nHoles = 0, nOutliers = 0, nDoF = 0;
  double chi2 = 0;
  // TrackProxy::referenceSurface / parameters / covariance: set when the
  // options name a reference surface (the track extrapolated to it)
  int referenceSurface = -1;
  std::array<double, 6> parameters{};
  std::array<double, 36> covariance{};  // row-major
};

struct TrackContainer {
  std::vector<TrackState> states;
  std::vector<Track> tracks;
  const TrackState* trackStates(size_t track) const { return states.data() + tracks[track].firstState; }
};

// CombinatorialKalmanFilterOptions with the propagator options, the
// MeasurementSelector cuts (one bin) and the examples' branch stopper
// (TrackSelector::Config): ck_ckf_options (cudakalman.h).
struct CombinatorialKalmanFilterOptions {
  ck_options options;
  ck_ckf_options ckf;
  CombinatorialKalmanFilterOptions() {
    ck_options_default(&options);
    ck_ckf_options_default(&ckf);
  }
};

// One seed of a track-finding call: the initial parameters, the
// DirectNavigator surface sequence and the event whose measurements it sees.
struct SeedInput {
  BoundTrackParameters start;
  const int* surfaceSequence = nullptr;
  size_t nSurfaces = 0;
  int event = 0;
};

// One track of a batch.
struct TrackInput {
  const SourceLink* sourceLinks = nullptr;
  size_t nSourceLinks = 0;
  BoundTrackParameters start;
  const int* surfaceSequence = nullptr;
  size_t nSurfaces = 0;
};

class CudaKalman {
 public:
  struct Config {
    std::vector<ck_surface> surfaces;
    ck_field field{};
    int device = 0;
    bool useGraph = true;
    int maxStates = 64;
  };

  explicit CudaKalman(Config cfg) : m_cfg(std::move(cfg)) {
    ck_config c{};
    c.device = m_cfg.device;
    c.n_surfaces = static_cast<int32_t>(m_cfg.surfaces.size());
    c.surfaces = m_cfg.surfaces.data();
    c.field = m_cfg.field;
    c.use_graph = m_cfg.useGraph ? 1 : 0;
    ck_status s = ck_create(&c, &m_handle);
    if (s != CK_OK) throw std::runtime_error(std::string("ck_create: ") + ck_last_error());
  }
  ~CudaKalman() {
    if (m_handle) ck_destroy(m_handle);
  }
  CudaKalman(const CudaKalman&) = delete;
  CudaKalman& operator=(const CudaKalman&) = delete;

  // KalmanFitter::fit with a DirectNavigator surface sequence: a batch of one.
  template <typename source_link_iterator_t>
  Result<size_t> fit(source_link_iterator_t begin, source_link_iterator_t end,
                     const BoundTrackParameters& start, const KalmanFitterOptions& options,
                     const std::vector<int>& sSequence, TrackContainer& container) const {
    std::vector<SourceLink> links(begin, end);
    TrackInput in;
    in.sourceLinks = links.data();
    in.nSourceLinks = links.size();
    in.start = start;
    in.surfaceSequence = sSequence.data();
    in.nSurfaces = sSequence.size();
    std::vector<Result<size_t>> r = fitBatch(&in, 1, options, container);
    return r.front();
  }

  // Fits n tracks in one call; one Result (track index or error) per input.
  std::vector<Result<size_t>> fitBatch(const TrackInput* tracks, size_t n,
                                       const KalmanFitterOptions& options,
                                       TrackContainer& container) const {
    std::vector<int32_t> seqOff(n + 1, 0), measOff(n + 1, 0), seq, measSurf, measSub, pdg(n);
    std::vector<double> measVal, measCov, sp(6 * n), sc(36 * n), frames(12 * n);
    std::vector<float> part(2 * n);
    for (size_t t = 0; t < n; ++t) {
      const TrackInput& ti = tracks[t];
      for (size_t k = 0; k < ti.nSurfaces; ++k) seq.push_back(ti.surfaceSequence[k]);
      seqOff[t + 1] = static_cast<int32_t>(seq.size());
      for (size_t k = 0; k < ti.nSourceLinks; ++k) {
        const SourceLink& sl = ti.sourceLinks[k];
        measSurf.push_back(sl.surface);
        measSub.push_back(sl.subspace);
        measVal.insert(measVal.end(), sl.value.begin(), sl.value.end());
        measCov.insert(measCov.end(), sl.covariance.begin(), sl.covariance.end());
      }
      measOff[t + 1] = static_cast<int32_t>(measSurf.size());
      std::memcpy(&sp[6 * t], ti.start.parameters.data(), 6 * sizeof(double));
      std::memcpy(&sc[36 * t], ti.start.covariance.data(), 36 * sizeof(double));
      std::memcpy(&frames[12 * t], ti.start.planeRotation.data(), 9 * sizeof(double));
      std::memcpy(&frames[12 * t + 9], ti.start.planeCenter.data(), 3 * sizeof(double));
      part[2 * t] = ti.start.mass;
      part[2 * t + 1] = ti.start.absCharge;
      pdg[t] = ti.start.absPdg;
    }
    ck_batch_in in{};
    in.n_tracks = static_cast<int32_t>(n);
    in.memory = CK_MEM_HOST;
    in.seq_offsets = seqOff.data();
    in.seq_surfaces = seq.data();
    in.meas_offsets = measOff.data();
    in.meas_surfaces = measSurf.data();
    in.meas_values = measVal.data();
    in.meas_cov = measCov.data();
    in.start_params = sp.data();
    in.start_cov = sc.data();
    in.start_frames = frames.data();
    in.particle = part.data();
    in.particle_pdg = pdg.data();
    in.meas_subspace = measSub.data();

    const int ms = m_cfg.maxStates;
    const size_t S = static_cast<size_t>(ms) * n;
    std::vector<int32_t> status(n), nStates(n), nMeas(n), nHoles(n), nOut(n), ndf(n), surf(S);
    std::vector<uint32_t> flags(S);
    // covariances cross the boundary packed (upper triangles, 21 values) and
    // are unfolded into the container's full matrices below
    std::vector<double> chi2(n), path(S), schi2(S), pr(6 * S), prc(21 * S), fi(6 * S), fic(21 * S),
        sm(6 * S), smc(21 * S), jac(36 * S), tp(6 * n), tc(36 * n);
    const bool ref = options.options.reference_surface >= 0;
    ck_batch_out out{};
    out.max_states = ms;
    out.components = CK_OUT_PREDICTED | CK_OUT_FILTERED | CK_OUT_SMOOTHED | CK_OUT_JACOBIAN |
                     CK_OUT_PACKED_COV | (ref ? CK_OUT_REFERENCE : 0u);
    if (ref) {
      out.track_params = tp.data();
      out.track_cov = tc.data();
    }
    out.memory = CK_MEM_HOST;
    out.status = status.data();
    out.n_states = nStates.data();
    out.n_measurements = nMeas.data();
    out.n_holes = nHoles.data();
    out.n_outliers = nOut.data();
    out.ndf = ndf.data();
    out.chi2_sum = chi2.data();
    out.state_surface = surf.data();
    out.state_flags = flags.data();
    out.state_path_length = path.data();
    out.state_chi2 = schi2.data();
    out.predicted = pr.data();
    out.predicted_cov = prc.data();
    out.filtered = fi.data();
    out.filtered_cov = fic.data();
    out.smoothed = sm.data();
    out.smoothed_cov = smc.data();
    out.jacobian = jac.data();
    ck_status s = ck_fit_batch(m_handle, &options.options, &in, &out, nullptr);
    if (s == CK_OK) s = ck_sync(m_handle);
    if (s != CK_OK) throw std::runtime_error(std::string("ck_fit_batch: ") + ck_last_error());

    std::vector<Result<size_t>> results;
    results.reserve(n);
    auto at = [&](size_t k, size_t C, size_t c, size_t t) { return (k * C + c) * n + t; };
    for (size_t t = 0; t < n; ++t) {
      if (status[t] != CK_TRACK_OK) {
        results.push_back(Result<size_t>::failure(status[t]));
        continue;
      }
      Track tr;
      tr.firstState = container.states.size();
      tr.nStates = static_cast<size_t>(nStates[t]);
      tr.nMeasurements = static_cast<size_t>(nMeas[t]);
      tr.nHoles = static_cast<size_t>(nHoles[t]);
      tr.nOutliers = static_cast<size_t>(nOut[t]);
      tr.nDoF = static_cast<size_t>(ndf[t]);
      tr.chi2 = chi2[t];
      if (ref) {
        tr.referenceSurface = options.options.reference_surface;
        for (size_t c = 0; c < 6; ++c) tr.parameters[c] = tp[c * n + t];
        for (size_t c = 0; c < 36; ++c) tr.covariance[c] = tc[c * n + t];
      }
      for (size_t k = 0; k < tr.nStates; ++k) {
        TrackState st;
        st.surface = surf[at(k, 1, 0, t)];
        st.typeFlags = flags[at(k, 1, 0, t)];
        st.pathLength = path[at(k, 1, 0, t)];
        st.chi2 = schi2[at(k, 1, 0, t)];
        for (size_t c = 0; c < 6; ++c) {
          st.predicted[c] = pr[at(k, 6, c, t)];
          st.filtered[c] = fi[at(k, 6, c, t)];
          st.smoothed[c] = sm[at(k, 6, c, t)];
        }
        for (size_t i = 0, c = 0; i < 6; ++i)
          for (size_t j = i; j < 6; ++j, ++c) {
            const size_t u = i * 6 + j, l = j * 6 + i;
            st.predictedCovariance[u] = st.predictedCovariance[l] = prc[at(k, 21, c, t)];
            st.filteredCovariance[u] = st.filteredCovariance[l] = fic[at(k, 21, c, t)];
            st.smoothedCovariance[u] = st.smoothedCovariance[l] = smc[at(k, 21, c, t)];
          }
        for (size_t c = 0; c < 36; ++c) st.jacobian[c] = jac[at(k, 36, c, t)];
        container.states.push_back(st);
      }
      container.tracks.push_back(tr);
      results.push_back(Result<size_t>::success(container.tracks.size() - 1));
    }
    return results;
  }

  // Finds the tracks of n seeds among the measurements of their events
  // (measurementEvent[i]: the event of measurement i; NULL: all in event 0).
  // Every found track is appended to the container (its states in
  // propagation order, sourceLink set on measurement and outlier states,
  // smoothed parameters NaN: the search does not smooth); one Result per
  // seed: the container indices of its tracks, or the seed's error.
  std::vector<Result<std::vector<size_t>>> findTracks(
      const SeedInput* seeds, size_t n, const SourceLink* measurements, size_t nMeas,
      const CombinatorialKalmanFilterOptions& options, TrackContainer& container,
      int nEvents = 1, const int* measurementEvent = nullptr) const {
    const int nS = static_cast<int>(m_cfg.surfaces.size());
    const int nEv = nEvents < 1 ? 1 : nEvents;
    // measurements grouped by (event, surface), stable: the candidate order
    std::vector<int64_t> key(nMeas);
    std::vector<size_t> order(nMeas);
    std::vector<int32_t> offs(static_cast<size_t>(nEv) * nS + 1, 0);
    for (size_t i = 0; i < nMeas; ++i) {
      const int ev = measurementEvent ? measurementEvent[i] : 0;
      const int sf = measurements[i].surface;
      if (ev < 0 || ev >= nEv || sf < 0 || sf >= nS)
        throw std::invalid_argument("measurement event or surface out of range");
      key[i] = static_cast<int64_t>(ev) * nS + sf;
      ++offs[key[i] + 1];
    }
    for (size_t k = 1; k < offs.size(); ++k) offs[k] += offs[k - 1];
    {
      std::vector<int32_t> fill(offs.begin(), offs.end() - 1);
      for (size_t i = 0; i < nMeas; ++i) order[fill[key[i]]++] = i;
    }
    std::vector<double> mv(2 * nMeas), mc(4 * nMeas);
    std::vector<int32_t> msub(nMeas);
    for (size_t j = 0; j < nMeas; ++j) {
      const SourceLink& sl = measurements[order[j]];
      mv[2 * j] = sl.value[0];
      mv[2 * j + 1] = sl.value[1];
      for (int c = 0; c < 4; ++c) mc[4 * j + c] = sl.covariance[c];
      msub[j] = sl.subspace;
    }
    std::vector<int32_t> seqOff(n + 1, 0), seq, pdg(n), sev(n);
    std::vector<double> sp(6 * n), sc(36 * n), frames(12 * n);
    std::vector<float> part(2 * n);
    for (size_t t = 0; t < n; ++t) {
      const SeedInput& si = seeds[t];
      for (size_t k = 0; k < si.nSurfaces; ++k) seq.push_back(si.surfaceSequence[k]);
      seqOff[t + 1] = static_cast<int32_t>(seq.size());
      std::memcpy(&sp[6 * t], si.start.parameters.data(), 6 * sizeof(double));
      std::memcpy(&sc[36 * t], si.start.covariance.data(), 36 * sizeof(double));
      std::memcpy(&frames[12 * t], si.start.planeRotation.data(), 9 * sizeof(double));
      std::memcpy(&frames[12 * t + 9], si.start.planeCenter.data(), 3 * sizeof(double));
      part[2 * t] = si.start.mass;
      part[2 * t + 1] = si.start.absCharge;
      pdg[t] = si.start.absPdg;
      sev[t] = si.event;
    }
    ck_ckf_in in{};
    in.n_seeds = static_cast<int32_t>(n);
    in.memory = CK_MEM_HOST;
    in.seq_offsets = seqOff.data();
    in.seq_surfaces = seq.data();
    in.start_params = sp.data();
    in.start_cov = sc.data();
    in.start_frames = frames.data();
    in.particle = part.data();
    in.particle_pdg = pdg.data();
    in.n_meas = static_cast<int32_t>(nMeas);
    in.n_surfaces = nS;
    in.surf_meas_offsets = offs.data();
    in.meas_values = mv.data();
    in.meas_cov = mc.data();
    in.meas_subspace = msub.data();
    in.n_events = nEv;
    in.seed_event = sev.data();
    const size_t T = static_cast<size_t>(options.ckf.max_tracks) * n;
    const size_t S = static_cast<size_t>(options.ckf.max_states) * n;
    std::vector<int32_t> status(n), nTr(n), nSt(n), tip(T), tnm(T), tnh(T), tno(T), tndf(T),
        prev(S), surf(S), meas(S);
    std::vector<uint32_t> flags(S);
    std::vector<double> tchi2(T), tpar(6 * T), tcov(21 * T), schi2(S), path(S), pr(6 * S),
        prc(21 * S), fi(6 * S), fic(21 * S), jac(36 * S);
    ck_ckf_out out{};
    out.status = status.data();
    out.n_tracks = nTr.data();
    out.n_states = nSt.data();
    out.track_tip = tip.data();
    out.track_n_measurements = tnm.data();
    out.track_n_holes = tnh.data();
    out.track_n_outliers = tno.data();
    out.track_ndf = tndf.data();
    out.track_chi2 = tchi2.data();
    out.track_params = tpar.data();
    out.track_cov = tcov.data();
    out.state_prev = prev.data();
    out.state_surface = surf.data();
    out.state_flags = flags.data();
    out.state_measurement = meas.data();
    out.state_chi2 = schi2.data();
    out.state_path_length = path.data();
    out.predicted = pr.data();
    out.predicted_cov = prc.data();
    out.filtered = fi.data();
    out.filtered_cov = fic.data();
    out.jacobian = jac.data();
    ck_status st = ck_find_tracks(m_handle, &options.options, &options.ckf, &in, &out, nullptr);
    if (st != CK_OK) throw std::runtime_error(std::string("ck_find_tracks: ") + ck_last_error());

    auto unpack = [](const double* p, BoundMatrix& m) {
      for (size_t i = 0, c = 0; i < 6; ++i)
        for (size_t j = i; j < 6; ++j, ++c) m[i * 6 + j] = m[j * 6 + i] = p[c];
    };
    const double nan = std::numeric_limits<double>::quiet_NaN();
    std::vector<Result<std::vector<size_t>>> results;
    results.reserve(n);
    for (size_t s = 0; s < n; ++s) {
      if (status[s] != CK_TRACK_OK) {
        results.push_back(Result<std::vector<size_t>>::failure(status[s]));
        continue;
      }
      std::vector<size_t> found;
      for (int k = 0; k < nTr[s]; ++k) {
        const size_t ti = s * options.ckf.max_tracks + k;
        std::vector<int> chain;
        for (int i = tip[ti]; i >= 0; i = prev[s * options.ckf.max_states + i]) chain.push_back(i);
        Track tr;
        tr.firstState = container.states.size();
        tr.nStates = chain.size();
        tr.nMeasurements = static_cast<size_t>(tnm[ti]);
        tr.nHoles = static_cast<size_t>(tnh[ti]);
        tr.nOutliers = static_cast<size_t>(tno[ti]);
        tr.nDoF = static_cast<size_t>(tndf[ti]);
        tr.chi2 = tchi2[ti];
        if (tpar[6 * ti] == tpar[6 * ti]) {  // parameters on the target surface
          tr.referenceSurface = options.ckf.target_surface;
          for (size_t c = 0; c < 6; ++c) tr.parameters[c] = tpar[6 * ti + c];
          BoundMatrix m{};
          unpack(&tcov[21 * ti], m);
          for (size_t c = 0; c < 36; ++c) tr.covariance[c] = m[c];
        }
        for (auto it = chain.rbegin(); it != chain.rend(); ++it) {
          const size_t i = s * options.ckf.max_states + *it;
          TrackState ts;
          ts.surface = surf[i];
          ts.typeFlags = flags[i];
          ts.pathLength = path[i];
          ts.chi2 = schi2[i];
          ts.sourceLink = meas[i] >= 0 ? static_cast<int>(order[meas[i]]) : -1;
          for (size_t c = 0; c < 6; ++c) {
            ts.predicted[c] = pr[6 * i + c];
            ts.filtered[c] = fi[6 * i + c];
            ts.smoothed[c] = nan;
          }
          unpack(&prc[21 * i], ts.predictedCovariance);
          unpack(&fic[21 * i], ts.filteredCovariance);
          for (size_t c = 0; c < 36; ++c) ts.jacobian[c] = jac[36 * i + c];
          container.states.push_back(ts);
        }
        container.tracks.push_back(tr);
        found.push_back(container.tracks.size() - 1);
      }
      results.push_back(Result<std::vector<size_t>>::success(found));
    }
    return results;
  }

  ck_handle* handle() const { return m_handle; }

 private:
  Config m_cfg;
  ck_handle* m_handle = nullptr;
};

}  // namespace ActsPlugins
