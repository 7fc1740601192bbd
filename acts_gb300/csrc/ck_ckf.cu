// ck_ckf.cu — ck_find_tracks: combinatorial Kalman filter track finding
// from seeds, the GPU counterpart of
//   CombinatorialKalmanFilter<Propagator<EigenStepper<>, DirectNavigator>,
//       TrackContainer>::findTracks(initialParameters, options, tracks)
//   (Core/include/Acts/TrackFinding/CombinatorialKalmanFilter.hpp:1191-1335)
// with the default TrackStateCreator / MeasurementSelector and the examples'
// branch stopper (Examples/Algorithms/TrackFinding/src/
// TrackFindingAlgorithm.cpp:203-261).
//
// One thread per seed runs the whole depth-first search: the fitter's own
// stepper, navigator, covariance transport, material and Kalman update (the
// Lane of ck_fitter.cuh, its step in the kStepCkf mode) under the CKF actor
// below. The seed's track states go straight into the output arrays (the
// reset to a branch reads its outermost state back from there); the stack
// of active branches lives in device scratch. Every loop is bounded: the
// accepted steps of all branches of a seed by maxSteps (the propagator's
// step counter is shared, as in the reference), the Runge-Kutta trials of a
// step by maxRungeKuttaStepTrials, the candidates by the surface's
// measurements, the states, tracks and branches by their capacities.
#include <cuda_runtime.h>
#include <math_constants.h>

#include <climits>
#include <cmath>
#include <cstring>
#include <mutex>

#include "ck_api_internal.h"
#include "ck_fitter.cuh"

using namespace ck;

namespace {

constexpr int kCkfBlock = 64;
constexpr int kCkfMaxCandidates = 16;

// A branch (the reference's TrackProxy of an active branch): its tip state
// and summary counters
struct CkfBranch {
  int tip, nMeas, nHoles, nOutliers, ndf, pad;
  double chi2;
};

struct CkfParams {
  ck_ckf_options o;
  // the target's bounds (0: unbounded): rectangle half lengths of a plane,
  // the half length in z of a cylinder
  double targetHalfX, targetHalfY, targetHalfZ;
  const int32_t* surf_meas_off;  // [n_events * n_surfaces + 1]
  const int32_t* seed_event;     // [n_seeds] or NULL (event 0)
  int n_events;
  ck_ckf_out out;                // device pointers
  CkfBranch* branches;           // [n_seeds * max_branches]
  const int32_t* order;          // [n_seeds] the seeds in processing order
  // the candidates of each surface sorted along one local axis (windowed
  // search); see surfaceIndexKernel
  const double* sortedKey;  // [n_meas], per surface segment
  const int32_t* sortedIdx;
  const int32_t* surfAxis;  // [n_events * n_surfaces]: 0 / 1 sorted along loc0 /
                            // loc1, -1 not sorted (linear scan), -2 an invalid subspace
  const double* surfVmax;   // largest measurement variance on that axis
};

// A surface's candidates sorted by their measured value along one local axis
// a (lexicographic (value, index)), where every measurement of the surface
// measures a: the predicted chi2 of a candidate is at least
// r_a^2 / (V_aa + P_aa) (the Schur complement of the 2x2 residual
// covariance), so a search outward from the predicted value can stop once
// that bound passes the cut (and, while nothing passed, the smallest chi2
// found, for the outlier) — the selection is the full scan's.
constexpr int kCkfSortMax = 16384;
constexpr int kCkfSortThreads = 1024;

__global__ void __launch_bounds__(kCkfSortThreads)
surfaceIndexKernel(const int32_t* __restrict__ off, const double* __restrict__ val,
                   const double* __restrict__ cov, const int32_t* __restrict__ sub, int nSeg,
                   double* __restrict__ key, int32_t* __restrict__ idx, int32_t* __restrict__ axis,
                   double* __restrict__ vmax) {
  extern __shared__ __align__(16) unsigned char smem[];
  double* sk = reinterpret_cast<double*>(smem);
  int32_t* si = reinterpret_cast<int32_t*>(smem + sizeof(double) * kCkfSortMax);
  __shared__ int has0, has1, bad;
  __shared__ double vm0, vm1;
  const int s = blockIdx.x;  // segment: event * n_surfaces + surface
  if (s >= nSeg) return;
  const int m0 = off[s], m1 = off[s + 1], L = m1 - m0;
  const int tid = threadIdx.x;
  if (tid == 0) {
    has0 = has1 = bad = 0;
    vm0 = vm1 = 0.0;
  }
  __syncthreads();
  // which axes the surface's measurements measure, and their largest variance
  int h0 = 0, h1 = 0, b = 0;
  double v0 = 0.0, v1 = 0.0;
  for (int i = tid; i < L; i += blockDim.x) {
    const int m = m0 + i;
    const int sb = sub ? sub[m] : CK_MEAS_LOC01;
    if (sb < CK_MEAS_LOC0 || sb > CK_MEAS_LOC01) {
      b = 1;
      continue;
    }
    const double a0 = val[2 * (size_t)m], a1 = val[2 * (size_t)m + 1];
    const double c0 = cov[4 * (size_t)m], c3 = cov[4 * (size_t)m + 3];
    if (sb == CK_MEAS_LOC0) {
      h0 = 1;
      b |= !(a0 == a0) || !(c0 == c0);
      v0 = fmax(v0, c0);
    } else if (sb == CK_MEAS_LOC1) {
      h1 = 1;
      b |= !(a0 == a0) || !(c0 == c0);
      v1 = fmax(v1, c0);
    } else {
      b |= !(a0 == a0) || !(a1 == a1) || !(c0 == c0) || !(c3 == c3);
      v0 = fmax(v0, c0);
      v1 = fmax(v1, c3);
    }
  }
  if (h0) atomicOr(&has0, 1);
  if (h1) atomicOr(&has1, 1);
  if (b) atomicOr(&bad, 1);
  // (non-negative doubles order as their bit patterns)
  atomicMax(reinterpret_cast<unsigned long long*>(&vm0), (unsigned long long)__double_as_longlong(v0));
  atomicMax(reinterpret_cast<unsigned long long*>(&vm1), (unsigned long long)__double_as_longlong(v1));
  __syncthreads();
  int a;
  bool invalidSub = false;
  if (bad) {
    // an invalid subspace fails the scan of this surface; a NaN value or
    // variance leaves the surface unsorted
    for (int i = 0; i < L && !invalidSub; ++i) {
      const int sb = sub ? sub[m0 + i] : CK_MEAS_LOC01;
      invalidSub = sb < CK_MEAS_LOC0 || sb > CK_MEAS_LOC01;
    }
    a = invalidSub ? -2 : -1;
  } else {
    a = (has0 && has1) ? -1 : (has1 ? 1 : 0);
  }
  if (L > kCkfSortMax && a >= 0) a = -1;
  if (tid == 0) {
    axis[s] = a;
    vmax[s] = a == 1 ? vm1 : vm0;
  }
  if (a < 0 || L == 0) return;
  int P = 1;
  while (P < L) P <<= 1;
  for (int i = tid; i < P; i += blockDim.x) {
    if (i < L) {
      const int m = m0 + i;
      const int sb = sub ? sub[m] : CK_MEAS_LOC01;
      // (a 1D measurement holds its value in the first slot)
      sk[i] = (a == 1 && sb == CK_MEAS_LOC01) ? val[2 * (size_t)m + 1] : val[2 * (size_t)m];
      si[i] = m;
    } else {
      sk[i] = CUDART_INF;
      si[i] = INT_MAX;
    }
  }
  __syncthreads();
  // bitonic sort, lexicographic (value, index)
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = tid; i < P; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const double ka = sk[i], kb = sk[ixj];
          const int ia = si[i], ib = si[ixj];
          const bool aGreater = ka > kb || (ka == kb && ia > ib);
          if (((i & k) == 0) == aGreater) {
            sk[i] = kb;
            sk[ixj] = ka;
            si[i] = ib;
            si[ixj] = ia;
          }
        }
      }
      __syncthreads();
    }
  for (int i = tid; i < L; i += blockDim.x) {
    key[m0 + i] = sk[i];
    idx[m0 + i] = si[i];
  }
}

// Group operations of the G lanes that share a seed (G divides 32; the
// group's lanes are consecutive and run the same control flow on the same
// data, so they meet at every shuffle)
template <int G>
CK_D unsigned groupMask() {
  if constexpr (G == 32) {
    return 0xffffffffu;
  } else {
    const int base = (threadIdx.x & 31) & ~(G - 1);
    return ((1u << G) - 1u) << base;
  }
}
// lexicographic minimum of (chi2, measurement index) over the group
template <int G>
CK_D void groupArgMin(unsigned mask, double& c, int& m) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const double oc = __shfl_xor_sync(mask, c, o, G);
    const int om = __shfl_xor_sync(mask, m, o, G);
    if (oc < c || (oc == c && om < m)) {
      c = oc;
      m = om;
    }
  }
}
template <int G>
CK_D int groupSum(unsigned mask, int v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o, G);
  return v;
}

// G lanes per seed: every lane of the group runs the seed's search on the
// same values (identical stores to the same addresses); the candidate scan
// of a surface is split over the group and merged by shuffles into the
// serial scan's selection (ties in input order). With G = 1 a surface whose
// candidates are sorted along one axis is searched outward from the
// prediction instead (the same selection).
template <typename P, typename CV, int G>
struct CkfLane : Lane<P, CV> {
  using B = Lane<P, CV>;
  using B::absQ;
  using B::cAcc;
  using B::cActor;
  using B::cNav;
  using B::coasting;
  using B::cov;
  using B::cUser;
  using B::currentSurface;
  using B::deriv;
  using B::dirSign;
  using B::extrapolating;
  using B::finished;
  using B::haveTarget;
  using B::mass;
  using B::navigationBreak;
  using B::nSeq;
  using B::pathAcc;
  using B::pdg;
  using B::phase;
  using B::seq0;
  using B::stepStarted;
  using B::steps;
  using B::surfaceIndex;
  using B::targetIdx;
  using B::targetSurf;

  int nStatesC, nTracksC, nActive;
  int evBase;    // first segment of the seed's event (event * n_surfaces)
  int ckfStart;  // the surface the current branch restarted from (-1: the seed's plane)
  double pathLimit;
  bool pathLimitSet, done;

  CK_D CkfBranch* stack(const CkfParams& cp) const {
    return cp.branches + (size_t)this->t * cp.o.max_branches;
  }
  CK_D size_t stateIdx(const CkfParams& cp, int k) const {
    return (size_t)this->t * cp.o.max_states + k;
  }

  // ------------------------------------------------------------ outputs
  CK_D void writeState(const CkfParams& cp, int k, int sid, int prev, int meas, uint32_t flags,
                       double chi2, const double pred[6], const CV Cp[21], const CV J[36]) const {
    const ck_ckf_out& o = cp.out;
    const size_t i = stateIdx(cp, k);
    o.state_prev[i] = prev;
    o.state_surface[i] = sid;
    o.state_flags[i] = flags;
    if (o.state_measurement) o.state_measurement[i] = meas;
    if (o.state_chi2) o.state_chi2[i] = chi2;
    if (o.state_path_length) o.state_path_length[i] = pathAcc;
    if (o.predicted)
      for (int c = 0; c < 6; ++c) o.predicted[i * 6 + c] = pred[c];
    if (o.predicted_cov)
      for (int c = 0; c < 21; ++c) o.predicted_cov[i * 21 + c] = (double)Cp[c];
    if (o.jacobian)
      for (int c = 0; c < 36; ++c) o.jacobian[i * 36 + c] = (double)J[c];
  }
  CK_D void writeFiltered(const CkfParams& cp, int k, const double f[6], const CV F[21]) const {
    const size_t i = stateIdx(cp, k);
    for (int c = 0; c < 6; ++c) cp.out.filtered[i * 6 + c] = f[c];
    for (int c = 0; c < 21; ++c) cp.out.filtered_cov[i * 21 + c] = (double)F[c];
  }

  // storeLastActiveBranch: the branch on top becomes a found track, with its
  // bound parameters on the target surface when it reached it
  CK_D int store(const CkfParams& cp, const double* params, const CV* pc) {
    if (nTracksC >= cp.o.max_tracks) return CK_TRACK_TOO_MANY_STATES;
    const CkfBranch b = stack(cp)[nActive - 1];
    const ck_ckf_out& o = cp.out;
    const size_t i = (size_t)this->t * cp.o.max_tracks + nTracksC++;
    o.track_tip[i] = b.tip;
    if (o.track_n_measurements) o.track_n_measurements[i] = b.nMeas;
    if (o.track_n_holes) o.track_n_holes[i] = b.nHoles;
    if (o.track_n_outliers) o.track_n_outliers[i] = b.nOutliers;
    if (o.track_ndf) o.track_ndf[i] = b.ndf;
    if (o.track_chi2) o.track_chi2[i] = b.chi2;
    if (o.track_params)
      for (int c = 0; c < 6; ++c) o.track_params[i * 6 + c] = params ? params[c] : CUDART_NAN;
    if (o.track_cov)
      for (int c = 0; c < 21; ++c) o.track_cov[i * 21 + c] = pc ? (double)pc[c] : CUDART_NAN;
    return CK_TRACK_OK;
  }

  // the examples' branch stopper: 0 continue, 1 stop and keep, 2 stop and drop
  CK_D static int stopper(const CkfParams& cp, const CkfBranch& b) {
    const bool tooMany = b.nHoles > cp.o.max_holes || b.nOutliers > cp.o.max_outliers ||
                         (long long)b.nHoles + b.nOutliers > cp.o.max_holes_and_outliers;
    if (!tooMany) return 0;
    return b.nMeas >= cp.o.min_measurements ? 1 : 2;
  }

  // the actor's targetReached (a SurfaceReached with an unlimited near
  // limit, StandardAborters.hpp:94-155): reached when the navigator's
  // current surface is the target; else the closest intersection within
  // the target's bounds (BoundaryTolerance::None) decides, and the first
  // one steers the actor step constraint
  CK_D bool targetCheck(const FitParams& fp, const CkfParams& cp) {
    const int tsid = cp.o.target_surface;
    if (tsid < 0) return false;
    if (currentSurface == tsid) return true;
    double path[2];
    int st[2];
    const int ni = this->intersectSurf(fp, tsid, path, st);
    Surf<double> ts;
    ts.load(fp.surfaces + tsid);
    for (int i = 0; i < ni; ++i) {
      if (st[i] == 0) continue;
      double p[3], l[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) p[k] = this->pos[k] + path[i] * this->dir[k];
      ts.toLocal3(p, l);
      bool inside = true;
      if (ts.type == CK_SURFACE_CYLINDER && cp.targetHalfZ > 0)
        inside = fabs(l[2]) < fabs(cp.targetHalfZ + fp.opt.surfaceTolerance);
      else if (ts.type == CK_SURFACE_PLANE && cp.targetHalfX > 0 && cp.targetHalfY > 0)
        inside = l[0] >= -cp.targetHalfX && l[0] <= cp.targetHalfX && l[1] >= -cp.targetHalfY &&
                 l[1] <= cp.targetHalfY;
      if (!inside) st[i] = 0;
    }
    int best = -1;
    for (int i = 0; i < ni; ++i)
      if (st[i] != 0 && (best < 0 || fabs(path[i]) < fabs(path[best]))) best = i;
    for (int i = 0; i < ni; ++i)
      if (st[i] != 0 && path[i] < kNotSet + kOnSurfaceTolerance) {
        cActor = kNotSet;
        cupdate(cActor, path[i]);
        break;
      }
    return best >= 0 && st[best] == 2;
  }

  // EigenStepper::initialize from bound parameters on a surface
  CK_D void initialize(const FitParams& fp, const Surf<double>& sf, const double b[6]) {
    this->boundToFree(sf, b);
    this->initT(sf);
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    pathAcc = 0.0;
    cNav = kNotSet;
    cActor = kNotSet;
    cUser = fp.opt.maxStepSize;
    cAcc = fp.opt.initialStepSize;
  }

  // Actor::reset (CombinatorialKalmanFilter.hpp:470-531): the propagation
  // restarts from the outermost state of the branch on top of the stack
  CK_D int reset(const FitParams& fp, const CkfParams& cp) {
    if (nActive == 0) {
      done = true;
      return CK_TRACK_OK;
    }
    const int tip = stack(cp)[nActive - 1].tip;
    // (a branch below the top always holds a state of its own)
    if (tip < 0 || tip >= nStatesC) return CK_TRACK_INCONSISTENT_STATES;
    const size_t i = stateIdx(cp, tip);
    const int sid = cp.out.state_surface[i];
    double f[6];
    for (int c = 0; c < 6; ++c) f[c] = cp.out.filtered[i * 6 + c];
    Surf<double> sf;
    sf.load(fp.surfaces + sid);
    initialize(fp, sf, f);
    for (int c = 0; c < 21; ++c) cov[c] = toP<CV>(cp.out.filtered_cov[i * 21 + c]);
    // DirectNavigator::initialize: the current surface is the start surface,
    // the sequence index the one before it
    currentSurface = sid;
    surfaceIndex = -1;
    for (int k = 0; k < nSeq; ++k)
      if (__ldg(&fp.seq_surf[seq0 + k]) == sid) {
        surfaceIndex = k - 1;
        break;
      }
    navigationBreak = false;
    ckfStart = sid;
    // the post-update material of the start surface
    Surf<P> spv;
    if constexpr (sizeof(P) == sizeof(float)) spv.load(fp.surfaces + sid);
    const Surf<P>& sp = pickSurf<P>(sf, spv);
    double l[3];
    this->local(sf, l);
    if (!this->material(fp, sid, sf, sp, l, 2)) return CK_TRACK_NOT_ON_SURFACE;
    pathLimit = this->loopLimit(fp, kNotSet, true);
    targetCheck(fp, cp);
    return CK_TRACK_OK;
  }

  // Actor::filter (CombinatorialKalmanFilter.hpp:556-782) on surface sid
  CK_D int filter(const FitParams& fp, const CkfParams& cp, int sid) {
    const int sflags = __ldg(&fp.surfaces[sid].flags);
    const bool sensitive = (sflags & CK_SURF_SENSITIVE) != 0;
    const bool hasMat = (sflags & CK_SURF_MATERIAL) != 0;
    if (!sensitive && !hasMat) return CK_TRACK_OK;  // passive
    if (!sensitive) return CK_TRACK_INVALID_INPUT;  // material-only: not supported
    Surf<double> sf;
    sf.load(fp.surfaces + sid);
    Surf<P> spv;
    if constexpr (sizeof(P) == sizeof(float)) spv.load(fp.surfaces + sid);
    const Surf<P>& sp = pickSurf<P>(sf, spv);
    double l[3];
    this->local(sf, l);
    CV J[36];
    this->transportToBound(sf, sp, l, J, false);
    // pre-update material (none on the surface the branch restarted from)
    if (sid != ckfStart && !this->material(fp, sid, sf, sp, l, 1))
      return CK_TRACK_NOT_ON_SURFACE;
    double bp[6];
    if (!this->freeToBound(fp, sf, l, bp)) return CK_TRACK_NOT_ON_SURFACE;
    // the mixed form's predicted chi2 and update run in FP32 on its float
    // covariance (as in its fit)
    constexpr bool kF32 = sizeof(CV) == sizeof(float);
    double Pp[21];
    if constexpr (!kF32) {
#pragma unroll
      for (int i = 0; i < 21; ++i) Pp[i] = toD(cov[i]);
    }
    constexpr bool kFastRcp = sizeof(P) == sizeof(float);
    CkfBranch* stk = stack(cp);
    const int prevTip = stk[nActive - 1].tip;

    // TrackStateCreator + MeasurementSelector (MeasurementSelector.ipp:19-124):
    // the predicted chi2 of every measurement on the surface; those below
    // the cut, ascending (ties in input order), at most max_candidates; none
    // below: the smallest becomes an outlier when below the outlier cut
    const int seg = evBase + sid;
    const int m0 = __ldg(&cp.surf_meas_off[seg]), m1 = __ldg(&cp.surf_meas_off[seg + 1]);
    int selM[kCkfMaxCandidates];
    double selC[kCkfMaxCandidates];
    int nSel = 0, nPassed = 0, minM = -1;
    double minChi2 = kNotSet;
    const int K = cp.o.max_candidates;
    const int gl = (int)(threadIdx.x & (G - 1));  // this lane's share: m0 + gl, m0 + gl + G, ...
    bool badSub = false;
    // one candidate: its predicted chi2 into the first minimum and the
    // sorted selection, both lexicographic in (chi2, index)
    auto consider = [&](int m, int sub) -> double {
      double V[4];
#pragma unroll
      for (int c = 0; c < 4; ++c) V[c] = __ldg(&fp.meas_cov[4 * (size_t)m + c]);
      double c2;
      if constexpr (kF32)
        c2 = predictedChi2SubF(bp, cov, sub, __ldg(&fp.meas_val[2 * (size_t)m]),
                               __ldg(&fp.meas_val[2 * (size_t)m + 1]), V);
      else
        c2 = predictedChi2Sub<kFastRcp>(bp, Pp, sub, __ldg(&fp.meas_val[2 * (size_t)m]),
                                        __ldg(&fp.meas_val[2 * (size_t)m + 1]), V);
      if (c2 < minChi2 || (c2 == minChi2 && m < minM)) {
        minChi2 = c2;
        minM = m;
      }
      if (!(c2 >= cp.o.chi2_cut)) {
        ++nPassed;
        int pos = nSel;
        while (pos > 0 && (selC[pos - 1] > c2 || (selC[pos - 1] == c2 && selM[pos - 1] > m))) --pos;
        if (pos < K) {
          for (int j = (nSel < K ? nSel : K - 1); j > pos; --j) {
            selM[j] = selM[j - 1];
            selC[j] = selC[j - 1];
          }
          selM[pos] = m;
          selC[pos] = c2;
          if (nSel < K) ++nSel;
        }
      }
      return c2;
    };
    const int axis = m1 > m0 ? __ldg(&cp.surfAxis[seg]) : -1;
    if (axis == -2) {
      badSub = true;
    } else if (G == 1 && axis >= 0) {
      // windowed: outward from the predicted value along the sorted axis,
      // the nearer side first; a side ends where the chi2 bound can no
      // longer pass the cut nor (while nothing passed) undercut the
      // smallest chi2 below the outlier cut. The bound carries a relative
      // margin of 1e-5 for the rounding of the computed chi2.
      const double pk = bp[axis];
      const double den = __ldg(&cp.surfVmax[seg]) + toD(cov[sidx(axis, axis)]);
      const double* key = cp.sortedKey;
      int lo = m0, hi = m1;  // first key >= pk
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&key[mid]) < pk)
          lo = mid + 1;
        else
          hi = mid;
      }
      int L = lo - 1, R = lo;
      while (true) {
        const double dl = L >= m0 ? pk - __ldg(&key[L]) : CUDART_INF;
        const double dr = R < m1 ? __ldg(&key[R]) - pk : CUDART_INF;
        const bool left = dl < dr;
        const double d = left ? dl : dr;
        if (!(d < CUDART_INF)) break;
        const double lb = d * d / den * (1.0 - 1e-5);
        const bool more = lb < cp.o.chi2_cut ||
                          (nPassed == 0 && lb <= minChi2 && lb < cp.o.chi2_cut_outlier);
        if (!more) break;
        const int pos = left ? L-- : R++;
        const int m = __ldg(&cp.sortedIdx[pos]);
        consider(m, fp.meas_sub ? __ldg(&fp.meas_sub[m]) : CK_MEAS_LOC01);
      }
    } else {
      for (int m = m0 + gl; m < m1; m += G) {
        const int sub = fp.meas_sub ? __ldg(&fp.meas_sub[m]) : CK_MEAS_LOC01;
        if (sub < CK_MEAS_LOC0 || sub > CK_MEAS_LOC01) {
          badSub = true;
          break;
        }
        consider(m, sub);
      }
    }
    if constexpr (G > 1) {
      // merge the group's partial scans: counts, the first minimum, and the
      // K smallest (chi2, index) pairs, popped one by one from the lanes'
      // sorted lists
      const unsigned mask = groupMask<G>();
      if (groupSum<G>(mask, badSub ? 1 : 0)) return CK_TRACK_INVALID_INPUT;
      nPassed = groupSum<G>(mask, nPassed);
      double mc = minM >= 0 ? minChi2 : CUDART_INF;
      int mm = minM >= 0 ? minM : INT_MAX;
      groupArgMin<G>(mask, mc, mm);
      minM = mm == INT_MAX ? -1 : mm;
      minChi2 = mm == INT_MAX ? kNotSet : mc;
      int outM[kCkfMaxCandidates];
      double outC[kCkfMaxCandidates];
      int h = 0, n = 0;
      for (; n < K; ++n) {
        double c = h < nSel ? selC[h] : CUDART_INF;
        int m = h < nSel ? selM[h] : INT_MAX;
        groupArgMin<G>(mask, c, m);
        if (m == INT_MAX) break;
        outC[n] = c;
        outM[n] = m;
        if (h < nSel && selM[h] == m) ++h;
      }
      nSel = n;
      for (int i = 0; i < n; ++i) {
        selC[i] = outC[i];
        selM[i] = outM[i];
      }
    } else {
      if (badSub) return CK_TRACK_INVALID_INPUT;
    }
    bool isOutlier = false;
    if (nPassed == 0 && minM >= 0 && minChi2 < cp.o.chi2_cut_outlier) {
      selM[0] = minM;
      selC[0] = minChi2;
      nSel = 1;
      isOutlier = true;
    }
    const uint32_t matFlag = hasMat ? CK_FLAG_HAS_MATERIAL : 0u;
    if (nSel > 0) {
      const int first = nStatesC;
      if (first + nSel > cp.o.max_states) return CK_TRACK_TOO_MANY_STATES;
      for (int i = 0; i < nSel; ++i)
        writeState(cp, first + i, sid, prevTip, selM[i],
                   CK_FLAG_HAS_PARAMETERS | CK_FLAG_HAS_MEASUREMENT | matFlag |
                       (isOutlier ? CK_FLAG_IS_OUTLIER : 0u),
                   selC[i], bp, cov, J);
      nStatesC += nSel;
      // processNewTrackStates (:836-898): the new branches from the worst
      // candidate to the best, the best on top of the stack
      const CkfBranch root = stk[nActive - 1];
      --nActive;
      int onSurface = 0;
      for (int i = nSel - 1; i >= 0; --i) {
        CkfBranch b = root;
        b.tip = first + i;
        if (isOutlier) {
          writeFiltered(cp, b.tip, bp, cov);
          ++b.nOutliers;
        } else {
          const int m = selM[i];
          const int sub = fp.meas_sub ? __ldg(&fp.meas_sub[m]) : CK_MEAS_LOC01;
          double V[4];
#pragma unroll
          for (int c = 0; c < 4; ++c) V[c] = __ldg(&fp.meas_cov[4 * (size_t)m + c]);
          double filt[6], c2 = 0.0;
          CV Fc[21];
          const double mv0 = __ldg(&fp.meas_val[2 * (size_t)m]);
          const double mv1 = __ldg(&fp.meas_val[2 * (size_t)m + 1]);
          if constexpr (kF32) {
            if (!kalmanUpdateSubF(bp, cov, sub, mv0, mv1, V, fp.opt.joseph != 0, filt, Fc, c2))
              return CK_TRACK_UPDATE_FAILED;
          } else {
            double F[21];
            if (!kalmanUpdateSub<kFastRcp>(bp, Pp, sub, mv0, mv1, V, fp.opt.joseph != 0, filt, F,
                                           c2))
              return CK_TRACK_UPDATE_FAILED;
#pragma unroll
            for (int c = 0; c < 21; ++c) Fc[c] = toP<CV>(F[c]);
          }
          writeFiltered(cp, b.tip, filt, Fc);
          if (cp.out.state_chi2) cp.out.state_chi2[stateIdx(cp, b.tip)] = c2;
          ++b.nMeas;
          b.ndf += (sub & 1) + ((sub >> 1) & 1);
          b.chi2 = b.chi2 + c2;
        }
        if (nActive >= cp.o.max_branches) return CK_TRACK_TOO_MANY_STATES;
        stk[nActive++] = b;
        const int r = stopper(cp, b);
        if (r == 0) {
          ++onSurface;
        } else {
          if (r == 1) {
            const int e = store(cp, nullptr, nullptr);
            if (e != CK_TRACK_OK) return e;
          }
          --nActive;
        }
      }
      if (onSurface == 0) return reset(fp, cp);
    } else {
      // a hole: a sensitive surface without a selected measurement
      if (nStatesC >= cp.o.max_states) return CK_TRACK_TOO_MANY_STATES;
      const int k = nStatesC++;
      writeState(cp, k, sid, prevTip, -1, CK_FLAG_HAS_PARAMETERS | CK_FLAG_IS_HOLE | matFlag, 0.0,
                 bp, cov, J);
      writeFiltered(cp, k, bp, cov);
      CkfBranch& b = stk[nActive - 1];
      b.tip = k;
      ++b.nHoles;
      const int r = stopper(cp, b);
      if (r != 0) {
        if (r == 1) {
          const int e = store(cp, nullptr, nullptr);
          if (e != CK_TRACK_OK) return e;
        }
        --nActive;
        return reset(fp, cp);
      }
    }
    // the stepper continues with the filtered parameters of the branch on
    // top when its state is a measurement (EigenStepper::update)
    const size_t ci = stateIdx(cp, stk[nActive - 1].tip);
    const uint32_t cf = cp.out.state_flags[ci];
    if ((cf & CK_FLAG_HAS_MEASUREMENT) && !(cf & CK_FLAG_IS_OUTLIER)) {
      double f[6];
      for (int c = 0; c < 6; ++c) f[c] = cp.out.filtered[ci * 6 + c];
      this->updateFree(sf, bp, f, l);
      for (int c = 0; c < 21; ++c) cov[c] = toP<CV>(cp.out.filtered_cov[ci * 21 + c]);
      this->initTP(sp);
      this->local(sf, l);
    }
    if (!this->material(fp, sid, sf, sp, l, 2)) return CK_TRACK_NOT_ON_SURFACE;
    return CK_TRACK_OK;
  }

  // Actor::act (CombinatorialKalmanFilter.hpp:330-448)
  CK_D int act(const FitParams& fp, const CkfParams& cp) {
    if (!pathLimitSet) {
      pathLimit = this->loopLimit(fp, kNotSet, true);
      pathLimitSet = true;
    }
    if (currentSurface >= 0) {
      const int r = filter(fp, cp, currentSurface);
      if (r != CK_TRACK_OK) return r;
      if (done) return CK_TRACK_OK;
    }
    // (the reference evaluates both aborters before it acts on the first
    // that fired: both step-size constraints are updated)
    const bool pathReached = this->pathLimitReached(fp, pathLimit);
    const bool targetReached = targetCheck(fp, cp);
    if (!pathReached && !targetReached) return CK_TRACK_OK;
    int e;
    if (!pathReached) {
      // the branch's parameters: the bound state on the target surface
      const int tsid = cp.o.target_surface;
      Surf<double> sf;
      sf.load(fp.surfaces + tsid);
      Surf<P> spv;
      if constexpr (sizeof(P) == sizeof(float)) spv.load(fp.surfaces + tsid);
      const Surf<P>& sp = pickSurf<P>(sf, spv);
      double l[3], bp[6];
      this->local(sf, l);
      if (!this->freeToBound(fp, sf, l, bp)) return CK_TRACK_NOT_ON_SURFACE;
      CV J[36];
      this->transportToBound(sf, sp, l, J, false);
      cNav = kNotSet;
      e = store(cp, bp, cov);
    } else {
      e = store(cp, nullptr, nullptr);
    }
    if (e != CK_TRACK_OK) return e;
    --nActive;
    return reset(fp, cp);
  }

  // the seed: validation, EigenStepper::initialize on the seed's plane, the
  // pre-propagation actor call and the first target (Propagator.ipp:25-96)
  CK_D int begin(const FitParams& fp, const CkfParams& cp, int seed) {
    this->t = seed;
    this->q = seed;
    seq0 = __ldg(&fp.seq_off[seed]);
    nSeq = __ldg(&fp.seq_off[seed + 1]) - seq0;
    nStatesC = 0;
    nTracksC = 0;
    nActive = 0;
    if (nSeq < 0) return CK_TRACK_INVALID_INPUT;
    {
      const int ev = cp.seed_event ? __ldg(&cp.seed_event[seed]) : 0;
      if (ev < 0 || ev >= cp.n_events) return CK_TRACK_INVALID_INPUT;
      evBase = ev * fp.n_surfaces;
    }
    for (int i = 0; i < nSeq; ++i) {
      const int sid = __ldg(&fp.seq_surf[seq0 + i]);
      if (sid < 0 || sid >= fp.n_surfaces || __ldg(&fp.surfaces[sid].type) == CK_SURFACE_LINE)
        return CK_TRACK_INVALID_INPUT;
    }
    {
      double sp[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) sp[i] = __ldg(&fp.start_params[6 * (size_t)seed + i]);
      Surf<double> start;
      start.loadPlane(fp.start_frames + 12 * (size_t)seed);
      initialize(fp, start, sp);
      const double* sc = fp.start_cov + 36 * (size_t)seed;
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) cov[sidx(i, j)] = toP<CV>(__ldg(&sc[i * 6 + j]));
    }
    mass = __ldg(&fp.particle[2 * (size_t)seed]);
    absQ = __ldg(&fp.particle[2 * (size_t)seed + 1]);
    pdg = fp.pdg ? __ldg(&fp.pdg[seed]) : 211;
    dirSign = 1.0;
    extrapolating = false;
    coasting = false;
    finished = false;
    stepStarted = false;
    steps = 0;
    surfaceIndex = -1;
    navigationBreak = false;
    currentSurface = -1;  // the seed's plane is not a table surface
    haveTarget = false;
    targetSurf = -1;
    targetIdx = 0;
    ckfStart = -1;
    pathLimit = kNotSet;
    pathLimitSet = false;
    done = false;
    CkfBranch root;
    root.tip = -1;
    root.nMeas = root.nHoles = root.nOutliers = root.ndf = root.pad = 0;
    root.chi2 = 0.0;
    stack(cp)[0] = root;
    nActive = 1;
    int e = act(fp, cp);
    if (e != CK_TRACK_OK || done) return e;
    e = nextTarget(fp, cp, false);
    if (e != CK_TRACK_OK || done) return e;
    phase = PH_STEP;
    return CK_TRACK_OK;
  }

  // the navigator's next target (Propagator.ipp:79-96, 166-181); with
  // end_of_world a branch whose navigator has no surface of the sequence
  // left ends there, kept, as EndOfWorldReached ends it in Actor::act
  // (CombinatorialKalmanFilter.hpp:392-436), and the next branch restarts
  // (each pass pops a branch: bounded)
  CK_D int nextTarget(const FitParams& fp, const CkfParams& cp, bool release) {
    while (true) {
      if (!haveTarget) {
        if (release) cNav = kNotSet;
        int e;
        haveTarget = this->getNextTarget(fp, e);
        if (e != CK_TRACK_OK) return e;
      }
      if (!(cp.o.end_of_world && navigationBreak)) return CK_TRACK_OK;
      int e = store(cp, nullptr, nullptr);
      if (e != CK_TRACK_OK) return e;
      --nActive;
      e = reset(fp, cp);
      if (e != CK_TRACK_OK || done) return e;
      release = true;
    }
  }
};

template <typename P, typename CV, int G>
__global__ void __launch_bounds__(kCkfBlock) ckfKernel(FitParams fp, CkfParams cp) {
  static_assert(G >= 1 && G <= 32 && (32 % G) == 0, "lanes per seed");
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); i < fp.n_tracks;
       i += (int)(gridDim.x * blockDim.x / G)) {
    const int s = __ldg(&cp.order[i]);
    CkfLane<P, CV, G> L;
    int e = L.begin(fp, cp, s);
    bool ok = e == CK_TRACK_OK;
    if (ok && !L.done) {
      // Propagator::propagate's stepping loop (Propagator.ipp:98-186): each
      // pass takes one accepted step (or fails), so maxSteps bounds it
      while (true) {
        while (L.phase == PH_STEP) L.template step<kStepCkf>(fp, s);
        if (L.phase != PH_SURFACE) {  // the step failed: status written
          ok = false;
          e = -1;
          break;
        }
        e = L.act(fp, cp);
        if (e != CK_TRACK_OK) {
          ok = false;
          break;
        }
        if (L.done) break;
        e = L.nextTarget(fp, cp, true);
        if (e != CK_TRACK_OK) {
          ok = false;
          break;
        }
        if (L.done) break;
        L.phase = PH_STEP;
      }
    }
    if (e > 0) cp.out.status[s] = e;
    if (ok) cp.out.status[s] = CK_TRACK_OK;
    cp.out.n_tracks[s] = ok ? L.nTracksC : 0;
    cp.out.n_states[s] = ok ? L.nStatesC : 0;
  }
}

// The processing order of the seeds: grouped by |q/p| (64 bins of a
// quarter octave from 2^-10 to 2^6 per GeV), so that the seeds a warp runs
// together take similar steps and branch alike (measured on 50 barrel
// events of 2,000 seeds: the search 41 % faster than in input order). The
// order inside a bin is whatever the atomics give: a seed's results do not
// depend on which thread or when it runs.
constexpr int kOrderBins = 64;
constexpr int kOrderBlock = 256;

__device__ __forceinline__ int qopBin(const double* __restrict__ sp, int t) {
  const double q = fabs(sp[6 * (size_t)t + 4]);
  if (!(q > 0.0)) return 0;
  const int b = (int)floor((log2(q) + 10.0) * 4.0);
  return b < 0 ? 0 : (b >= kOrderBins ? kOrderBins - 1 : b);
}

__global__ void __launch_bounds__(kOrderBlock) orderCount(const double* __restrict__ sp, int n,
                                                          int32_t* __restrict__ counts) {
  __shared__ int32_t h[kOrderBins];
  for (int i = threadIdx.x; i < kOrderBins; i += blockDim.x) h[i] = 0;
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) atomicAdd(&h[qopBin(sp, t)], 1);
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderBins; i += blockDim.x)
    if (h[i]) atomicAdd(&counts[i], h[i]);
}

// exclusive scan of the bin counts into cursors (one warp)
__global__ void orderScan(int32_t* __restrict__ counts) {
  const int lane = threadIdx.x;
  int32_t a = counts[lane], b = counts[lane + 32];
  int32_t sa = a, sb = b;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int32_t va = __shfl_up_sync(0xffffffffu, sa, d);
    const int32_t vb = __shfl_up_sync(0xffffffffu, sb, d);
    if (lane >= d) {
      sa += va;
      sb += vb;
    }
  }
  const int32_t totalA = __shfl_sync(0xffffffffu, sa, 31);
  counts[lane] = sa - a;
  counts[lane + 32] = totalA + sb - b;
}

__global__ void __launch_bounds__(kOrderBlock) orderScatter(const double* __restrict__ sp, int n,
                                                            int32_t* __restrict__ cursor,
                                                            int32_t* __restrict__ order) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) order[atomicAdd(&cursor[qopBin(sp, t)], 1)] = t;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" void ck_ckf_options_default(ck_ckf_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->chi2_cut = 15.0;
  o->chi2_cut_outlier = INFINITY;
  o->max_candidates = 1;
  o->min_measurements = 0;
  o->max_holes = INT32_MAX;
  o->max_outliers = INT32_MAX;
  o->max_holes_and_outliers = INT32_MAX;
  o->target_surface = -1;
  o->max_states = 64;
  o->max_tracks = 16;
  o->max_branches = 16;
}

extern "C" int32_t ck_last_ckf_lanes(ck_handle* h) { return h ? h->lastCkfLanes : 0; }

extern "C" ck_status ck_find_tracks(ck_handle* h, const ck_options* opt, const ck_ckf_options* ck,
                                    const ck_ckf_in* in, ck_ckf_out* out, void* stream) {
  if (!h || !ck || !in || !out) return fail(CK_ERR_INVALID_ARGUMENT, "NULL argument");
  ck_status vs = validateOptions(opt);
  if (vs != CK_OK) return vs;
  const int n = in->n_seeds;
  if (n < 0 || in->n_meas < 0) return fail(CK_ERR_INVALID_ARGUMENT, "negative count");
  if (in->memory != CK_MEM_HOST && in->memory != CK_MEM_DEVICE)
    return fail(CK_ERR_INVALID_ARGUMENT, "unknown memory kind");
  if (in->n_surfaces != h->nSurfaces)
    return fail(CK_ERR_INVALID_ARGUMENT, "n_surfaces differs from the handle's surface table");
  if (ck->max_candidates < 1 || ck->max_candidates > kCkfMaxCandidates)
    return fail(CK_ERR_INVALID_ARGUMENT, "max_candidates outside 1..16");
  {
    const int g = ck->lanes_per_seed;
    if (g != 0 && g != 1 && g != 2 && g != 4 && g != 8 && g != 16 && g != 32)
      return fail(CK_ERR_INVALID_ARGUMENT, "lanes_per_seed not 0, 1, 2, 4, 8, 16 or 32");
  }
  if (ck->max_states < 1 || ck->max_tracks < 1 || ck->max_branches < 1)
    return fail(CK_ERR_INVALID_ARGUMENT, "a capacity below 1");
  if (ck->target_surface < -1 || ck->target_surface >= h->nSurfaces)
    return fail(CK_ERR_INVALID_ARGUMENT, "target surface out of range");
  if (ck->target_surface >= 0 && h->hostSurfaces[ck->target_surface].type == CK_SURFACE_LINE)
    return fail(CK_ERR_INVALID_ARGUMENT, "the target surface must be a plane or a cylinder");
  if (n == 0) return CK_OK;
  if (!in->seq_offsets || !in->seq_surfaces || !in->start_params || !in->start_cov ||
      !in->start_frames || !in->particle || !in->surf_meas_offsets ||
      (in->n_meas > 0 && (!in->meas_values || !in->meas_cov)))
    return fail(CK_ERR_INVALID_ARGUMENT, "a required input array is NULL");
  if (!out->status || !out->n_tracks || !out->n_states || !out->track_tip || !out->state_prev ||
      !out->state_surface || !out->state_flags || !out->filtered || !out->filtered_cov)
    return fail(CK_ERR_INVALID_ARGUMENT, "a required output array is NULL");
  if (in->n_events < 0) return fail(CK_ERR_INVALID_ARGUMENT, "n_events < 0");
  const int nEv = std::max(in->n_events, 1);
  if ((long long)nEv * h->nSurfaces >= INT_MAX)
    return fail(CK_ERR_INVALID_ARGUMENT, "n_events x n_surfaces too large");
  const int nSeg = nEv * h->nSurfaces;
  const bool host = in->memory == CK_MEM_HOST;
  if (host) {
    // the grouping of the measurements by event and surface, and the seeds'
    // events, checked where they are readable
    const int32_t* so = in->surf_meas_offsets;
    bool bad = so[0] != 0 || so[nSeg] != in->n_meas;
    for (int s = 0; s < nSeg && !bad; ++s) bad = so[s + 1] < so[s];
    for (int s = 0; s < n && !bad; ++s) bad = in->seq_offsets[s + 1] < in->seq_offsets[s];
    if (bad) return fail(CK_ERR_INVALID_ARGUMENT, "offsets not a non-decreasing partition");
    if (in->seed_event)
      for (int s = 0; s < n; ++s)
        if (in->seed_event[s] < 0 || in->seed_event[s] >= nEv)
          return fail(CK_ERR_INVALID_ARGUMENT, "seed_event outside [0, n_events)");
  }
  std::lock_guard<std::mutex> lock(h->mu);
  cudaError_t e = cudaSetDevice(h->device);
  if (e != cudaSuccess) return cudaFail(e, "set device");
  cudaStream_t st = stream ? (cudaStream_t)stream : h->stream;

  const size_t nn = (size_t)n, S = (size_t)ck->max_states * nn, T = (size_t)ck->max_tracks * nn;
  const size_t nSeqAll = host ? (size_t)in->seq_offsets[n] : 0;
  const size_t nm = (size_t)in->n_meas, ns1 = (size_t)nSeg + 1;
  struct Arr {
    const void* src;
    void* dst;
    size_t bytes;
    bool input;
  };
  Arr arrs[] = {
      {in->seq_offsets, nullptr, 4 * (nn + 1), true},
      {in->seq_surfaces, nullptr, 4 * nSeqAll, true},
      {in->start_params, nullptr, 48 * nn, true},
      {in->start_cov, nullptr, 288 * nn, true},
      {in->start_frames, nullptr, 96 * nn, true},
      {in->particle, nullptr, 8 * nn, true},
      {in->particle_pdg, nullptr, 4 * nn, true},
      {in->surf_meas_offsets, nullptr, 4 * ns1, true},
      {in->meas_values, nullptr, 16 * nm, true},
      {in->meas_cov, nullptr, 32 * nm, true},
      {in->meas_subspace, nullptr, 4 * nm, true},
      {in->seed_event, nullptr, 4 * nn, true},
      {out->status, nullptr, 4 * nn, false},
      {out->n_tracks, nullptr, 4 * nn, false},
      {out->n_states, nullptr, 4 * nn, false},
      {out->track_tip, nullptr, 4 * T, false},
      {out->track_n_measurements, nullptr, 4 * T, false},
      {out->track_n_holes, nullptr, 4 * T, false},
      {out->track_n_outliers, nullptr, 4 * T, false},
      {out->track_ndf, nullptr, 4 * T, false},
      {out->track_chi2, nullptr, 8 * T, false},
      {out->track_params, nullptr, 48 * T, false},
      {out->track_cov, nullptr, 168 * T, false},
      {out->state_prev, nullptr, 4 * S, false},
      {out->state_surface, nullptr, 4 * S, false},
      {out->state_flags, nullptr, 4 * S, false},
      {out->state_measurement, nullptr, 4 * S, false},
      {out->state_chi2, nullptr, 8 * S, false},
      {out->state_path_length, nullptr, 8 * S, false},
      {out->predicted, nullptr, 48 * S, false},
      {out->predicted_cov, nullptr, 168 * S, false},
      {out->filtered, nullptr, 48 * S, false},
      {out->filtered_cov, nullptr, 168 * S, false},
      {out->jacobian, nullptr, 288 * S, false}};
  constexpr int kArrs = sizeof(arrs) / sizeof(arrs[0]);
  // device scratch: the fail path's tip array, the branch stacks and the
  // surfaces' sorted candidates
  const size_t tipBytes = align256(4 * nn);
  const size_t brBytes = align256(sizeof(CkfBranch) * (size_t)ck->max_branches * nn);
  const size_t keyBytes = align256(8 * nm), idxBytes = align256(4 * nm);
  const size_t axBytes = align256(4 * ns1), vmBytes = align256(8 * ns1);
  const size_t ordBytes = align256(4 * nn), binBytes = align256(4 * kOrderBins);
  const size_t scratchBytes =
      tipBytes + brBytes + keyBytes + idxBytes + axBytes + vmBytes + ordBytes + binBytes;
  size_t total = scratchBytes;
  if (host)
    for (int i = 0; i < kArrs; ++i)
      if (arrs[i].src) total += align256(arrs[i].bytes);
  if ((e = h->unitBuf.ensure(total)) != cudaSuccess) return cudaFail(e, "track-finding buffer");
  char* base = (char*)h->unitBuf.p;
  size_t off = scratchBytes;
  for (int i = 0; i < kArrs; ++i) {
    if (!arrs[i].src) continue;
    if (host) {
      arrs[i].dst = base + off;
      off += align256(arrs[i].bytes);
      if (arrs[i].input && arrs[i].bytes)
        cudaMemcpyAsync(arrs[i].dst, arrs[i].src, arrs[i].bytes, cudaMemcpyHostToDevice, st);
    } else {
      arrs[i].dst = const_cast<void*>(arrs[i].src);
    }
  }
  FitParams fp;
  std::memset(&fp, 0, sizeof(fp));
  fp.n_tracks = n;
  fp.n_queue = n;
  fp.seq_off = (const int32_t*)arrs[0].dst;
  fp.seq_surf = (const int32_t*)arrs[1].dst;
  fp.start_params = (const double*)arrs[2].dst;
  fp.start_cov = (const double*)arrs[3].dst;
  fp.start_frames = (const double*)arrs[4].dst;
  fp.particle = (const float*)arrs[5].dst;
  fp.pdg = (const int32_t*)arrs[6].dst;
  fp.meas_val = (const double*)arrs[8].dst;
  fp.meas_cov = (const double*)arrs[9].dst;
  fp.meas_sub = (const int32_t*)arrs[10].dst;
  fp.out.status = (int32_t*)arrs[12].dst;
  fp.tip = (int32_t*)base;
  fp.max_states = 1;
  fp.lanes_per_warp = 32;
  fp.steps_per_round = 1;
  fp.surfaces = h->dSurfaces;
  fp.n_surfaces = h->nSurfaces;
  fp.trig = h->dTrig;
  fp.field = h->field;
  fp.mc = h->mc;
  fp.opt = toDevOptions(*opt);
  fp.ref_surface = -1;
  CkfParams cp;
  std::memset(&cp, 0, sizeof(cp));
  cp.o = *ck;
  if (ck->target_surface >= 0) {
    const ck_surface& t = h->hostSurfaces[ck->target_surface];
    cp.targetHalfX = t.half_x;
    cp.targetHalfY = t.half_y;
    cp.targetHalfZ = t.half_length_z;
  }
  cp.surf_meas_off = (const int32_t*)arrs[7].dst;
  cp.seed_event = (const int32_t*)arrs[11].dst;
  cp.n_events = nEv;
  cp.branches = (CkfBranch*)(base + tipBytes);
  {
    char* p = base + tipBytes + brBytes;
    double* key = (double*)p;
    int32_t* idx = (int32_t*)(p + keyBytes);
    int32_t* ax = (int32_t*)(p + keyBytes + idxBytes);
    double* vm = (double*)(p + keyBytes + idxBytes + axBytes);
    if (!h->ckfSortSmemSet) {  // (a per-device attribute: set on the handle's device)
      if ((e = cudaFuncSetAttribute(surfaceIndexKernel,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(12 * kCkfSortMax))) != cudaSuccess)
        return cudaFail(e, "surface index kernel attributes");
      h->ckfSortSmemSet = true;
    }
    if (nSeg > 0)
      surfaceIndexKernel<<<nSeg, kCkfSortThreads, 12 * kCkfSortMax, st>>>(
          cp.surf_meas_off, fp.meas_val, fp.meas_cov, fp.meas_sub, nSeg, key, idx, ax, vm);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "surface index kernel launch");
    // the seeds' processing order
    int32_t* order = (int32_t*)(p + keyBytes + idxBytes + axBytes + vmBytes);
    int32_t* bins = (int32_t*)(p + keyBytes + idxBytes + axBytes + vmBytes + ordBytes);
    const int og = (n + kOrderBlock - 1) / kOrderBlock;
    cudaMemsetAsync(bins, 0, 4 * kOrderBins, st);
    orderCount<<<og, kOrderBlock, 0, st>>>(fp.start_params, n, bins);
    orderScan<<<1, 32, 0, st>>>(bins);
    orderScatter<<<og, kOrderBlock, 0, st>>>(fp.start_params, n, bins, order);
    if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "seed order launch");
    cp.order = order;
    cp.sortedKey = key;
    cp.sortedIdx = idx;
    cp.surfAxis = ax;
    cp.surfVmax = vm;
  }
  int32_t** outInts[] = {&cp.out.status,        &cp.out.n_tracks,         &cp.out.n_states,
                         &cp.out.track_tip,     &cp.out.track_n_measurements,
                         &cp.out.track_n_holes, &cp.out.track_n_outliers, &cp.out.track_ndf};
  for (int i = 0; i < 8; ++i) *outInts[i] = (int32_t*)arrs[12 + i].dst;
  cp.out.track_chi2 = (double*)arrs[20].dst;
  cp.out.track_params = (double*)arrs[21].dst;
  cp.out.track_cov = (double*)arrs[22].dst;
  cp.out.state_prev = (int32_t*)arrs[23].dst;
  cp.out.state_surface = (int32_t*)arrs[24].dst;
  cp.out.state_flags = (uint32_t*)arrs[25].dst;
  cp.out.state_measurement = (int32_t*)arrs[26].dst;
  cp.out.state_chi2 = (double*)arrs[27].dst;
  cp.out.state_path_length = (double*)arrs[28].dst;
  cp.out.predicted = (double*)arrs[29].dst;
  cp.out.predicted_cov = (double*)arrs[30].dst;
  cp.out.filtered = (double*)arrs[31].dst;
  cp.out.filtered_cov = (double*)arrs[32].dst;
  cp.out.jacobian = (double*)arrs[33].dst;
  const bool mixed = opt->precision == CK_PRECISION_MIXED;
  // (0: one lane per seed; the windowed candidate search visits few
  // candidates, and a group replicates the propagation on every lane)
  const int G = ck->lanes_per_seed > 0 ? ck->lanes_per_seed : 1;
  const int grid = (int)(((long long)n * G + kCkfBlock - 1) / kCkfBlock);
#define CK_CKF_LAUNCH(GG)                                                   \
  case GG:                                                                 \
    if (mixed)                                                             \
      ckfKernel<float, float, GG><<<grid, kCkfBlock, 0, st>>>(fp, cp);     \
    else                                                                   \
      ckfKernel<double, double, GG><<<grid, kCkfBlock, 0, st>>>(fp, cp);   \
    break;
  switch (G) {
    CK_CKF_LAUNCH(1)
    CK_CKF_LAUNCH(2)
    CK_CKF_LAUNCH(4)
    CK_CKF_LAUNCH(8)
    CK_CKF_LAUNCH(16)
    CK_CKF_LAUNCH(32)
    default:
      return fail(CK_ERR_INVALID_ARGUMENT, "lanes_per_seed not 0, 1, 2, 4, 8, 16 or 32");
  }
#undef CK_CKF_LAUNCH
  h->lastCkfLanes = G;
  if ((e = cudaGetLastError()) != cudaSuccess) return cudaFail(e, "track-finding kernel launch");
  if (host) {
    for (int i = 0; i < kArrs; ++i)
      if (arrs[i].src && !arrs[i].input)
        cudaMemcpyAsync(const_cast<void*>(arrs[i].src), arrs[i].dst, arrs[i].bytes,
                        cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cudaFail(e, "track-finding kernel");
  }
  h->lastLaunches = 5;
  return CK_OK;
}
