// ck_fitter.cuh — the per-track Kalman fit as a lane state machine, and the
// persistent, phase-scheduled fit kernel.
//
// The fit of one track restates
//   KalmanFitter::fit_impl / filter_impl        KalmanFitter.hpp:795-984
//   KalmanFitter::Actor::act / filter           KalmanFitter.hpp:337-671
//   Propagator::propagate stepping loop         Propagator.ipp:25-210
//   DirectNavigator::nextTarget / handleSurfaceReached  DirectNavigator.hpp:222-348
//   detail::updateSingleSurfaceStatus           SteppingHelper.hpp:41-78
//   ConstrainedStep                             ConstrainedStep.hpp:44-173
//   PathLimitReached + loop protection          StandardAborters.hpp, LoopProtection.hpp
//   GainMatrixSmoother::operator()              GainMatrixSmoother.hpp:43-99
// for the declared extension set (pass-through calibrator, GainMatrixUpdater,
// GainMatrixSmoother, predicted-chi2 outlier finder).
//
// Termination follows the reference: when outliers leave the track
// "incomplete" (measurementStates < #measurements) propagation continues
// after the last surface until the loop-protection path limit, and errors on
// the way (leaving the field map, step limits) fail the fit. States created
// there lie beyond the track's tip, so this "coasting" phase transports no
// covariance and stores no records. ck_options.early_termination stops at the
// last surface that carries a source link instead.
//
// Execution model (GB300): one lane owns one track at a time and keeps its
// whole state in registers. The fit is cut into phases — FETCH (take a track
// from the queue and initialise), STEP (one Runge-Kutta trial; a rejected
// trial simply stays in STEP), SURFACE (the actor on a reached surface:
// covariance transport, Kalman update, material) and SMOOTH (one backward
// RTS state). Every iteration the warp votes and runs the phase that most of
// its lanes are waiting for, so the FP64-heavy phases execute with many
// active lanes instead of serialising the divergent paths of 32 different
// tracks. A lane that finishes a track fetches the next one immediately.
// Positions are kept in double in both precision forms; intersections and
// local coordinates are evaluated in double so that the 1e-4 mm on-surface
// tolerance is resolvable.
#pragma once

#include <type_traits>

#include "ck_device.cuh"

namespace ck {

// Helpers called from several places. Measured on GB300: keeping them out
// of line shrinks the kernel ~3x but forces the lane state into local memory
// and costs 5-10 %, so they stay inlined.
#define CK_NI CK_D

enum Phase { PH_FETCH = 0, PH_STEP = 1, PH_SURFACE = 2, PH_DONE = 3 };
// What follows an accepted Runge-Kutta step: the fit's navigation and actor
// (kStepFit), the aborters of the extrapolation to the reference line
// (kStepExtrapolate), those of a plain propagation (kStepPropagate), or the
// navigator's post-step update alone, the track finder's actor running in
// its own loop (kStepCkf: the lane returns in the SURFACE phase).
enum StepMode { kStepFit = 0, kStepExtrapolate = 1, kStepPropagate = 2, kStepCkf = 3 };
// SurfaceReached's near limit (StandardAborters.hpp:76): -100 um
constexpr double kTargetNearLimit = -0.1;
// Runge-Kutta trials per round of the compaction kernels when at most half
// of a block's slots step
constexpr int kTailStepsPerRound = 32;

// ChargeHypothesis::extractMomentum (ChargeHypothesis.hpp:70-90)
template <typename P>
CK_D P absMomentum(float absQ, P qop) {
  float q;
  if constexpr (sizeof(P) == sizeof(float))
    q = copysignf(absQ, qop);  // the same value without a double round trip
  else
    q = (float)copysign((double)absQ, (double)qop);
  return (P)q / qop;
}

CK_D void cupdate(double& slot, double v) {
  if (fabs(v) < fabs(slot)) slot = v;
}

// scratch record access (one record set per resident lane)
// the surface in the stepper precision: the FP64 surface itself in the
// plain form, its FP32 copy in the mixed form
template <typename P>
CK_D const Surf<P>& pickSurf(const Surf<double>& d, const Surf<P>& p) {
  if constexpr (sizeof(P) == sizeof(double))
    return d;
  else
    return p;
}

template <typename CV>
struct Rec {
  RecState<CV>* base;  // state 0 of this queue position
  CK_D Rec(const FitParams& fp, int q)
      : base(static_cast<RecState<CV>*>(fp.rec) + (size_t)q * (size_t)fp.max_states) {}
  // bound parameters (FP64)
  CK_D double& p(int k, int f) const { return base[k].par[f]; }
  // covariances and jacobian (CV)
  CK_D CV& m(int k, int f) const { return base[k].mat[f]; }
  CK_D RecState<CV>& s(int k) const { return base[k]; }
};

// KalmanFitter.hpp:897-900: every track with reverseFiltering, else the
// tracks whose last measurement state's filtered momentum 1/|q/p| is at most
// the threshold (SimpleReverseFilteringLogic, Examples/Algorithms/
// TrackFitting/src/KalmanFitterFunction.cpp:50-58)
template <typename CV>
CK_D bool reverseSelected(const FitParams& fp, int q, int tip) {
  if (fp.opt.reverseFiltering) return true;
  if (!(fp.opt.reverseMomThreshold > 0.0)) return false;
  const Rec<CV> rec(fp, q);
  for (int k = tip; k >= 0; --k) {
    const uint32_t fl = (uint32_t)rec.s(k).flags;
    if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER))
      return fabs(1.0 / rec.p(k, kRecFilt + 4)) <= fp.opt.reverseMomThreshold;
  }
  return false;
}

// F2B: the lane applies the free-to-bound correction in its covariance
// transport when the options ask for it (instantiated separately, so that
// the default kernels carry none of its code).
// REV: the lane runs the reversed filter pass of reverse filtering
// (KalmanFitter.hpp:897-945): backwards along the sequence from the forward
// pass's last measurement state, which it reads from that pass's records;
// it writes no records, only its latest filtered measurement state (the
// extrapolation start slot 0) and, when it reaches the reference surface,
// the track parameters there.
template <typename P, typename CV, bool F2B = false, bool REV = false>
struct Lane {
  // ---- identity: track index and queue position (which indexes the records)
  int phase;
  int t;
  int q;
  // ---- stepper: the free parameters are accumulated in FP64 in every form;
  // the Runge-Kutta stages, field and transport are evaluated in P
  double pos[3];
  double tim;
  double dir[3];
  double qop;
  CV cov[21];
  Transport<P> T;
  P deriv[7];  // dir (3), dt/ds, k4 (3)
  double pathAcc;
  double cNav, cActor, cUser, cAcc;
  float mass, absQ;
  int pdg;
  // ---- pending Runge-Kutta step
  double initialH;
  double hd;  // step size (FP64 in every form; the stages use it rounded to P)
  unsigned trials;
  bool stepStarted;
  unsigned steps;
  // ---- navigation
  int surfaceIndex, currentSurface, targetSurf, targetIdx;
  bool navigationBreak, haveTarget;
  // ---- propagation direction (+1; -1 for a backward extrapolation) and the
  // mode of the lane: the fit, or the extrapolation to the reference surface
  double dirSign;
  bool extrapolating;
  // ---- Kalman fitter actor; lastSlSeq is the last sequence position in the
  // direction of travel that carries a source link. The reversed pass keeps
  // no track (no tip) and holds its start surface in the tip's place (an
  // extra field costs the FP64 kernel spills).
  int nStates;
  union {
    int lastMeasurementIndex;  // forward: the tip
    int startSid;              // reversed: the start surface (a table id)
  };
  int measurementStates, nDistinct, lastSlSeq;
  int measHint;  // where the next measurement lookup starts (distinct surfaces only)
  bool finished, coasting;
  double propLimit, kfLimit;
  int seq0, nSeq, m0, nMeas;

  // ------------------------------------------------------------ helpers
  CK_D double stepValue() const {
    double mn = fmin(cNav, fmin(cActor, cUser));
    double r = fmin(fabs(mn), cAcc);
    return signbit(mn) ? -r : r;
  }

  CK_D void fail(const FitParams& fp, int code) {
    const ck_batch_out& out = fp.out;
    out.status[t] = code;
    if (out.n_states) out.n_states[t] = 0;
    if (out.n_measurements) out.n_measurements[t] = 0;
    if (out.n_holes) out.n_holes[t] = 0;
    if (out.n_outliers) out.n_outliers[t] = 0;
    if (out.ndf) out.ndf[t] = 0;
    if (out.chi2_sum) out.chi2_sum[t] = 0.0;
    fp.tip[q] = -1;
    phase = PH_FETCH;
  }

  // findMeas when every measurement has its own surface: the search starts
  // after the last match, where the next surface's measurement usually is
  // (source links in propagation order); with repeated surfaces the first
  // match in input order is the one the reference keeps, so the plain search
  // runs.
  CK_D int findMeasHinted(const FitParams& fp, int sid) {
    if (nDistinct != nMeas) return findMeas(fp, sid);
    int j = measHint;
    for (int i = 0; i < nMeas; ++i) {
      if (j >= nMeas) j = 0;
      if (__ldg(&fp.meas_surf[m0 + j]) == sid) {
        measHint = j + 1;
        return m0 + j;
      }
      ++j;
    }
    return -1;
  }

  CK_D int findMeas(const FitParams& fp, int sid) const {
    for (int i = 0; i < nMeas; ++i)
      if (__ldg(&fp.meas_surf[m0 + i]) == sid) return m0 + i;
    return -1;
  }

  // Surface::intersect in double (BoundaryTolerance::Infinite), along the
  // direction of travel (the navigator's direction times the momentum's);
  // `coarse` as intersectMixed's (mixed form)
  CK_NI int intersectSurf(const FitParams& fp, int sid, double path[2], int st[2],
                          double coarse = kNotSet) const {
    Surf<double> sf;
    sf.load(fp.surfaces + sid);
    double nd[3] = {dir[0], dir[1], dir[2]};
    if constexpr (REV) {
      nd[0] = -dir[0];
      nd[1] = -dir[1];
      nd[2] = -dir[2];
    }
    if constexpr (sizeof(P) == sizeof(float)) {
      return intersectMixed(sf, pos, nd, fp.opt.surfaceTolerance, path, st, coarse);
    } else {
      return intersect(sf, pos, nd, fp.opt.surfaceTolerance, path, st);
    }
  }

  // Surface::isOnSurface part of globalToLocal: the check alone, without
  // the local coordinates
  // sqrt in the form's arithmetic: FP64 sqrt (plain), refined FP32
  // reciprocal square root (mixed)
  CK_D static double sqrtF(double v) {
    if constexpr (sizeof(P) == sizeof(float))
      return v > 0.0 ? v * rsqrtRefined(v) : 0.0;
    else
      return sqrt(v);
  }
  CK_D double atan2F(const FitParams& fp, double y, double x) const {
    if constexpr (sizeof(P) == sizeof(float))
      return atan2Table(y, x, fp.trig);
    else
      return atan2(y, x);
  }

  // local coordinates R^T (pos - c) of the current position
  CK_D void local(const Surf<double>& sf, double l[3]) const { sf.toLocal3(pos, l); }

  // Surface::isOnSurface part of globalToLocal, from the local coordinates
  CK_D static bool onSurfaceLocal(const Surf<double>& sf, const double l[3]) {
    if (sf.type == CK_SURFACE_PLANE) return fabs(l[2]) <= kOnSurfaceTolerance;
    double inttol = sf.radius * 0.0001;
    if (inttol < 0.01) inttol = 0.01;
    return fabs(sqrtF(l[0] * l[0] + l[1] * l[1]) - sf.radius) <= inttol;
  }
  CK_D bool onSurface(const Surf<double>& sf) const {
    double l[3];
    local(sf, l);
    return onSurfaceLocal(sf, l);
  }

  // Surface::globalToLocal in double (the bound parameters are outputs)
  CK_NI bool toLocal(const FitParams& fp, const Surf<double>& sf, const double l[3],
                     double loc[2]) const {
    if (sf.type == CK_SURFACE_PLANE) {
      if (fabs(l[2]) > kOnSurfaceTolerance) return false;
      loc[0] = l[0];
      loc[1] = l[1];
      return true;
    }
    double inttol = sf.radius * 0.0001;
    if (inttol < 0.01) inttol = 0.01;
    const double r = sqrtF(l[0] * l[0] + l[1] * l[1]);
    if (fabs(r - sf.radius) > inttol) return false;
    loc[0] = sf.radius * atan2F(fp, l[1], l[0]);
    loc[1] = l[2];
    return true;
  }

  // transformFreeToBoundParameters (TransformationHelpers.cpp:41-63), with
  // the local coordinates of the current position
  CK_NI bool freeToBound(const FitParams& fp, const Surf<double>& sf, const double l[3],
                         double b[6]) const {
    double loc[2];
    if (!toLocal(fp, sf, l, loc)) return false;
    b[0] = loc[0];
    b[1] = loc[1];
    b[5] = tim;
    b[2] = atan2F(fp, dir[1], dir[0]);
    b[3] = atan2F(fp, sqrtF(dir[0] * dir[0] + dir[1] * dir[1]), dir[2]);
    b[4] = qop;
    return true;
  }

  // transformBoundToFreeParameters (TransformationHelpers.cpp:17-39)
  CK_NI void boundToFree(const Surf<double>& sf, const double b[6]) {
    double sp, cp, st, ct;
    sincos(b[2], &sp, &cp);
    sincos(b[3], &st, &ct);
    dir[0] = cp * st;
    dir[1] = sp * st;
    dir[2] = ct;
    double l[3];
    if (sf.type == CK_SURFACE_PLANE) {
      l[0] = b[0];
      l[1] = b[1];
      l[2] = 0.0;
    } else {
      double sphi, cphi;
      sincos(b[0] / sf.radius, &sphi, &cphi);
      l[0] = sf.radius * cphi;
      l[1] = sf.radius * sphi;
      l[2] = b[1];
    }
    sf.toGlobal3(l, pos);
    tim = b[5];
    qop = b[4];
  }

  // stepper.update with the filtered parameters (EigenStepper.ipp:128-138).
  // The plain form evaluates transformBoundToFreeParameters; the mixed form
  // rotates the predicted free state (still held) by the small filtered
  // changes of phi, theta and the cylinder angle, with FP64 sines and cosines
  // of those changes from their Taylor series — no FP64 trigonometry.
  CK_D void updateFree(const Surf<double>& sf, const double pred[6], const double filt[6],
                       const double lp[3]) {
    if constexpr (sizeof(P) == sizeof(double)) {
      boundToFree(sf, filt);
    } else {
      const double dphi = radian_sym(filt[2] - pred[2]);
      const double dtheta = filt[3] - pred[3];
      const double dalpha = sf.type == CK_SURFACE_PLANE ? 0.0 : (filt[0] - pred[0]) / sf.radius;
      const double lim = 0.05;
      if (!(fabs(dphi) < lim && fabs(dtheta) < lim && fabs(dalpha) < lim)) {
        boundToFree(sf, filt);
        return;
      }
      auto sc = [](double x, double& sn, double& cs) {
        const double x2 = x * x;
        sn = x * (1.0 + x2 * (-1.0 / 6 + x2 * (1.0 / 120 + x2 * (-1.0 / 5040 + x2 * (1.0 / 362880)))));
        cs = 1.0 + x2 * (-0.5 + x2 * (1.0 / 24 + x2 * (-1.0 / 720 + x2 * (1.0 / 40320))));
      };
      // 1/sqrt(v) for v near a known scale: FP32 estimate, one FP64 Newton step
      auto rsq = [](double v) {
        const double y = toD(rsqrtf(d2f(v)));
        return y * (1.5 - 0.5 * v * y * y);
      };
      // direction
      const double s2 = dir[0] * dir[0] + dir[1] * dir[1];
      const double ist = rsq(s2);
      const double cphi = dir[0] * ist, sphi = dir[1] * ist;
      const double stheta = s2 * ist, ctheta = dir[2];
      double sdp, cdp, sdt, cdt;
      sc(dphi, sdp, cdp);
      sc(dtheta, sdt, cdt);
      const double cp = cphi * cdp - sphi * sdp, sp = sphi * cdp + cphi * sdp;
      const double st = stheta * cdt + ctheta * sdt, ct = ctheta * cdt - stheta * sdt;
      dir[0] = cp * st;
      dir[1] = sp * st;
      dir[2] = ct;
      // position
      double l[3];
      if (sf.type == CK_SURFACE_PLANE) {
        l[0] = filt[0];
        l[1] = filt[1];
        l[2] = 0.0;
      } else {
        const double ir = rsq(lp[0] * lp[0] + lp[1] * lp[1]);
        const double ca = lp[0] * ir, sa = lp[1] * ir;
        double sda, cda;
        sc(dalpha, sda, cda);
        l[0] = sf.radius * (ca * cda - sa * sda);
        l[1] = sf.radius * (sa * cda + ca * sda);
        l[2] = filt[1];
      }
      sf.toGlobal3(l, pos);
      tim = filt[5];
      qop = filt[4];
    }
  }

  // Surface::boundToFreeJacobian in transport form at the current state
  CK_NI void initT(const Surf<double>& sfd) {
    Surf<P> sf;
#pragma unroll
    for (int i = 0; i < 9; ++i) sf.R[i] = (P)sfd.R[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) sf.c[i] = (P)sfd.c[i];
    sf.radius = (P)sfd.radius;
    sf.type = sfd.type;
    initTP(sf);
  }
  CK_D void initTP(const Surf<P>& sf) {
    const P p[3] = {toP<P>(pos[0]), toP<P>(pos[1]), toP<P>(pos[2])};
    const P f[8] = {p[0],           p[1],           p[2],           toP<P>(tim),
                    toP<P>(dir[0]), toP<P>(dir[1]), toP<P>(dir[2]), toP<P>(qop)};
    initTransport(sf, f, T);
  }

  CK_D double loopLimit(const FitParams& fp, double previous, bool release) const {
    double limit = previous;
    if (!fp.opt.loopProtection) return limit;
    if (release) limit = kNotSet;
    P B[3];
    const P p[3] = {(P)pos[0], (P)pos[1], (P)pos[2]};
    if (!getField(fp.field, p, B)) return limit;
    const double Bn = sqrt((double)B[0] * (double)B[0] + (double)B[1] * (double)B[1] +
                           (double)B[2] * (double)B[2]);
    if (Bn == 0.0) return limit;
    const double pm = absMomentum(absQ, qop);
    const double ll = fp.opt.loopFraction * (2.0 * kPi * pm / Bn);
    if (fabs(ll) < fabs(limit)) limit = ll;
    return limit;
  }

  CK_D bool pathLimitReached(const FitParams& fp, double limit) {
    const double distance = fabs(limit) - fabs(pathAcc);
    if (fabs(distance) < fabs(fp.opt.surfaceTolerance)) return true;
    cupdate(cActor, distance);
    return false;
  }

  // 0 unreachable, 1 reachable, 2 on surface; updates the navigator constraint
  CK_D int surfaceStatus(const FitParams& fp, int sid, int idx) {
    double path[2];
    int st[2];
    // the next step is min(|min(cNav, cActor, cUser)|, cAcc): a path beyond
    // 2 cAcc + 1 mm neither binds it nor is on the surface, so the mixed form
    // keeps such a path's FP32 value (the step and the status are the same)
    intersectSurf(fp, sid, path, st, 2.0 * fabs(cAcc) + 1.0);
    const double pl = idx ? path[1] : path[0];
    const int stt = idx ? st[1] : st[0];
    if (stt != 0) {
      cNav = kNotSet;
      cupdate(cNav, pl);
    }
    return stt;
  }

  CK_D bool nextTargetNav(const FitParams& fp) {
    constexpr int inc = REV ? -1 : 1;  // DirectNavigator::State::nextSurface
    currentSurface = -1;
    if (navigationBreak) return false;
    surfaceIndex += inc;
    while (surfaceIndex >= 0 && surfaceIndex < nSeq) {
      const int sid = __ldg(&fp.seq_surf[seq0 + surfaceIndex]);
      double path[2];
      int st[2];
      const int ni = intersectSurf(fp, sid, path, st);
      for (int i = 0; i < ni; ++i) {
        if (st[i] != 0 && path[i] > fp.opt.nearLimit && path[i] < kNotSet) {
          targetSurf = sid;
          targetIdx = i;
          return true;
        }
      }
      surfaceIndex += inc;
    }
    navigationBreak = true;
    return false;
  }

  CK_D bool getNextTarget(const FitParams& fp, int& e) {
    e = CK_TRACK_OK;
    for (unsigned i = 0; i < fp.opt.maxTargetSkipping; ++i) {
      if (!nextTargetNav(fp)) return false;
      const int stt = surfaceStatus(fp, targetSurf, targetIdx);
      if (stt == 2) continue;
      if (stt == 1) return true;
    }
    e = CK_TRACK_NEXT_TARGET_LIMIT;
    return false;
  }

  // ------------------------------------------------------------ material
  // PointwiseMaterialInteraction: mode 1 pre, 2 post, 3 full; on the start
  // surface only the post-update part applies (determineMaterialUpdateMode,
  // PointwiseMaterialInteraction.cpp:16-29), and the pre/post split factors
  // follow the direction of travel (ISurfaceMaterial.cpp:18-31).
  CK_NI bool material(const FitParams& fp, int sid, const Surf<double>& sfd, const Surf<P>& sp,
                      const double l[3], int mode) {
    const DevSurface* ds = fp.surfaces + sid;
    if (!(__ldg(&ds->flags) & CK_SURF_MATERIAL)) return true;
    if constexpr (REV) {
      if (sid == startSid) mode &= 2;
    }
    const P d[3] = {toP<P>(dir[0]), toP<P>(dir[1]), toP<P>(dir[2])};
    P pc;
    if (sfd.type == CK_SURFACE_PLANE) {
      pc = P(1) / fabs(sp.R[2] * d[0] + sp.R[5] * d[1] + sp.R[8] * d[2]);
    } else {
      const P l0 = toP<P>(l[0]), l1 = toP<P>(l[1]);
      P n0 = l0, n1 = l1;
      const P n2 = l0 * l0 + l1 * l1;
      if (n2 > P(0)) {
        const P nn = sqrt(n2);
        n0 = l0 / nn;
        n1 = l1 / nn;
      }
      P ez[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) ez[i] = sp.R[i * 3 + 0] * n0 + sp.R[i * 3 + 1] * n1;
      pc = fabs(P(1) / (ez[0] * d[0] + ez[1] * d[1] + ez[2] * d[2]));
    }
    if (!onSurfaceLocal(sfd, l)) return false;
    float f1 = 1.0f;
    if (__ldg(&ds->vacuum) == 0) {
      const float split = __ldg(&ds->split);
      // forward: pre 1 - split, post split; backward the other way round
      const bool firstPart = (mode == 1) != REV;
      const double factor =
          mode == 0 ? 0.0 : (mode == 3 ? 1.0 : (firstPart ? 1.0 - (double)split : (double)split));
      if (factor == 0.0) return true;
      f1 = (float)factor;
    }
    bool vac = false;
    const float qOverPf = d2f(qop);
    const MatEffects e = materialEffects<P>(fp.mc, ds, f1, (float)pc, pdg, mass, absQ, d,
                                            qOverPf, fp.opt.multipleScattering != 0,
                                            fp.opt.energyLoss != 0, vac);
    if (vac) return true;
    const float signedQ = copysignf(absQ, qOverPf);
    // the energy decreases forward and increases backward (hpp:185-190)
    const double eLoss = REV ? -e.eLoss : e.eLoss;
    if constexpr (sizeof(P) == sizeof(double)) {
      // PointwiseMaterialInteraction::updateState (hpp:188-198) in FP64
      const double massd = (double)mass;
      const double mom = absMomentum(absQ, qop);
      const double nextE = sqrt(massd * massd + mom * mom) - eLoss;
      double nextP = 0.0;
      if (massd < nextE) {
        const double am = fabs(massd);
        nextP = sqrt((nextE - am) * (nextE + am));
      }
      nextP = fmax(0.01, nextP);
      qop = (double)signedQ / nextP;
    } else {
      // the same update as a relative change of q/p: with u = nextP^2/p^2 - 1
      // = -eLoss (2E - eLoss) / p^2, q/p scales by 1/sqrt(1 + u); the small
      // correction is formed in FP32 and applied to the FP64 q/p
      const float m = mass;
      const float p = fabsf(signedQ / d2f(qop));
      const float E = sqrtf(m * m + p * p);
      const float eLossF = (float)eLoss;
      const float nextE = E - eLossF;
      if (m < nextE && (nextE - m) * (nextE + m) >= 1e-4f) {
        const float u = -eLossF * (2.0f * E - eLossF) / (p * p);
        const float r = sqrtf(1.0f + u);
        const float delta = u / (r * (1.0f + r));  // 1/sqrt(1+u) - 1 = -u/(r(1+r))
        qop = qop - qop * toD(delta);
      } else {
        qop = (double)signedQ / 0.01;  // nextP clamped to 10 MeV
      }
    }
    if (!coasting) {
      cov[sidx(2, 2)] = fmax(CV(0), cov[sidx(2, 2)] + (CV)e.varPhi);
      cov[sidx(3, 3)] = fmax(CV(0), cov[sidx(3, 3)] + (CV)e.varTheta);
      cov[sidx(4, 4)] = fmax(CV(0), cov[sidx(4, 4)] + (CV)e.varQoP);
    }
    return true;
  }

  // ------------------------------------------------- covariance transport
  // J = F2B (I + deriv fTP) T, C <- J C J^T, reinitialise T at the surface
  // (CovarianceEngine.cpp:102-165). J is returned for the record.
  // correct: KalmanFitterOptions::freeToBoundCorrection (the covariance, and
  // the free state, through the unscented transform when it applies; l is
  // then updated to the new position)
  CK_NI void transportToBound(const Surf<double>& sfd, const Surf<P>& sf, double l[3],
                              CV Jout[36], bool correct) {
    const P p[3] = {toP<P>(pos[0]), toP<P>(pos[1]), toP<P>(pos[2])};
    P ex[3], ey[3], ez[3];
    referenceFrame(sf, p, ex, ey, ez);
    const P dir[3] = {toP<P>(this->dir[0]), toP<P>(this->dir[1]), toP<P>(this->dir[2])};
    const P dz = ez[0] * dir[0] + ez[1] * dir[1] + ez[2] * dir[2];
    const P idz = P(-1) / dz;
    const P f0 = ez[0] * idz, f1 = ez[1] * idz, f2 = ez[2] * idz;
    const Trig<P> tg = trig(dir);
    const P a0 = -tg.sinPhi * tg.invSinTheta, a1 = tg.cosPhi * tg.invSinTheta;
    const P b0 = tg.cosPhi * tg.cosTheta, b1 = tg.sinPhi * tg.cosTheta, b2 = -tg.sinTheta;
    const P exd = ex[0] * deriv[0] + ex[1] * deriv[1] + ex[2] * deriv[2];
    const P eyd = ey[0] * deriv[0] + ey[1] * deriv[1] + ey[2] * deriv[2];
    const P phd = a0 * deriv[4] + a1 * deriv[5];
    const P thd = b0 * deriv[4] + b1 * deriv[5] + b2 * deriv[6];
    P J[6][6];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const P t0 = T.loc[0][c], t1 = T.loc[1][c], t2 = T.loc[2][c];
      const P sc = f0 * t0 + f1 * t1 + f2 * t2;
      J[0][c] = (ex[0] * t0 + ex[1] * t1 + ex[2] * t2) + exd * sc;
      J[1][c] = (ey[0] * t0 + ey[1] * t1 + ey[2] * t2) + eyd * sc;
      J[2][c] = phd * sc;
      J[3][c] = thd * sc;
      J[4][c] = P(0);
      J[5][c] = deriv[3] * sc;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const P t0 = T.dyn[0][c], t1 = T.dyn[1][c], t2 = T.dyn[2][c];
      const P sc = f0 * t0 + f1 * t1 + f2 * t2;
      const P g0 = T.dyn[4][c], g1 = T.dyn[5][c], g2 = T.dyn[6][c];
      J[0][2 + c] = (ex[0] * t0 + ex[1] * t1 + ex[2] * t2) + exd * sc;
      J[1][2 + c] = (ey[0] * t0 + ey[1] * t1 + ey[2] * t2) + eyd * sc;
      J[2][2 + c] = (a0 * g0 + a1 * g1) + phd * sc;
      J[3][2 + c] = (b0 * g0 + b1 * g1 + b2 * g2) + thd * sc;
      J[4][2 + c] = (c == 2) ? P(1) : P(0);
      J[5][2 + c] = T.dyn[3][c] + deriv[3] * sc;
    }
#pragma unroll
    for (int r = 0; r < 6; ++r) J[r][5] = (r == 5) ? P(1) : P(0);
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) Jout[r * 6 + c] = (CV)J[r][c];
    if constexpr (F2B) {
      if (correct && correctTransport(sfd, l)) {
#pragma unroll
        for (int i = 0; i < 7; ++i) deriv[i] = P(0);
        if (onSurfaceLocal(sfd, l)) initTP(sf);
        return;
      }
    }
    // C <- J C J^T (packed); J row 4 is e4 and column 5 is e5
    CV JC[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        CV acc;
        if (i == 4) {
          acc = cov[sidx(4, j)];
        } else {
          acc = (CV)J[i][0] * cov[sidx(0, j)];
#pragma unroll
          for (int k = 1; k < 5; ++k) acc += (CV)J[i][k] * cov[sidx(k, j)];
          if (i == 5) acc += cov[sidx(5, j)];
        }
        JC[i][j] = acc;
      }
    CV outc[21];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j) {
        CV acc;
        if (j == 4) {
          acc = JC[i][4];
        } else {
          acc = JC[i][0] * (CV)J[j][0];
#pragma unroll
          for (int k = 1; k < 5; ++k) acc += JC[i][k] * (CV)J[j][k];
          if (j == 5) acc += JC[i][5];
        }
        outc[sidx(i, j)] = acc;
      }
#pragma unroll
    for (int i = 0; i < 21; ++i) cov[i] = outc[i];
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    if (onSurfaceLocal(sfd, l)) initTP(sf);
  }

  // CovarianceEngine.cpp:120-144 with CorrectedFreeToBoundTransformer: the
  // free covariance T C T^T goes through the unscented transform; when it
  // applies, the bound covariance is its result and the free state moves to
  // the corrected mean. The operands are copied to local arrays for the
  // out-of-line transformer (the option is off in the common case).
  CK_D bool correctTransport(const Surf<double>& sfd, double l[3]) {
    P tl[6], td[21];
    CV c[21];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
      for (int k = 0; k < 2; ++k) tl[r * 2 + k] = T.loc[r][k];
#pragma unroll
    for (int r = 0; r < 7; ++r)
#pragma unroll
      for (int k = 0; k < 3; ++k) td[r * 3 + k] = T.dyn[r][k];
#pragma unroll
    for (int i = 0; i < 21; ++i) c[i] = cov[i];
    const double fr[8] = {pos[0], pos[1], pos[2], tim, dir[0], dir[1], dir[2], qop};
    double mean[6], bc[21];
    if (!correctedTransport<P, CV>(sfd, tl, td, c, fr, mean, bc)) return false;
    boundToFree(sfd, mean);
#pragma unroll
    for (int i = 0; i < 21; ++i) cov[i] = (CV)bc[i];
    local(sfd, l);
    return true;
  }

  // --------------------------------------------------------------- actor
  CK_D void writeMeta(const FitParams& fp, int slot, int k, int sid, uint32_t flags, double chi2) {
    RecState<CV>& r = Rec<CV>(fp, slot).s(k);
    r.surface = sid;
    r.flags = (int32_t)flags;
    r.pathLength = pathAcc;
    r.chi2 = chi2;
  }

  // KalmanFitter::Actor::filter on surface `sid`
  CK_D int filter(const FitParams& fp, int slot, int sid) {
    const Rec<CV> rec(fp, slot);
    Surf<double> sf;
    sf.load(fp.surfaces + sid);
    Surf<P> spv;
    if constexpr (sizeof(P) == sizeof(float)) spv.load(fp.surfaces + sid);
    const Surf<P>& sp = pickSurf<P>(sf, spv);
    const int sflags = __ldg(&fp.surfaces[sid].flags);
    const bool sensitive = (sflags & CK_SURF_SENSITIVE) != 0;
    const bool hasMat = (sflags & CK_SURF_MATERIAL) != 0;
    const bool preceding = measurementStates > 0;
    // local coordinates of the position on arrival (the position changes
    // only with the update below)
    double l[3];
    local(sf, l);
    if (coasting) {
      if ((preceding && sensitive) || hasMat) {
        double bp[6];
        if (!freeToBound(fp, sf, l, bp)) return CK_TRACK_NOT_ON_SURFACE;
        if (!material(fp, sid, sf, sp, l, 3)) return CK_TRACK_NOT_ON_SURFACE;
      }
      return CK_TRACK_OK;
    }
    const int mi = findMeasHinted(fp, sid);
    if (mi >= 0) {
      CV J[36];
      transportToBound(sf, sp, l, J, fp.opt.freeToBoundCorrection != 0);
      if (!material(fp, sid, sf, sp, l, 1)) return CK_TRACK_NOT_ON_SURFACE;
      double bp[6];
      if (!freeToBound(fp, sf, l, bp)) return CK_TRACK_NOT_ON_SURFACE;
      // (the reversed pass's states are not part of the track: no records)
      if (!REV && nStates >= fp.max_states) return CK_TRACK_TOO_MANY_STATES;
      const int k = nStates++;
      // the mixed form's update and predicted chi2 run in FP32 on its float
      // covariance (with the free-to-bound correction, whose unscented
      // transform is sensitive to it, in FP64)
      constexpr bool kF32Update = sizeof(CV) == sizeof(float) && !F2B;
      double Pp[21];
      if constexpr (!kF32Update) {
#pragma unroll
        for (int i = 0; i < 21; ++i) Pp[i] = toD(cov[i]);
      }
      if constexpr (!REV) {
#pragma unroll
        for (int i = 0; i < 6; ++i) rec.p(k, kRecPred + i) = bp[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) rec.m(k, kRecPredCov + i) = cov[i];
#pragma unroll
        for (int i = 0; i < 36; ++i) rec.m(k, kRecJac + i) = J[i];
      }
      uint32_t flags = CK_FLAG_HAS_PARAMETERS | (hasMat ? CK_FLAG_HAS_MATERIAL : 0u);
      const double mv0 = __ldg(&fp.meas_val[2 * (size_t)mi]);
      const double mv1 = __ldg(&fp.meas_val[2 * (size_t)mi + 1]);
      double V[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) V[i] = __ldg(&fp.meas_cov[4 * (size_t)mi + i]);
      // (loc0, loc1), or a 1D measurement of loc h (value mv0, variance V[0])
      const int sub = fp.meas_sub ? __ldg(&fp.meas_sub[mi]) : CK_MEAS_LOC01;
      flags |= (uint32_t)sub << kRecSubShift;
      bool outlier = false;
      constexpr bool kFastRcp = sizeof(P) == sizeof(float);
      if (fp.opt.useOutlierCut) {
        if constexpr (kF32Update)
          outlier = predictedChi2SubF(bp, cov, sub, mv0, mv1, V) > fp.opt.outlierChi2Cut;
        else
          outlier = predictedChi2Sub<kFastRcp>(bp, Pp, sub, mv0, mv1, V) > fp.opt.outlierChi2Cut;
      }
      double chi2 = 0.0;
      if (!outlier) {
        double filt[6];
        CV F[21];
        const bool joseph = fp.opt.joseph != 0;
        if constexpr (kF32Update) {
          if (!kalmanUpdateSubF(bp, cov, sub, mv0, mv1, V, joseph, filt, F, chi2))
            return CK_TRACK_UPDATE_FAILED;
        } else {
          double Fd[21];
          if (!kalmanUpdateSub<kFastRcp>(bp, Pp, sub, mv0, mv1, V, joseph, filt, Fd, chi2))
            return CK_TRACK_UPDATE_FAILED;
#pragma unroll
          for (int i = 0; i < 21; ++i) F[i] = toP<CV>(Fd[i]);
        }
        flags |= CK_FLAG_HAS_MEASUREMENT;
        if constexpr (REV) {
          // the latest filtered measurement state of the reversed pass
          // (findLastMeasurementState of the reversed track)
          ExtStart& es = fp.ext[2 * (size_t)slot];
#pragma unroll
          for (int i = 0; i < 6; ++i) es.par[i] = filt[i];
#pragma unroll
          for (int i = 0; i < 21; ++i) es.cov[i] = (double)F[i];
          es.surface = sid;
        } else {
#pragma unroll
          for (int i = 0; i < 6; ++i) rec.p(k, kRecFilt + i) = filt[i];
        }
        updateFree(sf, bp, filt, l);
#pragma unroll
        for (int i = 0; i < 21; ++i) {
          cov[i] = F[i];
          if constexpr (!REV) rec.m(k, kRecFiltCov + i) = cov[i];
        }
        initTP(sp);
        local(sf, l);  // the updated position
        ++measurementStates;
      } else if constexpr (!REV) {
        flags |= CK_FLAG_HAS_MEASUREMENT | CK_FLAG_IS_OUTLIER;
#pragma unroll
        for (int i = 0; i < 6; ++i) rec.p(k, kRecFilt + i) = bp[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) rec.m(k, kRecFiltCov + i) = cov[i];
      }
      if constexpr (!REV) writeMeta(fp, slot, k, sid, flags, chi2);
      if (!material(fp, sid, sf, sp, l, 2)) return CK_TRACK_NOT_ON_SURFACE;
      if constexpr (!REV) lastMeasurementIndex = k;
    } else if ((preceding && sensitive) || hasMat) {
      double bp[6];
      if (!freeToBound(fp, sf, l, bp)) return CK_TRACK_NOT_ON_SURFACE;
      CV J[36];
      transportToBound(sf, sp, l, J, fp.opt.freeToBoundCorrection != 0);
      if constexpr (!REV) {
        if (nStates >= fp.max_states) return CK_TRACK_TOO_MANY_STATES;
        const int k = nStates++;
#pragma unroll
        for (int i = 0; i < 6; ++i) {
          rec.p(k, kRecPred + i) = bp[i];
          rec.p(k, kRecFilt + i) = bp[i];
        }
#pragma unroll
        for (int i = 0; i < 21; ++i) {
          rec.m(k, kRecPredCov + i) = cov[i];
          rec.m(k, kRecFiltCov + i) = cov[i];
        }
#pragma unroll
        for (int i = 0; i < 36; ++i) rec.m(k, kRecJac + i) = J[i];
        uint32_t flags = CK_FLAG_HAS_PARAMETERS | (hasMat ? CK_FLAG_HAS_MATERIAL : 0u);
        if (sensitive && preceding) flags |= CK_FLAG_IS_HOLE;
        writeMeta(fp, slot, k, sid, flags, 0.0);
      }
      if (!material(fp, sid, sf, sp, l, 3)) return CK_TRACK_NOT_ON_SURFACE;
    }
    return CK_TRACK_OK;
  }

  // Actor::act: filter on the current surface (if any) and the finalisation
  // checks (KalmanFitter.hpp:337-422)
  CK_D int act(const FitParams& fp, int slot) {
    if (finished) return CK_TRACK_OK;
    if (kfLimit == kNotSet) kfLimit = loopLimit(fp, kfLimit, true);
    if (currentSurface >= 0) {
      const int r = filter(fp, slot, currentSurface);
      if (r != CK_TRACK_OK) return r;
    }
    bool complete = measurementStates == nDistinct;
    if (!complete && lastSlSeq >= 0 && currentSurface >= 0 &&
        (REV ? surfaceIndex <= lastSlSeq : surfaceIndex >= lastSlSeq)) {
      // every later state would lie beyond the track's tip
      if (fp.opt.earlyTermination)
        complete = true;
      else if (!REV || fp.ref_surface < 0)
        coasting = true;  // (a reversed pass that may reach its target keeps its covariance)
    }
    const bool pathReached = pathLimitReached(fp, kfLimit);
    bool targetReached = false;
    if constexpr (REV) {
      if (fp.ref_surface >= 0) {
        // Actor::targetReached, a SurfaceReached on the reference surface
        // with an unlimited near limit (StandardAborters.hpp:94-155): its
        // distance becomes the actor step constraint
        Surf<double> ts;
        ts.load(fp.surfaces + fp.ref_surface);
        const double nd[3] = {-dir[0], -dir[1], -dir[2]};
        const double tol = fp.opt.surfaceTolerance;
        double u = 0.0;
        if (lineIntersect(ts, pos, nd, tol, u)) {
          cActor = kNotSet;
          cupdate(cActor, u);
          targetReached = !(fabs(u) > fabs(tol));
        }
        if (targetReached) {
          // the fitted parameters: the bound state on the target
          // (KalmanFitter.hpp:398-412)
          if (!writeReferenceState(fp, fp.ref_surface)) return CK_TRACK_NOT_ON_SURFACE;
          fp.ext[2 * (size_t)slot].fitted = 1;
        }
      }
    }
    if (complete || pathReached || targetReached) finished = true;
    return CK_TRACK_OK;
  }

  CK_D bool checkAbort(const FitParams& fp) {
    if (finished) return true;
    return pathLimitReached(fp, propLimit);
  }

  // after act(): abort check and the next target; ends propagation or
  // returns to STEP
  CK_D void afterAct(const FitParams& fp, int slot) {
    if (checkAbort(fp)) {
      endPropagation(fp, slot);
      return;
    }
    if (!haveTarget) {
      cNav = kNotSet;
      int e;
      haveTarget = getNextTarget(fp, e);
      if (e != CK_TRACK_OK) {
        fail(fp, e);
        return;
      }
    }
    phase = PH_STEP;
  }

  // ------------------------------------------------------------- phases
  // FETCH: initialise track t (EigenStepper::initialize, Propagator
  // pre-stepping: act, checkAbort, first target)
  CK_D void start(const FitParams& fp, int slot, int track) {
    t = track;
    seq0 = __ldg(&fp.seq_off[t]);
    nSeq = __ldg(&fp.seq_off[t + 1]) - seq0;
    m0 = __ldg(&fp.meas_off[t]);
    nMeas = __ldg(&fp.meas_off[t + 1]) - m0;
    {
      bool bad = nSeq < 0 || nMeas < 0;
      // (a line surface is only a reference surface: not in a sequence, no
      // measurement on it)
      for (int i = 0; i < nSeq && !bad; ++i) {
        const int sid = __ldg(&fp.seq_surf[seq0 + i]);
        bad |= sid < 0 || sid >= fp.n_surfaces || __ldg(&fp.surfaces[sid].type) == CK_SURFACE_LINE;
      }
      for (int i = 0; i < nMeas && !bad; ++i) {
        const int sid = __ldg(&fp.meas_surf[m0 + i]);
        bad |= sid < 0 || sid >= fp.n_surfaces || __ldg(&fp.surfaces[sid].type) == CK_SURFACE_LINE;
        if (fp.meas_sub) {
          const int sub = __ldg(&fp.meas_sub[m0 + i]);
          bad |= sub < CK_MEAS_LOC0 || sub > CK_MEAS_LOC01;
        }
      }
      if (bad) {
        fail(fp, CK_TRACK_INVALID_INPUT);
        return;
      }
    }
    {
      double sp[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) sp[i] = __ldg(&fp.start_params[6 * (size_t)t + i]);
      Surf<double> start;
      start.loadPlane(fp.start_frames + 12 * (size_t)t);
      boundToFree(start, sp);
      initT(start);
      const double* sc = fp.start_cov + 36 * (size_t)t;
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = i; j < 6; ++j) cov[sidx(i, j)] = toP<CV>(__ldg(&sc[i * 6 + j]));
    }
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    pathAcc = 0.0;
    cNav = kNotSet;
    cActor = kNotSet;
    cUser = fp.opt.maxStepSize;
    cAcc = fp.opt.initialStepSize;
    mass = __ldg(&fp.particle[2 * (size_t)t]);
    absQ = __ldg(&fp.particle[2 * (size_t)t + 1]);
    pdg = fp.pdg ? __ldg(&fp.pdg[t]) : 211;
    nDistinct = 0;
    for (int i = 0; i < nMeas; ++i) {
      const int si = __ldg(&fp.meas_surf[m0 + i]);
      bool dup = false;
      for (int j = 0; j < i; ++j) dup |= (__ldg(&fp.meas_surf[m0 + j]) == si);
      nDistinct += dup ? 0 : 1;
    }
    // the last sequence position that carries a source link
    lastSlSeq = -1;
    for (int k = nSeq - 1; k >= 0; --k)
      if (findMeas(fp, __ldg(&fp.seq_surf[seq0 + k])) >= 0) {
        lastSlSeq = k;
        break;
      }
    measHint = 0;
    dirSign = 1.0;
    extrapolating = false;
    propLimit = loopLimit(fp, fp.opt.pathLimit, false);
    kfLimit = kNotSet;
    surfaceIndex = -1;
    navigationBreak = false;
    currentSurface = -1;
    prePropagation(fp, slot);
  }

  // the common tail of both passes' initialisation: the actor's first call,
  // the abort check and the first navigation target
  CK_D void prePropagation(const FitParams& fp, int slot) {
    targetSurf = -1;
    targetIdx = 0;
    haveTarget = false;
    nStates = 0;
    if constexpr (!REV) lastMeasurementIndex = -1;
    measurementStates = 0;
    finished = false;
    coasting = false;
    stepStarted = false;
    steps = 0;
    const int err = act(fp, slot);
    if (err != CK_TRACK_OK) {
      fail(fp, err);
      return;
    }
    if (checkAbort(fp)) {
      endPropagation(fp, slot);
      return;
    }
    int e;
    haveTarget = getNextTarget(fp, e);
    if (e != CK_TRACK_OK) {
      fail(fp, e);
      return;
    }
    phase = PH_STEP;
  }

  // FETCH of the reversed pass (KalmanFitter.hpp:901-911): the start
  // parameters are the forward pass's last measurement state's filtered ones
  // (its smoothed parameters share them), the covariance scaled by
  // reverseFilteringCovarianceScaling; the DirectNavigator starts on that
  // surface (DirectNavigator.hpp:238-262) and the first actor call filters
  // it. Tracks the forward pass failed are skipped.
  CK_D void startReverse(const FitParams& fp, int slot, int track) {
    t = track;
    const int tip = fp.tip[slot];
    if (tip < 0 || !reverseSelected<CV>(fp, slot, tip)) {
      phase = PH_FETCH;
      return;
    }
    seq0 = __ldg(&fp.seq_off[t]);
    nSeq = __ldg(&fp.seq_off[t + 1]) - seq0;
    m0 = __ldg(&fp.meas_off[t]);
    nMeas = __ldg(&fp.meas_off[t + 1]) - m0;
    const Rec<CV> rec(fp, slot);
    int last = tip;
    for (int k = tip; k >= 0; --k) {
      const uint32_t fl = (uint32_t)rec.s(k).flags;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
        last = k;
        break;
      }
    }
    const int sid = rec.s(last).surface;
    {
      Surf<double> sf;
      sf.load(fp.surfaces + sid);
      double b[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) b[i] = rec.p(last, kRecFilt + i);
      boundToFree(sf, b);
      initT(sf);
      const CV scale = (CV)fp.opt.reverseCovScaling;
#pragma unroll
      for (int i = 0; i < 21; ++i) cov[i] = rec.m(last, kRecFiltCov + i) * scale;
    }
    ExtStart& es = fp.ext[2 * (size_t)slot];
    es.surface = -1;
    es.fitted = 0;
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    pathAcc = 0.0;
    cNav = kNotSet;
    cActor = kNotSet;
    cUser = fp.opt.maxStepSize;
    cAcc = fp.opt.initialStepSize;
    mass = __ldg(&fp.particle[2 * (size_t)t]);
    absQ = __ldg(&fp.particle[2 * (size_t)t + 1]);
    pdg = fp.pdg ? __ldg(&fp.pdg[t]) : 211;
    nDistinct = 0;
    for (int i = 0; i < nMeas; ++i) {
      const int si = __ldg(&fp.meas_surf[m0 + i]);
      bool dup = false;
      for (int j = 0; j < i; ++j) dup |= (__ldg(&fp.meas_surf[m0 + j]) == si);
      nDistinct += dup ? 0 : 1;
    }
    // the first sequence position that carries a source link
    lastSlSeq = -1;
    for (int k = 0; k < nSeq; ++k)
      if (findMeas(fp, __ldg(&fp.seq_surf[seq0 + k])) >= 0) {
        lastSlSeq = k;
        break;
      }
    measHint = 0;
    dirSign = -1.0;
    extrapolating = false;
    propLimit = loopLimit(fp, fp.opt.pathLimit, false);
    kfLimit = kNotSet;
    // the position after the start surface's first occurrence, or the end
    surfaceIndex = nSeq;
    for (int k = 0; k < nSeq; ++k)
      if (__ldg(&fp.seq_surf[seq0 + k]) == sid) {
        surfaceIndex = k + 1;
        break;
      }
    navigationBreak = false;
    currentSurface = sid;
    startSid = sid;
    prePropagation(fp, slot);
  }

  // the field at a Runge-Kutta stage point
  CK_D bool stageField(const FitParams& fp, const P p[3], P B[3]) const {
    return getField(fp.field, p, B);
  }

  // STEP: one Runge-Kutta trial (EigenStepper::step, EigenStepper.ipp:168-388)
  // MODE (StepMode): the lane fits, extrapolates to the reference surface or
  // propagates (signed step direction, the aborters after each step); the
  // fit kernels instantiate the forward-only step without the other code
  template <int MODE = kStepFit>
  CK_D void step(const FitParams& fp, int slot) {
    const DevOptions& o = fp.opt;
    if (!stepStarted) {
      if (steps >= o.maxSteps) {
        fail(fp, CK_TRACK_STEP_COUNT_LIMIT);
        return;
      }
      initialH = stepValue();
      if constexpr (MODE != kStepFit || REV) initialH *= dirSign;  // EigenStepper.ipp:272
      hd = initialH;
      trials = 0;
      stepStarted = true;
    }
    ++trials;
    const P pp[3] = {toP<P>(pos[0]), toP<P>(pos[1]), toP<P>(pos[2])};
    const P dir[3] = {toP<P>(this->dir[0]), toP<P>(this->dir[1]), toP<P>(this->dir[2])};
    const P qop = toP<P>(this->qop);
    P B1[3], B2[3], B3[3];
    if (!stageField(fp, pp, B1)) {
      fail(fp, CK_TRACK_FIELD_OUT_OF_BOUNDS);
      return;
    }
    P k1[3], k2[3], k3[3], k4[3];
    k1[0] = qop * (dir[1] * B1[2] - dir[2] * B1[1]);
    k1[1] = qop * (dir[2] * B1[0] - dir[0] * B1[2]);
    k1[2] = qop * (dir[0] * B1[1] - dir[1] * B1[0]);
    const P tol = toP<P>(o.stepTolerance);
    const P h = toP<P>(hd);
    const P h2 = h * h;
    const P hh = h * P(0.5);
    P p1[3], tt[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) p1[i] = pp[i] + hh * dir[i] + h2 * P(0.125) * k1[i];
    if (!stageField(fp, p1, B2)) {
      fail(fp, CK_TRACK_FIELD_OUT_OF_BOUNDS);
      return;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) tt[i] = dir[i] + hh * k1[i];
    k2[0] = qop * (tt[1] * B2[2] - tt[2] * B2[1]);
    k2[1] = qop * (tt[2] * B2[0] - tt[0] * B2[2]);
    k2[2] = qop * (tt[0] * B2[1] - tt[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) tt[i] = dir[i] + hh * k2[i];
    k3[0] = qop * (tt[1] * B2[2] - tt[2] * B2[1]);
    k3[1] = qop * (tt[2] * B2[0] - tt[0] * B2[2]);
    k3[2] = qop * (tt[0] * B2[1] - tt[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) p1[i] = pp[i] + h * dir[i] + h2 * P(0.5) * k3[i];
    if (!stageField(fp, p1, B3)) {
      fail(fp, CK_TRACK_FIELD_OUT_OF_BOUNDS);
      return;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) tt[i] = dir[i] + h * k3[i];
    k4[0] = qop * (tt[1] * B3[2] - tt[2] * B3[1]);
    k4[1] = qop * (tt[2] * B3[0] - tt[0] * B3[2]);
    k4[2] = qop * (tt[0] * B3[1] - tt[1] * B3[0]);
    const P l1 = fabs(((k1[0] - k2[0]) - k3[0]) + k4[0]) + fabs(((k1[1] - k2[1]) - k3[1]) + k4[1]) +
                 fabs(((k1[2] - k2[2]) - k3[2]) + k4[2]);
    P err = h2 * l1;
    err = fmax(err, (P)1e-20);
    P x = sqrt(sqrt(tol / err));
    x = fmin(fmax(x, P(0.25)), P(4));
    if (!(err <= P(4) * tol)) {
      hd = hd * toD(x);
      if (fabs(hd) < fabs(o.stepSizeCutOff)) {
        fail(fp, CK_TRACK_STEP_SIZE_STALLED);
        return;
      }
      if (trials > o.maxRkTrials) fail(fp, CK_TRACK_STEP_ADJUST_FAILED);
      return;  // next trial in a later STEP iteration
    }
    // accepted: propagateTime + transportMatrix (EigenStepperDefaultExtension.hpp:86-228)
    const P m = (P)mass;
    const P pm = absMomentum(absQ, qop);
    const P mp = m / pm;
    const P dtds = sqrt(P(1) + mp * mp);
    tim = tim + toD(h * dtds);
    if (!coasting) {
      deriv[3] = dtds;
      P dk1dL[3], dk2dL[3], dk3dL[3], dk4dL[3];
      dk1dL[0] = dir[1] * B1[2] - dir[2] * B1[1];
      dk1dL[1] = dir[2] * B1[0] - dir[0] * B1[2];
      dk1dL[2] = dir[0] * B1[1] - dir[1] * B1[0];
      const P qh = qop * hh, qf = qop * h;
#pragma unroll
      for (int i = 0; i < 3; ++i) tt[i] = dir[i] + hh * k1[i];
      dk2dL[0] = (tt[1] * B2[2] - tt[2] * B2[1]) + qh * (dk1dL[1] * B2[2] - dk1dL[2] * B2[1]);
      dk2dL[1] = (tt[2] * B2[0] - tt[0] * B2[2]) + qh * (dk1dL[2] * B2[0] - dk1dL[0] * B2[2]);
      dk2dL[2] = (tt[0] * B2[1] - tt[1] * B2[0]) + qh * (dk1dL[0] * B2[1] - dk1dL[1] * B2[0]);
#pragma unroll
      for (int i = 0; i < 3; ++i) tt[i] = dir[i] + hh * k2[i];
      dk3dL[0] = (tt[1] * B2[2] - tt[2] * B2[1]) + qh * (dk2dL[1] * B2[2] - dk2dL[2] * B2[1]);
      dk3dL[1] = (tt[2] * B2[0] - tt[0] * B2[2]) + qh * (dk2dL[2] * B2[0] - dk2dL[0] * B2[2]);
      dk3dL[2] = (tt[0] * B2[1] - tt[1] * B2[0]) + qh * (dk2dL[0] * B2[1] - dk2dL[1] * B2[0]);
#pragma unroll
      for (int i = 0; i < 3; ++i) tt[i] = dir[i] + h * k3[i];
      dk4dL[0] = (tt[1] * B3[2] - tt[2] * B3[1]) + qf * (dk3dL[1] * B3[2] - dk3dL[2] * B3[1]);
      dk4dL[1] = (tt[2] * B3[0] - tt[0] * B3[2]) + qf * (dk3dL[2] * B3[0] - dk3dL[0] * B3[2]);
      dk4dL[2] = (tt[0] * B3[1] - tt[1] * B3[0]) + qf * (dk3dL[0] * B3[1] - dk3dL[1] * B3[0]);
      P d1[3][3], d2[3][3], d3[3][3], d4[3][3];
      d1[0][0] = P(0);
      d1[0][1] = qop * B1[2];
      d1[0][2] = -qop * B1[1];
      d1[1][0] = -qop * B1[2];
      d1[1][1] = P(0);
      d1[1][2] = qop * B1[0];
      d1[2][0] = qop * B1[1];
      d1[2][1] = -qop * B1[0];
      d1[2][2] = P(0);
      auto crossCols = [&](const P in[3][3], const P* B, P outm[3][3]) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const P c0 = in[0][j], c1 = in[1][j], c2 = in[2][j];
          outm[0][j] = qop * (c1 * B[2] - c2 * B[1]);
          outm[1][j] = qop * (c2 * B[0] - c0 * B[2]);
          outm[2][j] = qop * (c0 * B[1] - c1 * B[0]);
        }
      };
      P tmp[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tmp[i][j] = (i == j ? P(1) : P(0)) + hh * d1[i][j];
      crossCols(tmp, B2, d2);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tmp[i][j] = (i == j ? P(1) : P(0)) + hh * d2[i][j];
      crossCols(tmp, B2, d3);
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) tmp[i][j] = (i == j ? P(1) : P(0)) + h * d3[i][j];
      crossCols(tmp, B3, d4);
      const P h6 = h * P(1.0 / 6.0);
      const P hh6 = h2 * P(1.0 / 6.0);
      P dFdT[3][3], dGdT[3][3], dFdL[3], dGdL[3];
#pragma unroll
      for (int i = 0; i < 3; ++i) {
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const P id = (i == j) ? P(1) : P(0);
          dFdT[i][j] = (id + h6 * ((d1[i][j] + d2[i][j]) + d3[i][j])) * h;
          dGdT[i][j] = id + h6 * ((d1[i][j] + P(2) * (d2[i][j] + d3[i][j])) + d4[i][j]);
        }
        dFdL[i] = hh6 * ((dk1dL[i] + dk2dL[i]) + dk3dL[i]);
        dGdL[i] = h6 * ((dk1dL[i] + P(2) * (dk2dL[i] + dk3dL[i])) + dk4dL[i]);
      }
      const P D37 = h * m * m / (pm * pm * qop * dtds);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const P g0 = T.dyn[4][c], g1 = T.dyn[5][c], g2 = T.dyn[6][c];
        const P t7 = (c == 2) ? P(1) : P(0);
#pragma unroll
        for (int i = 0; i < 3; ++i)
          T.dyn[i][c] =
              T.dyn[i][c] + (dFdT[i][0] * g0 + dFdT[i][1] * g1 + dFdT[i][2] * g2 + dFdL[i] * t7);
        T.dyn[3][c] = T.dyn[3][c] + D37 * t7;
#pragma unroll
        for (int i = 0; i < 3; ++i)
          T.dyn[4 + i][c] = dGdT[i][0] * g0 + dGdT[i][1] * g1 + dGdT[i][2] * g2 + dGdL[i] * t7;
      }
    }
    // parameter update (EigenStepper.ipp:354-366)
    {
      const P hh6 = h2 * P(1.0 / 6.0);
      const P h6 = h * P(1.0 / 6.0);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        pos[i] = pos[i] + (hd * this->dir[i] + toD(hh6 * ((k1[i] + k2[i]) + k3[i])));
        this->dir[i] = this->dir[i] + toD(h6 * ((k1[i] + P(2) * (k2[i] + k3[i])) + k4[i]));
      }
      double* nd = this->dir;
      const double n2 = nd[0] * nd[0] + nd[1] * nd[1] + nd[2] * nd[2];
      double inv;
      if constexpr (sizeof(P) == sizeof(float)) {
        // |dir|^2 is within a few 1e-3 of 1: an FP32 reciprocal square root
        // and one Newton step in FP64 give ~1e-14 relative accuracy
        const double y0 = toD(rsqrtf(d2f(n2)));
        inv = y0 * (1.5 - 0.5 * n2 * y0 * y0);
      } else {
        inv = 1.0 / sqrt(n2);
      }
      nd[0] = nd[0] * inv;
      nd[1] = nd[1] * inv;
      nd[2] = nd[2] * inv;
    }
    if (!coasting) {
      deriv[0] = toP<P>(this->dir[0]);
      deriv[1] = toP<P>(this->dir[1]);
      deriv[2] = toP<P>(this->dir[2]);
      deriv[4] = k4[0];
      deriv[5] = k4[1];
      deriv[6] = k4[2];
    }
    pathAcc += hd;
    const double nextAcc = fabs(hd * toD(x));
    if (nextAcc < fabs(initialH) || nextAcc > fabs(cAcc)) cAcc = nextAcc;
    stepStarted = false;
    ++steps;
    // post-step navigation (Propagator.ipp:113-141)
    cNav = kNotSet;
    cActor = kNotSet;
    if constexpr (MODE == kStepExtrapolate) {
      // no navigation target and no actors; the aborters decide
      if (extrapolationAbort(fp)) finishExtrapolation(fp);
      return;
    }
    if constexpr (MODE == kStepPropagate) {
      if (propagationAbort(fp)) finishPropagation(fp);
      return;
    }
    if constexpr (MODE == kStepCkf) {
      // a branch restart keeps the target of the branch before it
      // (DirectNavigator::checkTargetValid is always true) while the
      // sequence index restarts at the new branch's surface; a target reached
      // with the index before the sequence start sets no current surface
      if (haveTarget) {
        const int post = surfaceStatus(fp, targetSurf, targetIdx);
        if (post == 2 && !navigationBreak && surfaceIndex >= 0 && surfaceIndex < nSeq)
          currentSurface = __ldg(&fp.seq_surf[seq0 + surfaceIndex]);
        if (post != 1) haveTarget = false;
      }
      phase = PH_SURFACE;
      return;
    }
    if (haveTarget) {
      const int post = surfaceStatus(fp, targetSurf, targetIdx);
      if (post == 2 && !navigationBreak) currentSurface = __ldg(&fp.seq_surf[seq0 + surfaceIndex]);
      if (post != 1) haveTarget = false;
    }
    if (currentSurface >= 0) {
      phase = PH_SURFACE;  // the actor's filter runs in the SURFACE phase
      return;
    }
    const int e = act(fp, slot);
    if (e != CK_TRACK_OK) {
      fail(fp, e);
      return;
    }
    afterAct(fp, slot);
  }

  // ------------------------------------ extrapolation to the reference surface
  // extrapolateTrackToReferenceSurface (TrackHelpers.hpp:339-381): a plain
  // propagation (no actors; DirectNavigator without surfaces) from a smoothed
  // track state to the reference line surface with the ForcedSurfaceReached
  // and PathLimitReached aborters (StandardAborters.hpp:66-164), in the
  // direction of the straight-line distance to it; fp.opt holds the
  // reference's default propagator options here.

  // LineSurface::intersect (LineSurface.cpp:141-185): false when the track
  // is parallel to the line (invalid intersection)
  CK_D static bool lineIntersect(const Surf<double>& s, const double p[3], const double d[3],
                                 double tol, double& u) {
    const double eb[3] = {s.R[2], s.R[5], s.R[8]};
    const double mab[3] = {s.c[0] - p[0], s.c[1] - p[1], s.c[2] - p[2]};
    const double eaTeb = d[0] * eb[0] + d[1] * eb[1] + d[2] * eb[2];
    const double denom = 1.0 - eaTeb * eaTeb;
    if (fabs(denom) < fabs(tol)) return false;
    const double ma = mab[0] * d[0] + mab[1] * d[1] + mab[2] * d[2];
    const double mb = mab[0] * eb[0] + mab[1] * eb[1] + mab[2] * eb[2];
    u = (ma - mb * eaTeb) / denom;
    return true;
  }

  CK_D void startExtrapolation(const FitParams& fp, int queuePos, int track, const ExtStart& es,
                               double distance) {
    t = track;
    q = queuePos;
    extrapolating = true;
    dirSign = distance >= 0.0 ? 1.0 : -1.0;  // Direction::fromScalarZeroAsPositive
    Surf<double> sf;
    sf.load(fp.surfaces + es.surface);
    boundToFree(sf, es.par);
    initT(sf);
#pragma unroll
    for (int i = 0; i < 21; ++i) cov[i] = (CV)es.cov[i];
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    pathAcc = 0.0;
    cNav = kNotSet;
    cActor = kNotSet;
    cUser = fp.opt.maxStepSize;
    cAcc = fp.opt.initialStepSize;
    mass = __ldg(&fp.particle[2 * (size_t)t]);
    absQ = __ldg(&fp.particle[2 * (size_t)t + 1]);
    pdg = fp.pdg ? __ldg(&fp.pdg[t]) : 211;
    coasting = false;
    finished = false;
    stepStarted = false;
    steps = 0;
    haveTarget = false;
    navigationBreak = true;
    currentSurface = -1;
    propLimit = loopLimit(fp, fp.opt.pathLimit, false);
    phase = PH_STEP;
    if (extrapolationAbort(fp)) finishExtrapolation(fp);  // pre-propagation check
  }

  // the aborters in list order, the first that fires ends the propagation:
  // the target (its distance becomes the actor step constraint), then the
  // path limit
  CK_D bool extrapolationAbort(const FitParams& fp) {
    Surf<double> ts;
    ts.load(fp.surfaces + fp.ref_surface);
    const double d[3] = {dirSign * dir[0], dirSign * dir[1], dirSign * dir[2]};
    const double tol = fp.opt.surfaceTolerance;
    double u = 0.0;
    const bool valid = lineIntersect(ts, pos, d, tol, u);
    if (valid) {
      cActor = kNotSet;  // updateSingleSurfaceStatus: release, then update
      cupdate(cActor, u);
      if (!(fabs(u) > fabs(tol))) return true;  // on surface
    }
    return pathLimitReached(fp, propLimit);
  }

  CK_D void finishExtrapolation(const FitParams& fp) {
    if (!writeReferenceState(fp, fp.ref_surface)) {
      fail(fp, CK_TRACK_NOT_ON_SURFACE);
      return;
    }
    phase = PH_DONE;
  }

  // EigenStepper::boundState on the reference surface, written as the
  // track's parameters and covariance:
  // J = F2B (I + derivative x freeToPath) T with the line surface's frame and
  // path derivative (LineSurface.cpp:102-115,224-251), C <- J C J^T, and the
  // bound parameters (LineSurface::globalToLocal, LineSurface.cpp:70-96);
  // false when the position is not on the line
  // (sid: the line surface's table index)
  CK_D bool writeReferenceState(const FitParams& fp, int sid) {
    Surf<double> ts;
    ts.load(fp.surfaces + sid);
    const double z0[3] = {ts.R[2], ts.R[5], ts.R[8]};
    double d0[3] = {z0[1] * dir[2] - z0[2] * dir[1], z0[2] * dir[0] - z0[0] * dir[2],
                    z0[0] * dir[1] - z0[1] * dir[0]};
    const double dn = 1.0 / sqrt(d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2]);
#pragma unroll
    for (int i = 0; i < 3; ++i) d0[i] *= dn;
    const double dist[3] = {d0[1] * z0[2] - d0[2] * z0[1], d0[2] * z0[0] - d0[0] * z0[2],
                            d0[0] * z0[1] - d0[1] * z0[0]};
    const double pc[3] = {pos[0] - ts.c[0], pos[1] - ts.c[1], pos[2] - ts.c[2]};
    if (fabs(dist[0] * pc[0] + dist[1] * pc[1] + dist[2] * pc[2]) > fabs(kOnSurfaceTolerance))
      return false;
    // path derivative of the line surface
    const double pz = pc[0] * z0[0] + pc[1] * z0[1] + pc[2] * z0[2];
    const double dz = z0[0] * dir[0] + z0[1] * dir[1] + z0[2] * dir[2];
    const double nrm = 1.0 / (1.0 - dz * dz);
    double fpos[3], fdir[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      fpos[i] = nrm * (dz * z0[i] - dir[i]);
      fdir[i] = nrm * (pz * z0[i] - pc[i]);
    }
    const double dd[3] = {dir[0], dir[1], dir[2]};
    const Trig<double> tg = trig(dd);
    const double a0 = -tg.sinPhi * tg.invSinTheta, a1 = tg.cosPhi * tg.invSinTheta;
    const double b0 = tg.cosPhi * tg.cosTheta, b1 = tg.sinPhi * tg.cosTheta, b2 = -tg.sinTheta;
    double J[6][6];
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      // free column c of T = jacTransport * jacToGlobal
      double v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = 0.0;
      if (c < 2) {
#pragma unroll
        for (int r = 0; r < 3; ++r) v[r] = (double)T.loc[r][c];
      } else if (c < 5) {
#pragma unroll
        for (int r = 0; r < 7; ++r) v[r] = (double)T.dyn[r][c - 2];
        v[7] = c == 4 ? 1.0 : 0.0;
      } else {
        v[3] = 1.0;
      }
      const double sc = (fpos[0] * v[0] + fpos[1] * v[1] + fpos[2] * v[2]) +
                        (fdir[0] * v[4] + fdir[1] * v[5] + fdir[2] * v[6]);
#pragma unroll
      for (int r = 0; r < 7; ++r) v[r] += (double)deriv[r] * sc;
      J[0][c] = d0[0] * v[0] + d0[1] * v[1] + d0[2] * v[2];
      J[1][c] = z0[0] * v[0] + z0[1] * v[1] + z0[2] * v[2];
      J[2][c] = a0 * v[4] + a1 * v[5];
      J[3][c] = b0 * v[4] + b1 * v[5] + b2 * v[6];
      J[4][c] = v[7];
      J[5][c] = v[3];
    }
    double JC[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        double s = 0.0;
#pragma unroll
        for (int k = 0; k < 6; ++k) s += J[i][k] * (double)cov[sidx(k, j)];
        JC[i][j] = s;
      }
    const ck_batch_out& out = fp.out;
    const size_t n = (size_t)fp.n_tracks;
    if (fp.prop.jac) {
      // (the propagation entry's transport Jacobian)
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) fp.prop.jac[(size_t)(i * 6 + j) * n + t] = J[i][j];
    }
    if (out.track_cov) {
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < 6; ++k) s += JC[i][k] * J[j][k];
          out.track_cov[(size_t)(i * 6 + j) * n + t] = s;
        }
    }
    if (out.track_params) {
      const double b[6] = {d0[0] * pc[0] + d0[1] * pc[1] + d0[2] * pc[2], pz,
                           atan2(dir[1], dir[0]),
                           atan2(sqrt(dir[0] * dir[0] + dir[1] * dir[1]), dir[2]), qop, tim};
#pragma unroll
      for (int i = 0; i < 6; ++i) out.track_params[(size_t)i * n + t] = b[i];
    }
    return true;
  }

  // -------------------------------------------- propagation (ck_propagate)
  // Propagator<EigenStepper<>, VoidNavigator>::propagate(start[, target],
  // options) (Propagator.ipp:25-260): no navigation targets and no actors;
  // after every accepted step the aborters in list order — SurfaceReached on
  // the target (StandardAborters.hpp:94-155), then PathLimitReached with the
  // loop-protected limit (StandardAborters.hpp:41-61, LoopProtection.hpp:
  // 19-72). The direction is the sign of the path limit.
  CK_D void startPropagation(const FitParams& fp, int track) {
    t = track;
    q = track;
    const double limit = __ldg(&fp.prop.path_limit[t]);
    targetSurf = fp.prop.target ? __ldg(&fp.prop.target[t]) : -1;
    if (targetSurf < -1 || targetSurf >= fp.n_surfaces) {
      fail(fp, CK_TRACK_INVALID_INPUT);
      return;
    }
    dirSign = limit < 0.0 ? -1.0 : 1.0;  // Direction::fromScalar
    {
      double sp[6];
#pragma unroll
      for (int i = 0; i < 6; ++i) sp[i] = __ldg(&fp.start_params[6 * (size_t)t + i]);
      Surf<double> start;
      start.loadPlane(fp.start_frames + 12 * (size_t)t);
      boundToFree(start, sp);
      initT(start);
      if (fp.start_cov) {
        const double* sc = fp.start_cov + 36 * (size_t)t;
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = i; j < 6; ++j) cov[sidx(i, j)] = toP<CV>(__ldg(&sc[i * 6 + j]));
      } else {
#pragma unroll
        for (int i = 0; i < 21; ++i) cov[i] = CV(0);
      }
    }
#pragma unroll
    for (int i = 0; i < 7; ++i) deriv[i] = P(0);
    pathAcc = 0.0;
    cNav = kNotSet;
    cActor = kNotSet;
    cUser = fp.opt.maxStepSize;
    cAcc = fp.opt.initialStepSize;
    mass = __ldg(&fp.particle[2 * (size_t)t]);
    absQ = __ldg(&fp.particle[2 * (size_t)t + 1]);
    pdg = 211;
    coasting = false;
    finished = false;
    stepStarted = false;
    steps = 0;
    haveTarget = false;
    navigationBreak = true;
    currentSurface = -1;
    extrapolating = true;
    propLimit = loopLimit(fp, limit, false);
    phase = PH_STEP;
    if (propagationAbort(fp)) finishPropagation(fp);  // pre-propagation check
  }

  CK_D bool propagationAbort(const FitParams& fp) {
    if (targetSurf >= 0) {
      Surf<double> ts;
      ts.load(fp.surfaces + targetSurf);
      const double nd[3] = {dirSign * dir[0], dirSign * dir[1], dirSign * dir[2]};
      const double tol = fp.opt.surfaceTolerance;
      double path[2] = {0.0, 0.0};
      int st[2] = {0, 0};
      int ni = 1;
      if (ts.type == CK_SURFACE_LINE) {
        double u = 0.0;
        if (lineIntersect(ts, pos, nd, tol, u)) {
          path[0] = u;
          st[0] = fabs(u) > fabs(tol) ? 1 : 2;
        }
      } else if constexpr (sizeof(P) == sizeof(float)) {
        ni = intersectMixed(ts, pos, nd, tol, path, st);
      } else {
        ni = intersect(ts, pos, nd, tol, path, st);
      }
      // the closest intersection (Intersection::closestOrder: valid ones
      // first, then the smallest |path|) decides whether the target is
      // reached; the first valid one beyond the near limit steers the actor
      // step constraint (updateSingleSurfaceStatus)
      int best = -1;
      for (int i = 0; i < ni; ++i)
        if (st[i] != 0 && (best < 0 || fabs(path[i]) < fabs(path[best]))) best = i;
      for (int i = 0; i < ni; ++i)
        if (st[i] != 0 && path[i] > kTargetNearLimit && path[i] < kNotSet + kOnSurfaceTolerance) {
          cActor = kNotSet;
          cupdate(cActor, path[i]);
          break;
        }
      if (best >= 0 && st[best] == 2) return true;
    }
    return pathLimitReached(fp, propLimit);
  }

  // Propagator::makeResult: the bound state on the target (CovarianceEngine
  // boundState) or the curvilinear state at the end point (curvilinearState,
  // the plane through the end point with the curvilinear unit vectors)
  CK_D void finishPropagation(const FitParams& fp) {
    const size_t n = (size_t)fp.n_tracks;
    Surf<double> sf;
    bool curvilinear = false;
    if (targetSurf >= 0) {
      sf.load(fp.surfaces + targetSurf);
      if (sf.type == CK_SURFACE_LINE) {
        if (!writeReferenceState(fp, targetSurf)) {
          fail(fp, CK_TRACK_NOT_ON_SURFACE);
          return;
        }
        endPropagationOutputs(fp);
        return;
      }
    } else {
      // createCurvilinearUnitVectors (UnitVectors.hpp:94-150)
      double u[3] = {-dir[1], dir[0], 0.0};
      const double sc = sqrt(u[0] * u[0] + u[1] * u[1]);
      if (sc < 16.0 * 2.220446049250313e-16) {  // 16 epsilon
        u[0] = 1.0;
        u[1] = 0.0;
      } else {
        u[0] /= sc;
        u[1] /= sc;
      }
      double v[3] = {dir[1] * u[2] - dir[2] * u[1], dir[2] * u[0] - dir[0] * u[2],
                     dir[0] * u[1] - dir[1] * u[0]};
      const double vn = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        v[i] *= vn;
        sf.R[i * 3 + 0] = u[i];
        sf.R[i * 3 + 1] = v[i];
        sf.R[i * 3 + 2] = dir[i];
        sf.c[i] = pos[i];
      }
      sf.radius = 0.0;
      sf.type = CK_SURFACE_PLANE;
      curvilinear = true;
    }
    double l[3];
    local(sf, l);
    double b[6];
    if (!freeToBound(fp, sf, l, b)) {
      fail(fp, CK_TRACK_NOT_ON_SURFACE);
      return;
    }
    if (curvilinear) b[0] = b[1] = 0.0;  // BoundTrackParameters::createCurvilinear
    Surf<P> sp;
#pragma unroll
    for (int i = 0; i < 9; ++i) sp.R[i] = (P)sf.R[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) sp.c[i] = (P)sf.c[i];
    sp.radius = (P)sf.radius;
    sp.type = sf.type;
    CV J[36];
    transportToBound(sf, sp, l, J, false);
    const ck_batch_out& out = fp.out;
    if (out.track_params) {
#pragma unroll
      for (int i = 0; i < 6; ++i) out.track_params[(size_t)i * n + t] = b[i];
    }
    if (out.track_cov) {
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) out.track_cov[(size_t)(i * 6 + j) * n + t] = (double)cov[sidx(i, j)];
    }
    if (fp.prop.jac) {
#pragma unroll
      for (int i = 0; i < 36; ++i) fp.prop.jac[(size_t)i * n + t] = (double)J[i];
    }
    if (curvilinear && fp.prop.frames) {
      double* fr = fp.prop.frames + 12 * (size_t)t;
#pragma unroll
      for (int i = 0; i < 9; ++i) fr[i] = sf.R[i];
#pragma unroll
      for (int i = 0; i < 3; ++i) fr[9 + i] = sf.c[i];
    }
    endPropagationOutputs(fp);
  }

  CK_D void endPropagationOutputs(const FitParams& fp) {
    if (fp.prop.path) fp.prop.path[t] = pathAcc;
    if (fp.prop.steps) fp.prop.steps[t] = (int32_t)steps;
    fp.out.status[t] = CK_TRACK_OK;
    phase = PH_DONE;
  }

  // SURFACE: the actor on the reached surface
  CK_D void surface(const FitParams& fp, int slot) {
    const int e = act(fp, slot);
    if (e != CK_TRACK_OK) {
      fail(fp, e);
      return;
    }
    afterAct(fp, slot);
  }

  // end of propagation: NoMeasurementFound, or the track's tip is handed to
  // the smoother kernel. The reversed pass instead checks that its last
  // measurement state lies on the forward pass's first one's surface
  // (KalmanFitter.hpp:920-932); the output kernel then takes the track.
  CK_D void endPropagation(const FitParams& fp, int slot) {
    if (measurementStates == 0) {
      fail(fp, CK_TRACK_NO_MEASUREMENT_FOUND);
      return;
    }
    if constexpr (REV) {
      const Rec<CV> rec(fp, slot);
      const int tip = fp.tip[slot];
      int firstSurf = -1;
      for (int k = 0; k <= tip && firstSurf < 0; ++k) {
        const uint32_t fl = (uint32_t)rec.s(k).flags;
        if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) firstSurf = rec.s(k).surface;
      }
      if (fp.ext[2 * (size_t)slot].surface != firstSurf) {
        fail(fp, CK_TRACK_INCONSISTENT_STATES);
        return;
      }
    } else {
      // (with smoothing in the tail the tip publishes the track: its records
      // are ordered before it for the blocks that read them)
      if (fp.smoothed) __threadfence();
      *(volatile int32_t*)&fp.tip[slot] = lastMeasurementIndex;
    }
    phase = PH_FETCH;
  }
};

// RTS smoother of one track over its records (GainMatrixSmoother, driven as
// in KalmanFitter::finalize, KalmanFitter.hpp:795-984), then the track
// summary (calculateTrackQuantities, TrackHelpers.hpp:421-448).
template <typename CV>
struct Smoother {
  int t, q;
  int lastMeas, firstMeas;
  int nM, nH, nO, ndf;
  double chi2sum;

  // the per-track set-up of run(): the first and last measurement states, the
  // extrapolation start slots, zero counters (the staged kernel's entry)
  CK_D void begin(const FitParams& fp, int queuePos, int track, int tip) {
    t = track;
    q = queuePos;
    lastMeas = tip;
    firstMeas = -1;
    const Rec<CV> rec(fp, q);
    if (fp.ext) {
      fp.ext[2 * (size_t)q].surface = -1;
      fp.ext[2 * (size_t)q].fitted = 0;
      fp.ext[2 * (size_t)q + 1].surface = -1;
      for (int k = 0; k <= tip; ++k) {
        const uint32_t fl = (uint32_t)rec.s(k).flags;
        if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
          firstMeas = k;
          break;
        }
      }
    }
    for (int k = tip; k >= 0; --k) {
      const uint32_t fl = (uint32_t)rec.s(k).flags;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
        lastMeas = k;
        break;
      }
    }
    nM = nH = nO = ndf = 0;
    chi2sum = 0.0;
  }

  CK_D void run(const FitParams& fp, int queuePos, int track, int tip) {
    t = track;
    q = queuePos;
    lastMeas = tip;
    firstMeas = -1;
    const Rec<CV> rec(fp, q);
    if (fp.ext) {
      // the extrapolation's candidate start states: the first and the last
      // state with a non-outlier measurement (findFirst/LastMeasurementState,
      // TrackHelpers.hpp:64-102); none yet
      fp.ext[2 * (size_t)q].surface = -1;
      fp.ext[2 * (size_t)q].fitted = 0;
      fp.ext[2 * (size_t)q + 1].surface = -1;
      for (int k = 0; k <= tip; ++k) {
        const uint32_t fl = (uint32_t)rec.s(k).flags;
        if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
          firstMeas = k;
          break;
        }
      }
    }
    for (int k = tip; k >= 0; --k) {
      const uint32_t fl = (uint32_t)rec.s(k).flags;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
        lastMeas = k;
        break;
      }
    }
    nM = nH = nO = ndf = 0;
    chi2sum = 0.0;
    if (fp.opt.smoother == CK_SMOOTHER_MBF) {
      runMbf(fp, rec, tip);
      finish(fp, tip);
      return;
    }
    // the smoothed state of k+1, carried from one step to the next (the tip's
    // smoothed state is its filtered state)
    double ps[6];
    CV Psp[21];
#pragma unroll
    for (int i = 0; i < 6; ++i) ps[i] = rec.p(tip, kRecFilt + i);
#pragma unroll
    for (int i = 0; i < 21; ++i) Psp[i] = rec.m(tip, kRecFiltCov + i);
    writeState(fp, tip, ps, Psp, false);
    for (int k = tip - 1; k >= 0; --k) {
      double filt[6], pp[6], sm[6];
      CV Pf[21], Ppp[21], J[36], Ps[21];
#pragma unroll
      for (int i = 0; i < 6; ++i) filt[i] = rec.p(k, kRecFilt + i);
#pragma unroll
      for (int i = 0; i < 21; ++i) Pf[i] = rec.m(k, kRecFiltCov + i);
#pragma unroll
      for (int i = 0; i < 6; ++i) pp[i] = rec.p(k + 1, kRecPred + i);
#pragma unroll
      for (int i = 0; i < 21; ++i) Ppp[i] = rec.m(k + 1, kRecPredCov + i);
#pragma unroll
      for (int i = 0; i < 36; ++i) J[i] = rec.m(k + 1, kRecJac + i);
      if (!smoothStep<CV>(filt, Pf, pp, Ppp, J, ps, Psp, sm, Ps)) {
        failSmooth(fp);
        return;
      }
      writeState(fp, k, sm, Ps, k == lastMeas);
#pragma unroll
      for (int i = 0; i < 6; ++i) ps[i] = sm[i];
#pragma unroll
      for (int i = 0; i < 21; ++i) Psp[i] = Ps[i];
    }
    finish(fp, tip);
  }

  // MbfSmoother::operator() (MbfSmoother.hpp:48-90): backwards from the tip
  // with zero lambdas; each state is smoothed from its filtered state and the
  // lambdas of the states after it, then the lambdas move to the previous
  // state through its measurement (a non-outlier measurement state) and its
  // Jacobian. The first state updates no lambdas.
  CK_D void runMbf(const FitParams& fp, const Rec<CV>& rec, int tip) {
    const int m0 = __ldg(&fp.meas_off[t]);
    const int nMeas = __ldg(&fp.meas_off[t + 1]) - m0;
    CV L[21], l[6];
#pragma unroll
    for (int i = 0; i < 21; ++i) L[i] = CV(0);
#pragma unroll
    for (int i = 0; i < 6; ++i) l[i] = CV(0);
    for (int k = tip; k >= 0; --k) {
      double filt[6], sm[6];
      CV Pf[21], Ps[21];
#pragma unroll
      for (int i = 0; i < 6; ++i) filt[i] = rec.p(k, kRecFilt + i);
#pragma unroll
      for (int i = 0; i < 21; ++i) Pf[i] = rec.m(k, kRecFiltCov + i);
      mbfSmoothed<CV>(filt, Pf, L, l, k == lastMeas, sm, Ps);
      writeState(fp, k, sm, Ps, k == lastMeas);
      if (k == 0) break;
      const RecState<CV>& rs = rec.s(k);
      const uint32_t fl = (uint32_t)rs.flags;
      // the source link of a measurement state: the first measurement on its
      // surface (the one the forward filter used)
      int mi = -1;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
        for (int i = 0; i < nMeas && mi < 0; ++i)
          if (__ldg(&fp.meas_surf[m0 + i]) == rs.surface) mi = m0 + i;
      }
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER) && mi >= 0) {
        double pred[6], V[4];
        CV Pp[21];
#pragma unroll
        for (int i = 0; i < 6; ++i) pred[i] = rec.p(k, kRecPred + i);
#pragma unroll
        for (int i = 0; i < 21; ++i) Pp[i] = rec.m(k, kRecPredCov + i);
#pragma unroll
        for (int i = 0; i < 4; ++i) V[i] = __ldg(&fp.meas_cov[4 * (size_t)mi + i]);
        const int sub = ((uint32_t)rs.flags >> kRecSubShift) & 3u;
        if (sub == CK_MEAS_LOC01)
          mbfMeasurement<CV>(pred, Pp, __ldg(&fp.meas_val[2 * (size_t)mi]),
                             __ldg(&fp.meas_val[2 * (size_t)mi + 1]), V, L, l);
        else
          mbfMeasurement1<CV>(pred, Pp, sub >> 1, __ldg(&fp.meas_val[2 * (size_t)mi]), V[0], L, l);
      }
      CV F[36];
#pragma unroll
      for (int i = 0; i < 36; ++i) F[i] = rec.m(k, kRecJac + i);
      mbfTransport<CV>(F, L, l);
    }
  }

  // The output of a reverse-filtered track (KalmanFitter.hpp:889-945): every
  // state's predicted and filtered parameters and Jacobian as the forward
  // pass recorded them; smoothed parameters only on the last measurement
  // state (its filtered ones, shared) and on the first (the reversed pass's
  // last filtered state, extrapolation slot 0, which wins when the two are
  // one state); every other state's smoothed parameters are NaN.
  CK_D void runReverse(const FitParams& fp, int queuePos, int track, int tip) {
    t = track;
    q = queuePos;
    const Rec<CV> rec(fp, q);
    firstMeas = -1;
    lastMeas = tip;
    for (int k = 0; k <= tip && firstMeas < 0; ++k) {
      const uint32_t fl = (uint32_t)rec.s(k).flags;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) firstMeas = k;
    }
    for (int k = tip; k >= 0; --k) {
      const uint32_t fl = (uint32_t)rec.s(k).flags;
      if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
        lastMeas = k;
        break;
      }
    }
    fp.ext[2 * (size_t)q + 1].surface = -1;
    nM = nH = nO = ndf = 0;
    chi2sum = 0.0;
    const ExtStart& rv = fp.ext[2 * (size_t)q];
    for (int k = 0; k <= tip; ++k) {
      double sm[6];
      CV Ps[21];
      if (k == firstMeas) {
#pragma unroll
        for (int i = 0; i < 6; ++i) sm[i] = rv.par[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) Ps[i] = (CV)rv.cov[i];
      } else if (k == lastMeas) {
#pragma unroll
        for (int i = 0; i < 6; ++i) sm[i] = rec.p(k, kRecFilt + i);
#pragma unroll
        for (int i = 0; i < 21; ++i) Ps[i] = rec.m(k, kRecFiltCov + i);
      } else {
#pragma unroll
        for (int i = 0; i < 6; ++i) sm[i] = CUDART_NAN;
#pragma unroll
        for (int i = 0; i < 21; ++i) Ps[i] = (CV)CUDART_NAN;
      }
      writeState(fp, k, sm, Ps, false);
    }
    finish(fp, tip);
  }

  // status and calculateTrackQuantities (TrackHelpers.hpp:421-448)
  CK_D void finish(const FitParams& fp, int tip) {
    const ck_batch_out& out = fp.out;
    out.status[t] = CK_TRACK_OK;
    if (out.n_states) out.n_states[t] = tip + 1;
    if (out.n_measurements) out.n_measurements[t] = nM;
    if (out.n_holes) out.n_holes[t] = nH;
    if (out.n_outliers) out.n_outliers[t] = nO;
    if (out.ndf) out.ndf[t] = ndf;
    if (out.chi2_sum) out.chi2_sum[t] = chi2sum;
  }

  CK_D void failSmooth(const FitParams& fp) {
    const ck_batch_out& out = fp.out;
    out.status[t] = CK_TRACK_SMOOTH_FAILED;
    if (out.n_states) out.n_states[t] = 0;
    if (out.n_measurements) out.n_measurements[t] = 0;
    if (out.n_holes) out.n_holes[t] = 0;
    if (out.n_outliers) out.n_outliers[t] = 0;
    if (out.ndf) out.ndf[t] = 0;
    if (out.chi2_sum) out.chi2_sum[t] = 0.0;
  }

  CK_D void writeState(const FitParams& fp, int k, const double sm[6], const CV Ps[21],
                       bool filtOverride) {
    writeStateRec(fp, k, Rec<CV>(fp, q).s(k), sm, Ps, filtOverride);
  }

  // the outputs of state k from its record `rs` (in global memory, or staged)
  CK_D void writeStateRec(const FitParams& fp, int k, const RecState<CV>& rs, const double sm[6],
                          const CV Ps[21], bool filtOverride) {
    const ck_batch_out& out = fp.out;
    if (fp.ext && (k == firstMeas || k == lastMeas)) {
      // its smoothed parameters (TrackStateProxy::parameters) for the
      // extrapolation; slot 0 first, slot 1 last
      for (int slot = 0; slot < 2; ++slot) {
        if (k != (slot == 0 ? firstMeas : lastMeas)) continue;
        ExtStart& es = fp.ext[2 * (size_t)q + slot];
#pragma unroll
        for (int i = 0; i < 6; ++i) es.par[i] = sm[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) es.cov[i] = (double)Ps[i];
        es.surface = rs.surface;
      }
    }
    const size_t n = (size_t)fp.n_tracks;
    auto at = [&](int C, int c) -> size_t { return ((size_t)k * C + c) * n + t; };
    const uint32_t fl = (uint32_t)rs.flags & kRecFlagMask;
    const int sub = ((uint32_t)rs.flags >> kRecSubShift) & 3u;
    const double c2 = rs.chi2;
    if (out.state_surface) out.state_surface[at(1, 0)] = rs.surface;
    if (out.state_flags) out.state_flags[at(1, 0)] = fl;
    if (out.state_path_length)
      out.state_path_length[at(1, 0)] = rs.pathLength;
    if (out.state_chi2) out.state_chi2[at(1, 0)] = c2;
    if (fl & CK_FLAG_IS_HOLE) {
      ++nH;
    } else if (fl & CK_FLAG_IS_OUTLIER) {
      ++nO;
    } else if (fl & CK_FLAG_HAS_MEASUREMENT) {
      ++nM;
      chi2sum += c2;
      ndf += (sub & 1) + (sub >> 1);
    }
    // CK_OUT_PACKED_COV: the upper triangle (21) instead of the full matrix
    const bool packed = (out.components & CK_OUT_PACKED_COV) != 0;
    if (out.smoothed) {
#pragma unroll
      for (int i = 0; i < 6; ++i) out.smoothed[at(6, i)] = sm[i];
      if (packed) {
#pragma unroll
        for (int i = 0; i < 21; ++i) out.smoothed_cov[at(21, i)] = toDi(Ps[i]);
      } else {
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = i; j < 6; ++j) {
            const double v = toDi(Ps[sidx(i, j)]);
            out.smoothed_cov[at(36, i * 6 + j)] = v;
            if (j != i) out.smoothed_cov[at(36, j * 6 + i)] = v;
          }
      }
    }
    if (out.filtered) {
#pragma unroll
      for (int i = 0; i < 6; ++i)
        out.filtered[at(6, i)] = filtOverride ? sm[i] : rs.par[kRecFilt + i];
      if (packed) {
#pragma unroll
        for (int i = 0; i < 21; ++i)
          out.filtered_cov[at(21, i)] = (double)(filtOverride ? Ps[i] : rs.mat[kRecFiltCov + i]);
      } else {
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = 0; j < 6; ++j)
            out.filtered_cov[at(36, i * 6 + j)] =
                (double)(filtOverride ? Ps[sidx(i, j)] : rs.mat[kRecFiltCov + sidx(i, j)]);
      }
    }
    if (out.predicted) {
#pragma unroll
      for (int i = 0; i < 6; ++i) out.predicted[at(6, i)] = rs.par[kRecPred + i];
      if (packed) {
#pragma unroll
        for (int i = 0; i < 21; ++i) out.predicted_cov[at(21, i)] = (double)rs.mat[kRecPredCov + i];
      } else {
#pragma unroll
        for (int i = 0; i < 6; ++i)
#pragma unroll
          for (int j = 0; j < 6; ++j)
            out.predicted_cov[at(36, i * 6 + j)] = (double)rs.mat[kRecPredCov + sidx(i, j)];
      }
    }
    if (out.jacobian) {
#pragma unroll
      for (int i = 0; i < 36; ++i) out.jacobian[at(36, i)] = (double)rs.mat[kRecJac + i];
    }
  }
};

// Persistent forward-filter kernel with warp-level phase scheduling: each
// warp votes the phase most of its lanes are in (fetch a track, one
// Runge-Kutta trial, the actor on a reached surface) and runs it for those
// lanes; fetching lanes take consecutive queue positions with one atomic per
// warp. Records are indexed by queue position.
template <typename P, typename CV, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) fitKernel(FitParams fp) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  Lane<P, CV> L;
  L.phase = lane < fp.lanes_per_warp ? PH_FETCH : PH_DONE;
  L.t = -1;
  L.q = -1;
  while (true) {
    const unsigned mFetch = __ballot_sync(FULL, L.phase == PH_FETCH);
    const unsigned mStep = __ballot_sync(FULL, L.phase == PH_STEP);
    const unsigned mSurf = __ballot_sync(FULL, L.phase == PH_SURFACE);
    if ((mFetch | mStep | mSurf) == 0u) break;
    int best = PH_FETCH, bc = __popc(mFetch);
    if (__popc(mStep) > bc) {
      best = PH_STEP;
      bc = __popc(mStep);
    }
    if (__popc(mSurf) > bc) best = PH_SURFACE;
    if (best == PH_FETCH) {
      // warp-aggregated ticket for every fetching lane
      const int leader = __ffs(mFetch) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(fp.ticket, __popc(mFetch));
      base = __shfl_sync(FULL, base, leader);
      if (L.phase == PH_FETCH) {
        const int q = base + __popc(mFetch & ((1u << lane) - 1u));
        if (q >= fp.n_queue) {
          L.phase = PH_DONE;
        } else {
          L.q = q;
          L.start(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q);
        }
      }
    } else if (L.phase == best) {
      if (best == PH_STEP)
        L.step(fp, L.q);
      else
        L.surface(fp, L.q);
    }
  }
}

// Persistent forward-filter kernel with block-level phase compaction. The
// state of every track in flight lives in shared memory (one Lane per slot,
// S slots per block). Each round the block counts its slots per phase, picks
// the phase most slots are in, lists those slots contiguously and lets
// thread i advance slot list[i] by one phase step — so the chosen phase runs
// on full warps. On GB300 an FP64 warp instruction holds the SM's FP64 unit
// for 16 clocks however few of its lanes are active, so the lanes a warp
// carries are the FP64 throughput it gets.
// One phase step of a slot; fetching threads take one ticket per warp (the
// threads of the warp that run this call together).
template <typename P, typename CV, bool F2B, bool REV>
__device__ __forceinline__ void advanceSlot(const FitParams& fp, Lane<P, CV, F2B, REV>& L,
                                            int c, int lane, int spr) {
  if (c == PH_FETCH) {
    const unsigned act = __activemask();
    const int leader = __ffs(act) - 1;
    int qb = 0;
    if (lane == leader) qb = atomicAdd(fp.ticket, __popc(act));
    qb = __shfl_sync(act, qb, leader);
    const int q = qb + __popc(act & ((1u << lane) - 1u));
    if (q >= fp.n_queue) {
      L.phase = PH_DONE;
    } else {
      L.q = q;
      if constexpr (REV)
        L.startReverse(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q);
      else
        L.start(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q);
    }
  } else if (c == PH_STEP) {
    // up to spr Runge-Kutta trials while the track stays in STEP
    for (int k = 0; k < spr && L.phase == PH_STEP; ++k) L.step(fp, L.q);
  } else {
    L.surface(fp, L.q);
  }
}

// Smoothing in the forward filter's tail, by a warp whose block has no
// forward work left: claims 32 queue positions at a time, in queue order,
// and smooths those whose forward pass has ended successfully (tip >= 0,
// published after the track's records); positions still in flight, or
// failed, are left to the smoother kernel. Nothing waits: each position is
// claimed once, and the smoother kernel, launched after this kernel, takes
// every successful track not marked smoothed.
template <typename CV>
__device__ __noinline__ void smoothInTail(const FitParams& fp) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  while (true) {
    int base = 0;
    if (lane == 0) base = atomicAdd(fp.smooth_ticket, 32);
    base = __shfl_sync(FULL, base, 0);
    if (base >= fp.n_queue) return;
    const int q = base + lane;
    const int tip = q < fp.n_queue ? *(const volatile int32_t*)&fp.tip[q] : -1;
    if (tip >= 0) {
      __threadfence();  // (the records, after the tip that published them)
      Smoother<CV> S;
      S.run(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q, tip);
      fp.smoothed[q] = 1;
    }
  }
}

template <typename P, typename CV, int S, bool F2B = false, bool REV = false>
__global__ void __launch_bounds__(S, 1) fitKernelCompact(FitParams fp) {
  extern __shared__ __align__(16) unsigned char smem[];
  using LaneT = Lane<P, CV, F2B, REV>;
  LaneT* st = reinterpret_cast<LaneT*>(smem);
  int* items = reinterpret_cast<int*>(smem + sizeof(LaneT) * S);
  __shared__ int warpCnt[S / 32][3];
  __shared__ int chosen, nItems;
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  st[tid].phase = tid < fp.lanes_per_warp * (S / 32) ? PH_FETCH : PH_DONE;
  st[tid].t = -1;
  st[tid].q = -1;
  __syncthreads();
  while (true) {
    const int ph = st[tid].phase;
    const unsigned mF = __ballot_sync(FULL, ph == PH_FETCH);
    const unsigned mS = __ballot_sync(FULL, ph == PH_STEP);
    const unsigned mU = __ballot_sync(FULL, ph == PH_SURFACE);
    if (lane == 0) {
      warpCnt[warp][0] = __popc(mF);
      warpCnt[warp][1] = __popc(mS);
      warpCnt[warp][2] = __popc(mU);
    }
    __syncthreads();
    if (tid == 0) {
      int tot[3] = {0, 0, 0};
      for (int w = 0; w < S / 32; ++w)
        for (int k = 0; k < 3; ++k) tot[k] += warpCnt[w][k];
      int best = PH_FETCH, bc = tot[0];
      if (tot[1] > bc) {
        best = PH_STEP;
        bc = tot[1];
      }
      if (tot[2] > bc) {
        best = PH_SURFACE;
        bc = tot[2];
      }
      chosen = bc > 0 ? best : -1;
      nItems = bc;
    }
    __syncthreads();
    const int c = chosen;
    if (c < 0) break;
    const unsigned m = c == PH_FETCH ? mF : (c == PH_STEP ? mS : mU);
    int base = 0;
    for (int w = 0; w < warp; ++w) base += warpCnt[w][c];
    if (ph == c) items[base + __popc(m & ((1u << lane) - 1u))] = tid;
    __syncthreads();
    if (tid < nItems) {
      const int slot = items[tid];
      // At most half of the block's slots stepping (small batches, and the
      // end of the queue, where a track running into the step limit would
      // otherwise take a round of the block's phase vote per few trials):
      // many trials per round. Measured on GB300 (mixed, 256 slots): 10k
      // uneven tracks 3.44 -> 2.52 ms against a one-warp threshold, 1M barrel
      // tracks unchanged. Results do not depend on the trials per round.
      const int spr = nItems <= S / 2 ? max(fp.steps_per_round, kTailStepsPerRound)
                                      : fp.steps_per_round;
      // the phase step works on a register copy of the slot's state
      LaneT L = st[slot];
      advanceSlot(fp, L, c, lane, spr);
      st[slot] = L;
    }
    __syncthreads();
  }
  if constexpr (!REV) {
    if (fp.smoothed) smoothInTail<CV>(fp);
  }
}

template <typename P, typename CV, int S>
constexpr size_t compactSmemBytes() {
  return sizeof(Lane<P, CV>) * S + sizeof(int) * S;
}

// Persistent forward-filter kernel with warp-autonomous phase pools. The
// state of every track in flight lives in shared memory (one Lane per slot,
// S slots, more slots than the T threads of the block). A slot waiting for
// a phase step sits in that phase's pool, a bit mask in shared memory. Each
// warp on its own, without block barriers: counts the pools, claims up to 32
// slots of the fullest one (atomicAnd on the mask words), advances them by
// one phase step on its lanes, and returns each slot to the pool of its new
// phase (atomicOr), or retires it when the work queue is empty. With S > T
// the pools hold S - T slots or more while every warp is busy, so a warp
// finds full sets of one phase; no warp waits for the slowest item of a
// block-wide round. A warp leaves when all pools are empty: slots still in
// flight belong to warps that are running and that claim them again after
// returning them, so every slot is finished, and nothing spins.
template <typename P, typename CV, int S, int T>
__global__ void __launch_bounds__(T, 1) fitKernelPool(FitParams fp) {
  static_assert(S % 32 == 0 && S / 32 <= 32 && T % 32 == 0, "pool shape");
  constexpr int W = S / 32;  // mask words per phase
  extern __shared__ __align__(16) unsigned char smem[];
  using LaneT = Lane<P, CV>;
  LaneT* st = reinterpret_cast<LaneT*>(smem);
  __shared__ unsigned pool[3][W];
  __shared__ int items[T / 32][32];
  const unsigned FULL = 0xffffffffu;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // slots that take tracks: all of them for large batches; a small batch
  // spreads over all blocks
  const int perBlock = (fp.n_queue + (int)gridDim.x - 1) / (int)gridDim.x;
  const int active = min(S, max(1, perBlock));
  for (int sl = tid; sl < S; sl += T) {
    st[sl].phase = sl < active ? PH_FETCH : PH_DONE;
    st[sl].t = -1;
    st[sl].q = -1;
  }
  if (tid < W) {
    const int lo = tid * 32;
    const int k = min(32, max(0, active - lo));
    pool[PH_FETCH][tid] = k == 32 ? FULL : ((1u << k) - 1u);
    pool[PH_STEP][tid] = 0u;
    pool[PH_SURFACE][tid] = 0u;
  }
  __syncthreads();
  volatile unsigned* vpool = &pool[0][0];
  while (true) {
    // pool sizes (lane w < W reads word w of every pool)
    unsigned w0 = 0u, w1 = 0u, w2 = 0u;
    if (lane < W) {
      w0 = vpool[PH_FETCH * W + lane];
      w1 = vpool[PH_STEP * W + lane];
      w2 = vpool[PH_SURFACE * W + lane];
    }
    const int n0 = __reduce_add_sync(FULL, __popc(w0));
    const int n1 = __reduce_add_sync(FULL, __popc(w1));
    const int n2 = __reduce_add_sync(FULL, __popc(w2));
    int c = -1, best = 0;
    if (n1 > best) {
      c = PH_STEP;
      best = n1;
    }
    if (n2 > best) {
      c = PH_SURFACE;
      best = n2;
    }
    if (n0 > best) {
      c = PH_FETCH;
      best = n0;
    }
    if (c < 0) break;  // every pool empty
    // claim up to 32 slots of pool c: word w gives at most what the words
    // before it left of 32
    const unsigned word = c == PH_FETCH ? w0 : (c == PH_STEP ? w1 : w2);
    const int cnt = __popc(word);
    int before = cnt;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(FULL, before, d);
      if (lane >= d) before += v;
    }
    before -= cnt;  // exclusive prefix
    const int want = max(0, min(cnt, 32 - before));
    unsigned take = 0u, rest = word;
    for (int i = 0; i < want; ++i) {
      const unsigned b = rest & (0u - rest);
      take |= b;
      rest ^= b;
    }
    unsigned got = 0u;
    if (take) got = atomicAnd(&pool[c][lane], ~take) & take;
    const int gc = __popc(got);
    int base = gc;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(FULL, base, d);
      if (lane >= d) base += v;
    }
    const int total = __shfl_sync(FULL, base, 31);
    base -= gc;
    for (unsigned g = got; g; g &= g - 1u) items[warp][base++] = lane * 32 + (__ffs(g) - 1);
    __syncwarp();
    if (total == 0) continue;  // another warp took them first
    __threadfence_block();     // (acquire: the claimed slots' states)
    if (lane < total) {
      const int slot = items[warp][lane];
      // few items: many Runge-Kutta trials per claim (the end of the queue,
      // small batches); results do not depend on the trials per claim
      const int spr = total <= 16 ? max(fp.steps_per_round, kTailStepsPerRound)
                                  : fp.steps_per_round;
      LaneT L = st[slot];
      advanceSlot(fp, L, c, lane, spr);
      st[slot] = L;
      __threadfence_block();  // (release: the state before the slot is published)
      if (L.phase != PH_DONE) atomicOr(&pool[L.phase][slot >> 5], 1u << (slot & 31));
    }
    __syncwarp();
  }
}

template <typename P, typename CV, int S>
constexpr size_t poolSmemBytes() {
  return sizeof(Lane<P, CV>) * S;
}

// Smoother kernel: one lane per queue position; lanes of a warp hold tracks
// of similar length (the queue is ordered by sequence length).
// Output kernel of reverse filtering, after the reversed pass: one lane per
// queue position, for the tracks both passes fitted.
template <typename CV, int BLOCK>
__global__ void __launch_bounds__(BLOCK) reverseOutputKernel(FitParams fp) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < fp.n_queue;
       q += gridDim.x * blockDim.x) {
    const int tip = fp.tip[q];
    if (tip < 0 || !reverseSelected<CV>(fp, q, tip)) continue;
    Smoother<CV> S;
    S.runReverse(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q, tip);
  }
}

// Smoother kernel with warp-cooperative record staging: one lane per queue
// position as in smoothKernel, but the state records are read coalesced.
// Iteration j of a warp smooths state k = tip - j of every lane's track: the
// 32 records (one per lane, 432 / 744 B each, contiguous) are copied into
// shared memory by the whole warp in 16 / 8 B chunks, consecutive lanes
// reading consecutive chunks, so every DRAM sector of a record is fetched
// once; the previous iteration's records (state k + 1) stay staged in the
// second buffer. Only the RTS gain-matrix smoother takes this path.
template <typename CV, int BLOCK>
__global__ void __launch_bounds__(BLOCK) smoothKernelStaged(FitParams fp) {
  using R = RecState<CV>;
  using Chunk = typename std::conditional<sizeof(R) % 16 == 0, uint4, uint2>::type;
  constexpr int NCH = (int)(sizeof(R) / sizeof(Chunk));
  static_assert(sizeof(R) % sizeof(Chunk) == 0, "record chunks");
  extern __shared__ __align__(16) unsigned char smem[];
  R* buf = reinterpret_cast<R*>(smem);  // [2][BLOCK]
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
  const R* recs = static_cast<const R*>(fp.rec);
  const int ms = fp.max_states;
  for (int q0 = blockIdx.x * BLOCK; q0 < fp.n_queue; q0 += gridDim.x * BLOCK) {
    const int q = q0 + threadIdx.x;
    int tip = q < fp.n_queue ? fp.tip[q] : -1;
    if (tip >= 0 && fp.smoothed && fp.smoothed[q]) tip = -1;  // smoothed in the filter's tail
    // (tracks the reverse-filtering logic selects take the reversed pass)
    if (tip >= 0 && fp.opt.reverseMomThreshold > 0.0 && reverseSelected<CV>(fp, q, tip)) tip = -1;
    const int iters = __reduce_max_sync(FULL, tip + 1);
    Smoother<CV> S;
    double ps[6];
    CV Psp[21];
    bool ok = tip >= 0;
    if (ok) S.begin(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q, tip);
    for (int j = 0; j < iters; ++j) {
      // stage state k = tip - j of every lane with such a state
      const int myK = ok && tip - j >= 0 ? tip - j : -1;
      R* cur = buf + (size_t)(j & 1) * BLOCK;
      R* prev = buf + (size_t)((j + 1) & 1) * BLOCK;
      __syncwarp();
      for (int i = lane; i < 32 * NCH; i += 32) {
        const int L = i / NCH, c = i - L * NCH;
        const int kL = __shfl_sync(FULL, myK, L);  // (every lane takes part)
        const int qL = q0 + wbase + L;
        if (kL >= 0) {
          const Chunk* src = reinterpret_cast<const Chunk*>(recs + (size_t)qL * ms + kL);
          reinterpret_cast<Chunk*>(cur + wbase + L)[c] = src[c];
        }
      }
      __syncwarp();
      if (myK < 0) continue;
      const R& rk = cur[threadIdx.x];
      if (j == 0) {
        // the tip's smoothed state is its filtered state
#pragma unroll
        for (int i = 0; i < 6; ++i) ps[i] = rk.par[kRecFilt + i];
#pragma unroll
        for (int i = 0; i < 21; ++i) Psp[i] = rk.mat[kRecFiltCov + i];
        S.writeStateRec(fp, myK, rk, ps, Psp, false);
        if (myK == 0) S.finish(fp, tip);
        continue;
      }
      const R& rn = prev[threadIdx.x];  // state k + 1
      double filt[6], pp[6], sm[6];
      CV Pf[21], Ppp[21], J[36], Ps[21];
#pragma unroll
      for (int i = 0; i < 6; ++i) filt[i] = rk.par[kRecFilt + i];
#pragma unroll
      for (int i = 0; i < 21; ++i) Pf[i] = rk.mat[kRecFiltCov + i];
#pragma unroll
      for (int i = 0; i < 6; ++i) pp[i] = rn.par[kRecPred + i];
#pragma unroll
      for (int i = 0; i < 21; ++i) Ppp[i] = rn.mat[kRecPredCov + i];
#pragma unroll
      for (int i = 0; i < 36; ++i) J[i] = rn.mat[kRecJac + i];
      if (!smoothStep<CV>(filt, Pf, pp, Ppp, J, ps, Psp, sm, Ps)) {
        S.failSmooth(fp);
        ok = false;
        continue;
      }
      S.writeStateRec(fp, myK, rk, sm, Ps, myK == S.lastMeas);
#pragma unroll
      for (int i = 0; i < 6; ++i) ps[i] = sm[i];
#pragma unroll
      for (int i = 0; i < 21; ++i) Psp[i] = Ps[i];
      if (myK == 0) S.finish(fp, tip);
    }
    __syncwarp();
  }
}

template <typename CV, int BLOCK>
constexpr size_t stagedSmoothSmemBytes() {
  return 2 * sizeof(RecState<CV>) * BLOCK;
}

template <typename CV, int BLOCK>
__global__ void __launch_bounds__(BLOCK) smoothKernel(FitParams fp) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < fp.n_queue;
       q += gridDim.x * blockDim.x) {
    const int tip = fp.tip[q];
    if (tip < 0) continue;
    if (fp.smoothed && fp.smoothed[q]) continue;  // smoothed in the filter's tail
    // (tracks the reverse-filtering logic selects take the reversed pass)
    if (fp.opt.reverseMomThreshold > 0.0 && reverseSelected<CV>(fp, q, tip)) continue;
    Smoother<CV> S;
    S.run(fp, q, fp.perm ? __ldg(&fp.perm[q]) : q, tip);
  }
}

}  // namespace ck
