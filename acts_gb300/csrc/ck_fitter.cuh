// ck_fitter.cuh — the per-track Kalman fit and the persistent fit kernel.
//
// fitTrack() is the device restatement of
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
// One thread fits one track; warps pull 32 consecutive queue slots at a time
// from an atomic ticket (the queue is ordered by descending sequence length).
#pragma once

#include "ck_device.cuh"

namespace ck {

enum { kNav = 0, kActor = 1 };

template <typename P, typename CV>
struct FitState {
  // stepper
  P pars[8];
  CV cov[21];
  Transport<P> T;
  P deriv[7];  // dir (3), dt/ds, k4 (3); the q/p entry is always zero
  double pathAcc;
  double cNav, cActor, cUser, cAcc;  // ConstrainedStep values
  float mass, absQ;
  int pdg;
  // last transport Jacobian (bound -> bound), row-major
  double jac[36];
};

template <typename P, typename CV>
CK_D double stepValue(const FitState<P, CV>& s) {
  double mn = fmin(s.cNav, fmin(s.cActor, s.cUser));
  double r = fmin(fabs(mn), s.cAcc);
  return signbit(mn) ? -r : r;
}

CK_D void cupdate(double& slot, double v) {
  if (fabs(v) < fabs(slot)) slot = v;
}

// ChargeHypothesis::extractMomentum (ChargeHypothesis.hpp:70-90)
template <typename P>
CK_D P absMomentum(float absQ, P qop) {
  float q = (float)copysign((double)absQ, (double)qop);
  return (P)q / qop;
}

enum StepErr { kStepOk = 0, kStepField = 1, kStepStalled = 2, kStepAdjust = 3 };

// EigenStepper::step with the default extension; transports T.
template <typename P, typename CV>
CK_D int rkStep(FitState<P, CV>& s, const DevField& F, const DevOptions& o, bool transport) {
  const P pos[3] = {s.pars[0], s.pars[1], s.pars[2]};
  const P dir[3] = {s.pars[4], s.pars[5], s.pars[6]};
  const P qop = s.pars[7];
  P B1[3], B2[3], B3[3];
  if (!getField(F, pos, B1)) return kStepField;
  P k1[3], k2[3], k3[3], k4[3];
  k1[0] = qop * (dir[1] * B1[2] - dir[2] * B1[1]);
  k1[1] = qop * (dir[2] * B1[0] - dir[0] * B1[2]);
  k1[2] = qop * (dir[0] * B1[1] - dir[1] * B1[0]);
  const P tol = (P)o.stepTolerance;
  const double initialH = stepValue(s);
  P h = (P)initialH;
  P err = P(0), h2 = P(0), hh = P(0);
  unsigned trials = 0;
  while (true) {
    ++trials;
    h2 = h * h;
    hh = h * P(0.5);
    P p1[3], t[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) p1[i] = pos[i] + hh * dir[i] + h2 * P(0.125) * k1[i];
    if (!getField(F, p1, B2)) return kStepField;
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * k1[i];
    k2[0] = qop * (t[1] * B2[2] - t[2] * B2[1]);
    k2[1] = qop * (t[2] * B2[0] - t[0] * B2[2]);
    k2[2] = qop * (t[0] * B2[1] - t[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * k2[i];
    k3[0] = qop * (t[1] * B2[2] - t[2] * B2[1]);
    k3[1] = qop * (t[2] * B2[0] - t[0] * B2[2]);
    k3[2] = qop * (t[0] * B2[1] - t[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) p1[i] = pos[i] + h * dir[i] + h2 * P(0.5) * k3[i];
    if (!getField(F, p1, B3)) return kStepField;
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + h * k3[i];
    k4[0] = qop * (t[1] * B3[2] - t[2] * B3[1]);
    k4[1] = qop * (t[2] * B3[0] - t[0] * B3[2]);
    k4[2] = qop * (t[0] * B3[1] - t[1] * B3[0]);
    P l1 = fabs(((k1[0] - k2[0]) - k3[0]) + k4[0]) + fabs(((k1[1] - k2[1]) - k3[1]) + k4[1]) +
           fabs(((k1[2] - k2[2]) - k3[2]) + k4[2]);
    err = h2 * l1;
    err = fmax(err, (P)1e-20);
    if (err <= P(4) * tol) break;
    P x = sqrt(sqrt(tol / err));
    x = fmin(fmax(x, P(0.25)), P(4));
    h = h * x;
    if (fabs((double)h) < fabs(o.stepSizeCutOff)) return kStepStalled;
    if (trials > o.maxRkTrials) return kStepAdjust;
  }
  // propagateTime + transportMatrix (EigenStepperDefaultExtension.hpp:86-228)
  const P m = (P)s.mass;
  const P p = absMomentum(s.absQ, qop);
  const P mp = m / p;
  const P dtds = sqrt(P(1) + mp * mp);
  s.pars[3] = s.pars[3] + h * dtds;
  s.deriv[3] = dtds;
  if (transport) {
    P dk1dL[3], dk2dL[3], dk3dL[3], dk4dL[3], t[3];
    dk1dL[0] = dir[1] * B1[2] - dir[2] * B1[1];
    dk1dL[1] = dir[2] * B1[0] - dir[0] * B1[2];
    dk1dL[2] = dir[0] * B1[1] - dir[1] * B1[0];
    const P qh = qop * hh, qf = qop * h;
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * k1[i];
    dk2dL[0] = (t[1] * B2[2] - t[2] * B2[1]) + qh * (dk1dL[1] * B2[2] - dk1dL[2] * B2[1]);
    dk2dL[1] = (t[2] * B2[0] - t[0] * B2[2]) + qh * (dk1dL[2] * B2[0] - dk1dL[0] * B2[2]);
    dk2dL[2] = (t[0] * B2[1] - t[1] * B2[0]) + qh * (dk1dL[0] * B2[1] - dk1dL[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * k2[i];
    dk3dL[0] = (t[1] * B2[2] - t[2] * B2[1]) + qh * (dk2dL[1] * B2[2] - dk2dL[2] * B2[1]);
    dk3dL[1] = (t[2] * B2[0] - t[0] * B2[2]) + qh * (dk2dL[2] * B2[0] - dk2dL[0] * B2[2]);
    dk3dL[2] = (t[0] * B2[1] - t[1] * B2[0]) + qh * (dk2dL[0] * B2[1] - dk2dL[1] * B2[0]);
#pragma unroll
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + h * k3[i];
    dk4dL[0] = (t[1] * B3[2] - t[2] * B3[1]) + qf * (dk3dL[1] * B3[2] - dk3dL[2] * B3[1]);
    dk4dL[1] = (t[2] * B3[0] - t[0] * B3[2]) + qf * (dk3dL[2] * B3[0] - dk3dL[0] * B3[2]);
    dk4dL[2] = (t[0] * B3[1] - t[1] * B3[0]) + qf * (dk3dL[0] * B3[1] - dk3dL[1] * B3[0]);

    // dkdT matrices (column j = d k / d T_j); cross of each column with B
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
    auto crossCols = [&](const P in[3][3], const P* B, P out[3][3]) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const P c0 = in[0][j], c1 = in[1][j], c2 = in[2][j];
        out[0][j] = qop * (c1 * B[2] - c2 * B[1]);
        out[1][j] = qop * (c2 * B[0] - c0 * B[2]);
        out[2][j] = qop * (c0 * B[1] - c1 * B[0]);
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

    const P h6 = h / P(6);
    const P hh6 = (h * h) / P(6);
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
    const P D37 = h * m * m / (p * p * qop * dtds);
    // T <- D T on the dynamic block (EigenStepper.ipp:310-352 in T form)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const P g0 = s.T.dyn[4][c], g1 = s.T.dyn[5][c], g2 = s.T.dyn[6][c];
      const P t7 = (c == 2) ? P(1) : P(0);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        s.T.dyn[i][c] =
            s.T.dyn[i][c] + (dFdT[i][0] * g0 + dFdT[i][1] * g1 + dFdT[i][2] * g2 + dFdL[i] * t7);
      }
      s.T.dyn[3][c] = s.T.dyn[3][c] + D37 * t7;
#pragma unroll
      for (int i = 0; i < 3; ++i)
        s.T.dyn[4 + i][c] = dGdT[i][0] * g0 + dGdT[i][1] * g1 + dGdT[i][2] * g2 + dGdL[i] * t7;
    }
  }
  // parameter update (EigenStepper.ipp:354-366)
  const P hh6 = h2 / P(6);
  const P h6 = h / P(6);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    s.pars[i] = s.pars[i] + (h * dir[i] + hh6 * ((k1[i] + k2[i]) + k3[i]));
    s.pars[4 + i] = s.pars[4 + i] + h6 * ((k1[i] + P(2) * (k2[i] + k3[i])) + k4[i]);
  }
  {
    P n2 = s.pars[4] * s.pars[4] + s.pars[5] * s.pars[5] + s.pars[6] * s.pars[6];
    P n = sqrt(n2);
    s.pars[4] = s.pars[4] / n;
    s.pars[5] = s.pars[5] / n;
    s.pars[6] = s.pars[6] / n;
  }
  s.deriv[0] = s.pars[4];
  s.deriv[1] = s.pars[5];
  s.deriv[2] = s.pars[6];
  s.deriv[4] = k4[0];
  s.deriv[5] = k4[1];
  s.deriv[6] = k4[2];
  s.pathAcc += (double)h;
  // step size accuracy (EigenStepper.ipp:379-385)
  P x = sqrt(sqrt(tol / err));
  x = fmin(fmax(x, P(0.25)), P(4));
  const double nextAcc = fabs((double)(h * x));
  if (nextAcc < fabs(initialH) || nextAcc > fabs(s.cAcc)) s.cAcc = nextAcc;
  return kStepOk;
}

// transportCovarianceToBound: J = F2B (I + deriv fTP) T, C <- J C J^T,
// reinitialise T at the surface (CovarianceEngine.cpp:102-165).
template <typename P, typename CV>
CK_D void transportToBound(FitState<P, CV>& s, const Surf<P>& sf) {
  const P pos[3] = {s.pars[0], s.pars[1], s.pars[2]};
  const P dir[3] = {s.pars[4], s.pars[5], s.pars[6]};
  P ex[3], ey[3], ez[3];
  referenceFrame(sf, pos, ex, ey, ez);
  const P dz = ez[0] * dir[0] + ez[1] * dir[1] + ez[2] * dir[2];
  const P f0 = -ez[0] / dz, f1 = -ez[1] / dz, f2 = -ez[2] / dz;
  const Trig<P> tg = trig(dir);
  // freeToSphericalDirectionJacobian rows
  const P a0 = -tg.sinPhi * tg.invSinTheta, a1 = tg.cosPhi * tg.invSinTheta;
  const P b0 = tg.cosPhi * tg.cosTheta, b1 = tg.sinPhi * tg.cosTheta, b2 = -tg.sinTheta;
  const P exd = ex[0] * s.deriv[0] + ex[1] * s.deriv[1] + ex[2] * s.deriv[2];
  const P eyd = ey[0] * s.deriv[0] + ey[1] * s.deriv[1] + ey[2] * s.deriv[2];
  const P phd = a0 * s.deriv[4] + a1 * s.deriv[5];
  const P thd = b0 * s.deriv[4] + b1 * s.deriv[5] + b2 * s.deriv[6];
  P J[6][6];
  // loc columns: T rows 0-2 only
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    const P t0 = s.T.loc[0][c], t1 = s.T.loc[1][c], t2 = s.T.loc[2][c];
    const P sc = f0 * t0 + f1 * t1 + f2 * t2;
    J[0][c] = (ex[0] * t0 + ex[1] * t1 + ex[2] * t2) + exd * sc;
    J[1][c] = (ey[0] * t0 + ey[1] * t1 + ey[2] * t2) + eyd * sc;
    J[2][c] = phd * sc;
    J[3][c] = thd * sc;
    J[4][c] = P(0);
    J[5][c] = s.deriv[3] * sc;
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const P t0 = s.T.dyn[0][c], t1 = s.T.dyn[1][c], t2 = s.T.dyn[2][c];
    const P sc = f0 * t0 + f1 * t1 + f2 * t2;
    const P g0 = s.T.dyn[4][c], g1 = s.T.dyn[5][c], g2 = s.T.dyn[6][c];
    J[0][2 + c] = (ex[0] * t0 + ex[1] * t1 + ex[2] * t2) + exd * sc;
    J[1][2 + c] = (ey[0] * t0 + ey[1] * t1 + ey[2] * t2) + eyd * sc;
    J[2][2 + c] = (a0 * g0 + a1 * g1) + phd * sc;
    J[3][2 + c] = (b0 * g0 + b1 * g1 + b2 * g2) + thd * sc;
    J[4][2 + c] = (c == 2) ? P(1) : P(0);
    J[5][2 + c] = s.T.dyn[3][c] + s.deriv[3] * sc;
  }
#pragma unroll
  for (int r = 0; r < 6; ++r) J[r][5] = (r == 5) ? P(1) : P(0);
#pragma unroll
  for (int r = 0; r < 6; ++r)
#pragma unroll
    for (int c = 0; c < 6; ++c) s.jac[r * 6 + c] = (double)J[r][c];
  // C <- J C J^T (packed)
  CV JC[6][6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      CV acc = CV(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) acc += (CV)J[i][k] * s.cov[sidx(k, j)];
      JC[i][j] = acc;
    }
  CV out[21];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      CV acc = CV(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) acc += JC[i][k] * (CV)J[j][k];
      out[sidx(i, j)] = acc;
    }
#pragma unroll
  for (int i = 0; i < 21; ++i) s.cov[i] = out[i];
  // reinitializeJacobians: only when the position is on the surface
#pragma unroll
  for (int i = 0; i < 7; ++i) s.deriv[i] = P(0);
  P loc[2];
  if (globalToLocal(sf, pos, kOnSurfaceTolerance, loc)) initTransport(sf, s.pars, s.T);
}

// scratch record access
struct Rec {
  double* base;
  int ns;
  int slot;
  CK_D double& at(int k, int f) const {
    return base[((size_t)k * kRecDoubles + f) * (size_t)ns + slot];
  }
};

template <typename P, typename CV>
CK_D void fitTrack(const FitParams& fp, int slot, int t) {
  const DevOptions& o = fp.opt;
  FitState<P, CV> s;
  const int maxStates = fp.max_states;
  Rec rec{fp.rec, fp.n_slots, slot};
  auto metaI = [&](int k, int f) -> int32_t& {
    return fp.rec_meta[((size_t)k * 2 + f) * (size_t)fp.n_slots + slot];
  };
  auto metaD = [&](int k, int f) -> double& {
    return fp.rec_meta_d[((size_t)k * 2 + f) * (size_t)fp.n_slots + slot];
  };
  const ck_batch_out& out = fp.out;
  const size_t n = (size_t)fp.n_tracks;
  auto fail = [&](int code) {
    out.status[t] = code;
    if (out.n_states) out.n_states[t] = 0;
    if (out.n_measurements) out.n_measurements[t] = 0;
    if (out.n_holes) out.n_holes[t] = 0;
    if (out.n_outliers) out.n_outliers[t] = 0;
    if (out.ndf) out.ndf[t] = 0;
    if (out.chi2_sum) out.chi2_sum[t] = 0.0;
  };

  // ---- initialise the stepper (EigenStepper.ipp:37-70)
  {
    double sp[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) sp[i] = fp.start_params[6 * (size_t)t + i];
    Surf<P> start;
    start.loadPlane(fp.start_frames + 12 * (size_t)t);
    boundToFree(start, sp, s.pars);
    initTransport(start, s.pars, s.T);
    const double* sc = fp.start_cov + 36 * (size_t)t;
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j) s.cov[sidx(i, j)] = (CV)sc[i * 6 + j];
  }
#pragma unroll
  for (int i = 0; i < 7; ++i) s.deriv[i] = P(0);
  s.pathAcc = 0.0;
  s.cNav = kNotSet;
  s.cActor = kNotSet;
  s.cUser = o.maxStepSize;
  s.cAcc = o.initialStepSize;
  s.mass = fp.particle[2 * (size_t)t];
  s.absQ = fp.particle[2 * (size_t)t + 1];
  s.pdg = fp.pdg ? fp.pdg[t] : 211;

  const int seq0 = fp.seq_off[t], nSeq = fp.seq_off[t + 1] - seq0;
  const int m0 = fp.meas_off[t], nMeas = fp.meas_off[t + 1] - m0;
  // surface ids index the device table: reject out-of-range ids
  {
    bool bad = nSeq < 0 || nMeas < 0;
    for (int i = 0; i < nSeq && !bad; ++i) {
      const int sid = fp.seq_surf[seq0 + i];
      bad |= sid < 0 || sid >= fp.n_surfaces;
    }
    for (int i = 0; i < nMeas && !bad; ++i) {
      const int sid = fp.meas_surf[m0 + i];
      bad |= sid < 0 || sid >= fp.n_surfaces;
    }
    if (bad) {
      fail(CK_TRACK_INVALID_INPUT);
      return;
    }
  }
  auto findMeas = [&](int sid) -> int {
    for (int i = 0; i < nMeas; ++i)
      if (fp.meas_surf[m0 + i] == sid) return m0 + i;
    return -1;
  };
  int nDistinct = 0;
  for (int i = 0; i < nMeas; ++i) {
    const int si = fp.meas_surf[m0 + i];
    bool dup = false;
    for (int j = 0; j < i; ++j) dup |= (fp.meas_surf[m0 + j] == si);
    nDistinct += dup ? 0 : 1;
  }
  int lastSlSeq = -1;
  for (int k = 0; k < nSeq; ++k)
    if (findMeas(fp.seq_surf[seq0 + k]) >= 0) lastSlSeq = k;

  // loop protection (LoopProtection.hpp:19-72)
  auto loopLimit = [&](double previous, bool release) -> double {
    double limit = previous;
    if (!o.loopProtection) return limit;
    if (release) limit = kNotSet;
    P B[3];
    const P pos[3] = {s.pars[0], s.pars[1], s.pars[2]};
    if (!getField(fp.field, pos, B)) return limit;
    const double Bn = sqrt((double)B[0] * (double)B[0] + (double)B[1] * (double)B[1] +
                           (double)B[2] * (double)B[2]);
    if (Bn == 0.0) return limit;
    const double p = (double)absMomentum(s.absQ, s.pars[7]);
    const double ll = o.loopFraction * (2.0 * kPi * p / Bn);
    if (fabs(ll) < fabs(limit)) limit = ll;
    return limit;
  };
  const double propLimit = loopLimit(o.pathLimit, false);
  double kfLimit = kNotSet;
  auto pathLimitReached = [&](double limit) -> bool {
    const double distance = fabs(limit) - fabs(s.pathAcc);
    if (fabs(distance) < fabs(o.surfaceTolerance)) return true;
    cupdate(s.cActor, distance);
    return false;
  };

  // navigator
  int surfaceIndex = -1;
  bool navigationBreak = false;
  int currentSurface = -1;
  int targetSurf = -1, targetIdx = 0;
  bool haveTarget = false;

  int nStates = 0;
  int lastMeasurementIndex = -1;
  int measurementStates = 0;
  bool finished = false;
  // After the last surface that carries a source link every further state
  // lies beyond the track's tip: only the trajectory and the errors it may
  // raise stay observable, so covariance and Jacobian transport stop.
  bool coasting = false;
  int err = CK_TRACK_OK;

  auto intersectSurf = [&](int sid, P path[2], int st[2]) -> int {
    Surf<P> sf;
    sf.load(fp.surfaces + sid);
    const P pos[3] = {s.pars[0], s.pars[1], s.pars[2]};
    const P dir[3] = {s.pars[4], s.pars[5], s.pars[6]};
    return intersect(sf, pos, dir, (P)o.surfaceTolerance, path, st);
  };

  // material interaction; mode 1 pre, 2 post, 3 full. False: not on surface
  auto material = [&](int sid, const Surf<P>& sf, int mode) -> bool {
    const DevSurface* ds = fp.surfaces + sid;
    if (!(__ldg(&ds->flags) & CK_SURF_MATERIAL)) return true;
    const P pos[3] = {s.pars[0], s.pars[1], s.pars[2]};
    const P dir[3] = {s.pars[4], s.pars[5], s.pars[6]};
    const P pc = pathCorrection(sf, pos, dir);
    P loc[2];
    if (!globalToLocal(sf, pos, kOnSurfaceTolerance, loc)) return false;
    float f1 = 1.0f;
    if (__ldg(&ds->vacuum) == 0) {
      const float split = __ldg(&ds->split);
      const double factor = (mode == 3) ? 1.0 : (mode == 1 ? 1.0 - (double)split : (double)split);
      if (factor == 0.0) return true;
      f1 = (float)factor;
    }
    bool vac = false;
    const float qOverPf = (float)s.pars[7];
    const MatEffects e =
        materialEffects<P>(fp.mc, ds, f1, (float)pc, s.pdg, s.mass, s.absQ, dir, qOverPf,
                           o.multipleScattering != 0, o.energyLoss != 0, vac);
    if (vac) return true;
    const double massd = (double)s.mass;
    const double mom = (double)absMomentum(s.absQ, s.pars[7]);
    const double nextE = sqrt(massd * massd + mom * mom) - e.eLoss;
    double nextP = 0.0;
    if (massd < nextE) {
      const double am = fabs(massd);
      nextP = sqrt((nextE - am) * (nextE + am));
    }
    nextP = fmax(0.01, nextP);
    const float signedQ = (float)copysign((double)s.absQ, (double)qOverPf);
    s.pars[7] = (P)((double)signedQ / nextP);
    s.cov[sidx(2, 2)] = (CV)fmax(0.0, (double)s.cov[sidx(2, 2)] + e.varPhi);
    s.cov[sidx(3, 3)] = (CV)fmax(0.0, (double)s.cov[sidx(3, 3)] + e.varTheta);
    s.cov[sidx(4, 4)] = (CV)fmax(0.0, (double)s.cov[sidx(4, 4)] + e.varQoP);
    return true;
  };

  auto writeRecordPred = [&](int k, const double bp[6]) {
#pragma unroll
    for (int i = 0; i < 6; ++i) rec.at(k, kRecPred + i) = bp[i];
#pragma unroll
    for (int i = 0; i < 21; ++i) rec.at(k, kRecPredCov + i) = (double)s.cov[i];
#pragma unroll
    for (int i = 0; i < 36; ++i) rec.at(k, kRecJac + i) = s.jac[i];
  };

  // KalmanFitter::Actor::filter
  auto filter = [&](int sid) -> int {
    Surf<P> sf;
    sf.load(fp.surfaces + sid);
    const int sflags = __ldg(&fp.surfaces[sid].flags);
    const bool sensitive = (sflags & CK_SURF_SENSITIVE) != 0;
    const bool hasMat = (sflags & CK_SURF_MATERIAL) != 0;
    const bool preceding = measurementStates > 0;
    if (coasting) {
      if ((preceding && sensitive) || hasMat) {
        double bp[6];
        if (!freeToBound(s.pars, sf, bp)) return CK_TRACK_NOT_ON_SURFACE;
        if (!material(sid, sf, 3)) return CK_TRACK_NOT_ON_SURFACE;
      }
      return CK_TRACK_OK;
    }
    const int mi = findMeas(sid);
    if (mi >= 0) {
      transportToBound(s, sf);
      if (!material(sid, sf, 1)) return CK_TRACK_NOT_ON_SURFACE;
      double bp[6];
      if (!freeToBound(s.pars, sf, bp)) return CK_TRACK_NOT_ON_SURFACE;
      if (nStates >= maxStates) return CK_TRACK_TOO_MANY_STATES;
      const int k = nStates++;
      writeRecordPred(k, bp);
      uint32_t flags = CK_FLAG_HAS_PARAMETERS | (hasMat ? CK_FLAG_HAS_MATERIAL : 0u);
      double Pp[21];
#pragma unroll
      for (int i = 0; i < 21; ++i) Pp[i] = (double)s.cov[i];
      const double mv0 = fp.meas_val[2 * (size_t)mi], mv1 = fp.meas_val[2 * (size_t)mi + 1];
      double V[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) V[i] = fp.meas_cov[4 * (size_t)mi + i];
      bool outlier = false;
      if (o.useOutlierCut) outlier = predictedChi2(bp, Pp, mv0, mv1, V) > o.outlierChi2Cut;
      double chi2 = 0.0;
      if (!outlier) {
        double filt[6], F[21];
        if (!kalmanUpdate(bp, Pp, mv0, mv1, V, o.joseph != 0, filt, F, chi2))
          return CK_TRACK_UPDATE_FAILED;
        flags |= CK_FLAG_HAS_MEASUREMENT;
#pragma unroll
        for (int i = 0; i < 6; ++i) rec.at(k, kRecFilt + i) = filt[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) rec.at(k, kRecFiltCov + i) = F[i];
        // stepper.update (EigenStepper.ipp:128-138)
        boundToFree(sf, filt, s.pars);
#pragma unroll
        for (int i = 0; i < 21; ++i) s.cov[i] = (CV)F[i];
        initTransport(sf, s.pars, s.T);
        ++measurementStates;
      } else {
        flags |= CK_FLAG_HAS_MEASUREMENT | CK_FLAG_IS_OUTLIER;
#pragma unroll
        for (int i = 0; i < 6; ++i) rec.at(k, kRecFilt + i) = bp[i];
#pragma unroll
        for (int i = 0; i < 21; ++i) rec.at(k, kRecFiltCov + i) = Pp[i];
      }
      metaI(k, 0) = sid;
      metaI(k, 1) = (int32_t)flags;
      metaD(k, 0) = s.pathAcc;
      metaD(k, 1) = chi2;
      if (!material(sid, sf, 2)) return CK_TRACK_NOT_ON_SURFACE;
      lastMeasurementIndex = k;
    } else if ((preceding && sensitive) || hasMat) {
      double bp[6];
      if (!freeToBound(s.pars, sf, bp)) return CK_TRACK_NOT_ON_SURFACE;
      transportToBound(s, sf);
      if (nStates >= maxStates) return CK_TRACK_TOO_MANY_STATES;
      const int k = nStates++;
      writeRecordPred(k, bp);
#pragma unroll
      for (int i = 0; i < 6; ++i) rec.at(k, kRecFilt + i) = bp[i];
#pragma unroll
      for (int i = 0; i < 21; ++i) rec.at(k, kRecFiltCov + i) = (double)s.cov[i];
      uint32_t flags = CK_FLAG_HAS_PARAMETERS | (hasMat ? CK_FLAG_HAS_MATERIAL : 0u);
      if (sensitive && preceding) flags |= CK_FLAG_IS_HOLE;
      metaI(k, 0) = sid;
      metaI(k, 1) = (int32_t)flags;
      metaD(k, 0) = s.pathAcc;
      metaD(k, 1) = 0.0;
      if (!material(sid, sf, 3)) return CK_TRACK_NOT_ON_SURFACE;
    }
    return CK_TRACK_OK;
  };

  auto act = [&]() -> int {
    if (finished) return CK_TRACK_OK;
    if (kfLimit == kNotSet) kfLimit = loopLimit(kfLimit, true);
    if (currentSurface >= 0) {
      const int r = filter(currentSurface);
      if (r != CK_TRACK_OK) return r;
    }
    bool complete = measurementStates == nDistinct;
    // every later state would be created after the track's tip
    if (!complete && lastSlSeq >= 0 && currentSurface >= 0 && surfaceIndex >= lastSlSeq) {
      if (o.earlyTermination)
        complete = true;
      else
        coasting = true;
    }
    const bool pathReached = pathLimitReached(kfLimit);
    if (complete || pathReached) finished = true;
    return CK_TRACK_OK;
  };
  auto checkAbort = [&]() -> bool {
    if (finished) return true;
    return pathLimitReached(propLimit);
  };
  auto nextTargetNav = [&]() -> bool {
    currentSurface = -1;
    if (navigationBreak) return false;
    ++surfaceIndex;
    while (surfaceIndex < nSeq) {
      const int sid = fp.seq_surf[seq0 + surfaceIndex];
      P path[2];
      int st[2];
      const int ni = intersectSurf(sid, path, st);
      for (int i = 0; i < ni; ++i) {
        if (st[i] != 0 && (double)path[i] > o.nearLimit && (double)path[i] < kNotSet) {
          targetSurf = sid;
          targetIdx = i;
          return true;
        }
      }
      ++surfaceIndex;
    }
    navigationBreak = true;
    return false;
  };
  // 0 unreachable, 1 reachable, 2 on surface
  auto surfaceStatus = [&](int sid, int idx) -> int {
    P path[2];
    int st[2];
    intersectSurf(sid, path, st);
    const P pl = idx ? path[1] : path[0];
    const int stt = idx ? st[1] : st[0];
    if (stt == 2 || stt == 1) {
      s.cNav = kNotSet;
      cupdate(s.cNav, (double)pl);
    }
    return stt;
  };
  auto getNextTarget = [&](int& e) -> bool {
    e = CK_TRACK_OK;
    for (unsigned i = 0; i < o.maxTargetSkipping; ++i) {
      if (!nextTargetNav()) return false;
      const int stt = surfaceStatus(targetSurf, targetIdx);
      if (stt == 2) continue;
      if (stt == 1) return true;
    }
    e = CK_TRACK_NEXT_TARGET_LIMIT;
    return false;
  };

  // ---- Propagator::propagate
  err = act();
  if (err == CK_TRACK_OK && !checkAbort()) {
    int e;
    haveTarget = getNextTarget(e);
    if (e != CK_TRACK_OK) err = e;
    bool terminated = false;
    unsigned steps = 0;
    for (; err == CK_TRACK_OK && steps < o.maxSteps; ++steps) {
      const int se = rkStep(s, fp.field, o, !coasting);
      if (se != kStepOk) {
        err = se == kStepField ? CK_TRACK_FIELD_OUT_OF_BOUNDS
                               : (se == kStepStalled ? CK_TRACK_STEP_SIZE_STALLED
                                                     : CK_TRACK_STEP_ADJUST_FAILED);
        break;
      }
      s.cNav = kNotSet;
      s.cActor = kNotSet;
      if (haveTarget) {
        const int post = surfaceStatus(targetSurf, targetIdx);
        if (post == 2 && !navigationBreak) currentSurface = fp.seq_surf[seq0 + surfaceIndex];
        if (post != 1) haveTarget = false;
      }
      err = act();
      if (err != CK_TRACK_OK) break;
      if (checkAbort()) {
        terminated = true;
        break;
      }
      if (!haveTarget) {
        s.cNav = kNotSet;
        haveTarget = getNextTarget(e);
        if (e != CK_TRACK_OK) {
          err = e;
          break;
        }
      }
    }
    if (err == CK_TRACK_OK && !terminated) err = CK_TRACK_STEP_COUNT_LIMIT;
  }
  if (err != CK_TRACK_OK) {
    fail(err);
    return;
  }
  if (measurementStates == 0) {
    fail(CK_TRACK_NO_MEASUREMENT_FOUND);
    return;
  }

  // ---- smoothing (GainMatrixSmoother) and output
  const int tip = lastMeasurementIndex;
  int lastMeas = tip;
  for (int k = tip; k >= 0; --k) {
    const uint32_t fl = (uint32_t)metaI(k, 1);
    if ((fl & CK_FLAG_HAS_MEASUREMENT) && !(fl & CK_FLAG_IS_OUTLIER)) {
      lastMeas = k;
      break;
    }
  }
  auto at = [&](int k, int C, int c) -> size_t { return ((size_t)k * C + c) * n + t; };
  int nM = 0, nH = 0, nO = 0, ndf = 0;
  double chi2sum = 0.0;
  double ps[6], Psp[21];
  // writes state k; `sm`/`Ps` its smoothed state, filtered from the record
  // unless `filtOverride` (the shared smoothed/filtered storage case)
  auto writeState = [&](int k, const double sm[6], const double Ps[21], bool filtOverride) {
    const uint32_t fl = (uint32_t)metaI(k, 1);
    if (out.state_surface) out.state_surface[at(k, 1, 0)] = metaI(k, 0);
    if (out.state_flags) out.state_flags[at(k, 1, 0)] = fl;
    if (out.state_path_length) out.state_path_length[at(k, 1, 0)] = metaD(k, 0);
    const double c2 = metaD(k, 1);
    if (out.state_chi2) out.state_chi2[at(k, 1, 0)] = c2;
    if (fl & CK_FLAG_IS_HOLE) {
      ++nH;
    } else if (fl & CK_FLAG_IS_OUTLIER) {
      ++nO;
    } else if (fl & CK_FLAG_HAS_MEASUREMENT) {
      ++nM;
      chi2sum += c2;
      ndf += 2;
    }
    if (out.smoothed) {
#pragma unroll
      for (int i = 0; i < 6; ++i) out.smoothed[at(k, 6, i)] = sm[i];
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j) out.smoothed_cov[at(k, 36, i * 6 + j)] = Ps[sidx(i, j)];
    }
    if (out.filtered) {
#pragma unroll
      for (int i = 0; i < 6; ++i)
        out.filtered[at(k, 6, i)] = filtOverride ? sm[i] : rec.at(k, kRecFilt + i);
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j)
          out.filtered_cov[at(k, 36, i * 6 + j)] =
              filtOverride ? Ps[sidx(i, j)] : rec.at(k, kRecFiltCov + sidx(i, j));
    }
    if (out.predicted) {
#pragma unroll
      for (int i = 0; i < 6; ++i) out.predicted[at(k, 6, i)] = rec.at(k, kRecPred + i);
#pragma unroll
      for (int i = 0; i < 6; ++i)
#pragma unroll
        for (int j = 0; j < 6; ++j)
          out.predicted_cov[at(k, 36, i * 6 + j)] = rec.at(k, kRecPredCov + sidx(i, j));
    }
    if (out.jacobian) {
#pragma unroll
      for (int i = 0; i < 36; ++i) out.jacobian[at(k, 36, i)] = rec.at(k, kRecJac + i);
    }
  };
#pragma unroll
  for (int i = 0; i < 6; ++i) ps[i] = rec.at(tip, kRecFilt + i);
#pragma unroll
  for (int i = 0; i < 21; ++i) Psp[i] = rec.at(tip, kRecFiltCov + i);
  writeState(tip, ps, Psp, false);
  int status = CK_TRACK_OK;
  for (int k = tip - 1; k >= 0; --k) {
    double filt[6], Pf[21], pp[6], Ppp[21], J[36], sm[6], Ps[21];
#pragma unroll
    for (int i = 0; i < 6; ++i) filt[i] = rec.at(k, kRecFilt + i);
#pragma unroll
    for (int i = 0; i < 21; ++i) Pf[i] = rec.at(k, kRecFiltCov + i);
#pragma unroll
    for (int i = 0; i < 6; ++i) pp[i] = rec.at(k + 1, kRecPred + i);
#pragma unroll
    for (int i = 0; i < 21; ++i) Ppp[i] = rec.at(k + 1, kRecPredCov + i);
#pragma unroll
    for (int i = 0; i < 36; ++i) J[i] = rec.at(k + 1, kRecJac + i);
    if (!smoothStep(filt, Pf, pp, Ppp, J, ps, Psp, sm, Ps)) {
      status = CK_TRACK_SMOOTH_FAILED;
      break;
    }
    writeState(k, sm, Ps, k == lastMeas);
#pragma unroll
    for (int i = 0; i < 6; ++i) ps[i] = sm[i];
#pragma unroll
    for (int i = 0; i < 21; ++i) Psp[i] = Ps[i];
  }
  if (status != CK_TRACK_OK) {
    fail(status);
    return;
  }
  out.status[t] = CK_TRACK_OK;
  if (out.n_states) out.n_states[t] = tip + 1;
  if (out.n_measurements) out.n_measurements[t] = nM;
  if (out.n_holes) out.n_holes[t] = nH;
  if (out.n_outliers) out.n_outliers[t] = nO;
  if (out.ndf) out.ndf[t] = ndf;
  if (out.chi2_sum) out.chi2_sum[t] = chi2sum;
}

// Persistent fit kernel: each warp takes 32 consecutive queue slots per
// ticket until the queue is drained.
template <typename P, typename CV, int BLOCK, int MINB>
__global__ void __launch_bounds__(BLOCK, MINB) fitKernel(FitParams fp) {
  const int lane = threadIdx.x & 31;
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  while (true) {
    int base = 0;
    if (lane == 0) base = atomicAdd(fp.ticket, 32);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= fp.n_queue) break;
    const int q = base + lane;
    if (q < fp.n_queue) fitTrack<P, CV>(fp, slot, fp.perm ? fp.perm[q] : q);
  }
}

}  // namespace ck
