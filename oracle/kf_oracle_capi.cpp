// kf_oracle_capi.cpp — C entry points of the CPU oracle (test infrastructure).
//
// Loaded only by tests/, __graft_entry__.smoke() and bench.py's CPU legs,
// always as the checker or the timed CPU baseline, never as the product.
// Inputs and outputs use the public structs of include/cudakalman.h so that
// the oracle and the CUDA fitter are fed from and compared on the very same
// arrays.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <thread>
#include <vector>

#include "kf_oracle.hpp"

using namespace kfo;

namespace {

struct Ctx {
  std::vector<Surface<double>> surfaces;
  Fitter<double> fitter;
};

void writeTrack(const TrackOut& t, int tr, int n, const ck_batch_out* out) {
  const int ms = out->max_states;
  out->status[tr] = t.status;
  if (out->n_states) out->n_states[tr] = (int)t.states.size();
  if (out->n_measurements) out->n_measurements[tr] = t.nMeasurements;
  if (out->n_holes) out->n_holes[tr] = t.nHoles;
  if (out->n_outliers) out->n_outliers[tr] = t.nOutliers;
  if (out->ndf) out->ndf[tr] = t.ndf;
  if (out->chi2_sum) out->chi2_sum[tr] = t.chi2;
  const int ns = (int)t.states.size();
  if (ns > ms) {
    out->status[tr] = CK_TRACK_TOO_MANY_STATES;
    if (out->n_states) out->n_states[tr] = 0;
    return;
  }
  if (t.hasTrackParams) {
    for (int c = 0; c < 6; ++c)
      if (out->track_params) out->track_params[(size_t)c * n + tr] = t.trackParams[c];
    for (int c = 0; c < 36; ++c)
      if (out->track_cov) out->track_cov[(size_t)c * n + tr] = t.trackCov[c];
  }
  auto at = [&](int k, int C, int c) -> size_t { return ((size_t)k * C + c) * n + tr; };
  for (int k = 0; k < ns; ++k) {
    const TrackOut::St& s = t.states[k];
    if (out->state_surface) out->state_surface[at(k, 1, 0)] = s.surface;
    if (out->state_flags) out->state_flags[at(k, 1, 0)] = s.flags;
    if (out->state_path_length) out->state_path_length[at(k, 1, 0)] = s.pathLength;
    if (out->state_chi2) out->state_chi2[at(k, 1, 0)] = s.chi2;
    for (int c = 0; c < 6; ++c) {
      if (out->predicted) out->predicted[at(k, 6, c)] = s.pred[c];
      if (out->filtered) out->filtered[at(k, 6, c)] = s.filt[c];
      if (out->smoothed) out->smoothed[at(k, 6, c)] = s.smth[c];
    }
    for (int c = 0; c < 36; ++c) {
      if (out->predicted_cov) out->predicted_cov[at(k, 36, c)] = s.predCov[c];
      if (out->filtered_cov) out->filtered_cov[at(k, 36, c)] = s.filtCov[c];
      if (out->smoothed_cov) out->smoothed_cov[at(k, 36, c)] = s.smthCov[c];
      if (out->jacobian) out->jacobian[at(k, 36, c)] = s.jac[c];
    }
  }
}

void fitOne(const Ctx& ctx, const ck_batch_in* in, int tr, TrackOut& t) {
  const int ns = (int)ctx.surfaces.size();
  // (a line surface is only a reference surface: not in a sequence, no
  // measurement on it)
  auto bad = [&](int sid) { return sid < 0 || sid >= ns || ctx.surfaces[sid].type == CK_SURFACE_LINE; };
  for (int k = in->seq_offsets[tr]; k < in->seq_offsets[tr + 1]; ++k)
    if (bad(in->seq_surfaces[k])) {
      t.status = CK_TRACK_INVALID_INPUT;
      return;
    }
  for (int k = in->meas_offsets[tr]; k < in->meas_offsets[tr + 1]; ++k)
    if (bad(in->meas_surfaces[k]) ||
        (in->meas_subspace && (in->meas_subspace[k] < CK_MEAS_LOC0 ||
                               in->meas_subspace[k] > CK_MEAS_LOC01))) {
      t.status = CK_TRACK_INVALID_INPUT;
      return;
    }
  std::vector<MeasRec<double>> meas;
  for (int m = in->meas_offsets[tr]; m < in->meas_offsets[tr + 1]; ++m) {
    MeasRec<double> r;
    r.surface = in->meas_surfaces[m];
    r.sub = in->meas_subspace ? in->meas_subspace[m] : CK_MEAS_LOC01;
    r.v[0] = in->meas_values[2 * m];
    r.v[1] = in->meas_values[2 * m + 1];
    for (int c = 0; c < 4; ++c) r.cov[c] = in->meas_cov[4 * m + c];
    meas.push_back(r);
  }
  Surface<double> start = Surface<double>::plane(in->start_frames + 12 * (size_t)tr);
  Vec<double, 6> sp = get6<double>(in->start_params + 6 * (size_t)tr);
  Mat<double, 6, 6> sc = get36<double>(in->start_cov + 36 * (size_t)tr);
  const int s0 = in->seq_offsets[tr], s1 = in->seq_offsets[tr + 1];
  ctx.fitter.fit(start, sp, sc, in->particle[2 * tr], in->particle[2 * tr + 1],
                 in->particle_pdg ? in->particle_pdg[tr] : 211, in->seq_surfaces + s0, s1 - s0,
                 meas, t);
}

}  // namespace

extern "C" {

// Fits a host-memory batch on `n_threads` host threads (dynamic scheduling
// over tracks). `coast` = 1 reproduces the reference termination exactly
// (propagation continues to the path limit when outliers keep the track
// incomplete); 0 stops after the last surface that carries a source link
// (ck_options.early_termination); -1 follows the options. Returns the wall
// time in seconds.
double kfo_fit_batch(const ck_options* opt, int n_surfaces, const ck_surface* surfaces,
                     const ck_field* field, const ck_batch_in* in, const ck_batch_out* out,
                     int n_threads, int coast, int first, int count) {
  Ctx ctx;
  for (int i = 0; i < n_surfaces; ++i) ctx.surfaces.push_back(Surface<double>::fromCk(surfaces[i]));
  ctx.fitter.surfaces = &ctx.surfaces;
  ctx.fitter.field = Field<double>::make(*field);
  ctx.fitter.mc = MatConst::make();
  const bool doCoast = coast < 0 ? (opt->early_termination == 0) : (coast != 0);
  ctx.fitter.o = Options::fromCk(*opt, doCoast);
  const int n = in->n_tracks;
  if (count < 0) count = n - first;
  if (n_threads < 1) n_threads = 1;
  std::atomic<int> next{first};
  const int end = first + count;
  auto t0 = std::chrono::steady_clock::now();
  auto worker = [&]() {
    TrackOut t;
    while (true) {
      int tr = next.fetch_add(1);
      if (tr >= end) break;
      t = TrackOut();
      fitOne(ctx, in, tr, t);
      if (out) writeTrack(t, tr, n, out);
    }
  };
  if (n_threads == 1) {
    worker();
  } else {
    std::vector<std::thread> th;
    for (int i = 0; i < n_threads; ++i) th.emplace_back(worker);
    for (auto& x : th) x.join();
  }
  auto t1 = std::chrono::steady_clock::now();
  return std::chrono::duration<double>(t1 - t0).count();
}

// GainMatrixUpdater on n states (AoS), as ck_gain_matrix_update.
void kfo_gain_matrix_update(int n, int joseph, const double* pred, const double* predCov,
                            const double* meas, const double* measCov, const int* subspace,
                            double* filt, double* filtCov, double* chi2, int* status) {
  for (int i = 0; i < n; ++i) {
    Vec<double, 6> p = get6<double>(pred + 6 * i), f;
    Mat<double, 6, 6> P = get36<double>(predCov + 36 * i), F;
    double c2 = 0;
    MeasRec<double> m;
    m.surface = 0;
    m.sub = subspace ? subspace[i] : CK_MEAS_LOC01;
    for (int c = 0; c < 2; ++c) m.v[c] = meas[2 * i + c];
    for (int c = 0; c < 4; ++c) m.cov[c] = measCov[4 * i + c];
    bool ok = gainMatrixUpdateSub(p, P, m, joseph != 0, f, F, c2);
    status[i] = ok ? CK_TRACK_OK : CK_TRACK_UPDATE_FAILED;
    if (ok) {
      put6(filt + 6 * i, f);
      put36(filtCov + 36 * i, F);
      chi2[i] = c2;
    }
  }
}

// GainMatrixSmoother on n_traj trajectories of n_states (forward order).
void kfo_gain_matrix_smooth(int n_traj, int n_states, const double* pred, const double* predCov,
                            const double* filt, const double* filtCov, const double* jac,
                            double* smth, double* smthCov, int* status) {
  for (int t = 0; t < n_traj; ++t) {
    size_t b = (size_t)t * n_states;
    int last = n_states - 1;
    std::vector<Vec<double, 6>> S(n_states);
    std::vector<Mat<double, 6, 6>> SC(n_states);
    S[last] = get6<double>(filt + 6 * (b + last));
    SC[last] = get36<double>(filtCov + 36 * (b + last));
    status[t] = CK_TRACK_OK;
    for (int k = last - 1; k >= 0; --k) {
      bool ok = smoothStep(get6<double>(filt + 6 * (b + k)), get36<double>(filtCov + 36 * (b + k)),
                           get6<double>(pred + 6 * (b + k + 1)),
                           get36<double>(predCov + 36 * (b + k + 1)),
                           get36<double>(jac + 36 * (b + k + 1)), S[k + 1], SC[k + 1], S[k], SC[k]);
      if (!ok) {
        status[t] = CK_TRACK_SMOOTH_FAILED;
        break;
      }
    }
    for (int k = 0; k < n_states; ++k) {
      put6(smth + 6 * (b + k), S[k]);
      put36(smthCov + 36 * (b + k), SC[k]);
    }
  }
}

// MbfSmoother on n_traj trajectories of n_states (forward order), smoothed
// backwards from the last state; flags select the measurement visit.
void kfo_mbf_smooth(int n_traj, int n_states, const uint32_t* flags, const double* pred,
                    const double* predCov, const double* filt, const double* filtCov,
                    const double* jac, const double* meas, const double* measCov, double* smth,
                    double* smthCov) {
  for (int t = 0; t < n_traj; ++t) {
    size_t b = (size_t)t * n_states;
    Mat<double, 6, 6> L = Mat<double, 6, 6>::zero();
    Vec<double, 6> l = Vec<double, 6>::zero();
    for (int k = n_states - 1; k >= 0; --k) {
      const size_t s = b + k;
      Vec<double, 6> sm;
      Mat<double, 6, 6> Ps;
      mbfSmoothed(get6<double>(filt + 6 * s), get36<double>(filtCov + 36 * s), L, l, false, sm,
                  Ps);
      put6(smth + 6 * s, sm);
      put36(smthCov + 36 * s, Ps);
      if (k == 0) break;
      const Mat<double, 6, 6> F = get36<double>(jac + 36 * s);
      if ((flags[s] & CK_FLAG_HAS_MEASUREMENT) && !(flags[s] & CK_FLAG_IS_OUTLIER))
        mbfVisitMeasurement(F, get6<double>(pred + 6 * s), get36<double>(predCov + 36 * s),
                            meas + 2 * s, measCov + 4 * s, L, l);
      else
        mbfVisitNonMeasurement(F, L, l);
    }
  }
}

// LineSurface::globalToLocal / intersect (LineSurface.cpp:70-96,141-185) of
// a line surface with rotation rot (row-major, line = column 2) through
// center, for the known-answer tests. globalToLocal: 1 on success (the
// tolerance is infinite, as the reference test calls it); intersect: the
// status 0 unreachable, 1 reachable, 2 on surface, and the path length.
int kfo_line_global_to_local(const double* center, const double* rot, const double* pos,
                             const double* dir, double* loc) {
  ck_surface cs{};
  cs.type = CK_SURFACE_LINE;
  for (int i = 0; i < 9; ++i) cs.rotation[i] = rot[i];
  for (int i = 0; i < 3; ++i) cs.center[i] = center[i];
  Surface<double> s = Surface<double>::fromCk(cs);
  V3<double> p{{pos[0], pos[1], pos[2]}}, d{{dir[0], dir[1], dir[2]}};
  return s.globalToLocal(p, d, std::numeric_limits<double>::max(), loc) ? 1 : 0;
}

int kfo_line_intersect(const double* center, const double* rot, const double* pos,
                       const double* dir, double* path) {
  ck_surface cs{};
  cs.type = CK_SURFACE_LINE;
  for (int i = 0; i < 9; ++i) cs.rotation[i] = rot[i];
  for (int i = 0; i < 3; ++i) cs.center[i] = center[i];
  Surface<double> s = Surface<double>::fromCk(cs);
  V3<double> p{{pos[0], pos[1], pos[2]}}, d{{dir[0], dir[1], dir[2]}};
  Intersection<double> is[2];
  const int n = s.intersect(p, d, kOnSurfaceTolerance, is);
  *path = is[0].pathLength;
  if (n == 0) return 0;
  return is[0].status == IStatus::onSurface ? 2 : 1;
}

// detail::CorrectedFreeToBoundTransformer on one free state and covariance
// (8, 64 row-major) and a surface: 1 with the corrected bound mean (6) and
// covariance (36), 0 when no correction applies.
int kfo_corrected_free_to_bound(const ck_surface* cs, const double* freePars,
                                const double* freeCov, double* mean, double* cov) {
  Surface<double> s = Surface<double>::fromCk(*cs);
  Vec<double, 8> f;
  for (int i = 0; i < 8; ++i) f[i] = freePars[i];
  Mat<double, 8, 8> C;
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) C.a[i][j] = freeCov[i * 8 + j];
  Vec<double, 6> m;
  Mat<double, 6, 6> bc;
  if (!correctedFreeToBound(f, C, s, m, bc)) return 0;
  put6(mean, m);
  put36(cov, bc);
  return 1;
}

// Interactions.cpp entry points for the material known-answer tests.
// slab: thickness, X0, L0, Ar, Z, molarRho (mol/mm^3); which: 0 Bethe,
// 1 Landau (most probable), 2 Landau sigma(q/p), 3 theta0, 4 Landau FWHM.
float kfo_interaction(int which, float thickness, float X0, float L0, float Ar, float Z,
                      float molarRho, int absPdg, float m, float qOverP, float absQ) {
  ck_surface cs{};
  cs.mat_thickness = thickness;
  cs.mat_x0 = X0;
  cs.mat_l0 = L0;
  cs.mat_ar = Ar;
  cs.mat_z = Z;
  cs.mat_molar_rho = molarRho;
  cs.mat_molar_electron_rho = Z * molarRho;
  cs.mat_mean_excitation = (float)(lit_eV(16.0L) * std::pow(Z, 0.9f));
  Slab s = Slab::make(cs);
  MatConst C = MatConst::make();
  switch (which) {
    case 0:
      return computeEnergyLossBethe(C, s, m, qOverP, absQ);
    case 1:
      return computeEnergyLossLandau(C, s, m, qOverP, absQ);
    case 2:
      return computeEnergyLossLandauSigmaQOverP(C, s, m, qOverP, absQ);
    case 3:
      return computeMultipleScatteringTheta0(C, s, absPdg, m, qOverP, absQ);
    case 4: {
      RelQ rq(m, qOverP, absQ);
      return computeEnergyLossLandauFwhm(C, s, rq);
    }
    default:
      return 0.0f;
  }
}

// Material effects for a surface slab scaled by `scale` (as the fitter's
// pathCorrection * split factor); returns eLoss, varPhi, varTheta, varQoP.
void kfo_material_effects(const ck_surface* cs, float scale, const double* dir, double qop,
                          float mass, float absQ, int pdg, int ms, int el, double* outv) {
  Slab s = Slab::make(*cs);
  s.scaleThickness(scale);
  V3<double> d{{dir[0], dir[1], dir[2]}};
  MatEffects e = computeMaterialEffects<double>(MatConst::make(), s, pdg, mass, absQ, d,
                                                (float)qop, ms != 0, el != 0);
  outv[0] = e.eLoss;
  outv[1] = e.variancePhi;
  outv[2] = e.varianceTheta;
  outv[3] = e.varianceQoverP;
}

// Field lookup (status 0 ok, CK_TRACK_FIELD_OUT_OF_BOUNDS otherwise).
void kfo_field_lookup(const ck_field* f, int n, const double* pos, double* outB, int* status) {
  Field<double> F = Field<double>::make(*f);
  for (int i = 0; i < n; ++i) {
    V3<double> p{{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}}, b;
    bool ok = F.get(p, b);
    status[i] = ok ? 0 : CK_TRACK_FIELD_OUT_OF_BOUNDS;
    for (int c = 0; c < 3; ++c) outB[3 * i + c] = ok ? b[c] : 0.0;
  }
}

// The propagation restatement on a batch in ck_propagate's layout (inputs
// per track, outputs [c * n + t]); host arrays; the options' stepper fields.
void kfo_propagate(const ck_options* opt, int n_surfaces, const ck_surface* surfaces,
                   const ck_field* field, const ck_propagate_in* in, ck_propagate_out* out,
                   int n_threads) {
  std::vector<Surface<double>> sf;
  for (int i = 0; i < n_surfaces; ++i) sf.push_back(Surface<double>::fromCk(surfaces[i]));
  const Field<double> F = Field<double>::make(*field);
  const Options o = Options::fromCk(*opt, false);
  const int n = in->n;
  std::atomic<int> next{0};
  auto worker = [&]() {
    while (true) {
      const int t = next.fetch_add(1);
      if (t >= n) break;
      const Surface<double> start = Surface<double>::plane(in->start_frames + 12 * (size_t)t);
      const Vec<double, 6> p = get6<double>(in->start_params + 6 * (size_t)t);
      Mat<double, 6, 6> c = Mat<double, 6, 6>::zero();
      if (in->start_cov) c = get36<double>(in->start_cov + 36 * (size_t)t);
      const int tg = in->target ? in->target[t] : -1;
      PropResult r;
      if (tg < -1 || tg >= n_surfaces) {
        r.status = CK_TRACK_INVALID_INPUT;
      } else {
        r = propagate(F, o, start, p, c, in->particle[2 * (size_t)t], in->particle[2 * (size_t)t + 1],
                      tg >= 0 ? &sf[tg] : nullptr, in->path_limit[t]);
      }
      out->status[t] = r.status;
      if (r.status != CK_TRACK_OK) continue;
      for (int i = 0; i < 6; ++i) out->end_params[(size_t)i * n + t] = r.params[i];
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
          if (out->end_cov) out->end_cov[(size_t)(i * 6 + j) * n + t] = r.cov.a[i][j];
          if (out->jacobian) out->jacobian[(size_t)(i * 6 + j) * n + t] = r.jacobian.a[i][j];
        }
      if (out->end_frames && tg < 0)
        for (int i = 0; i < 12; ++i) out->end_frames[12 * (size_t)t + i] = r.frame[i];
      if (out->path_length) out->path_length[t] = r.pathLength;
      if (out->steps) out->steps[t] = r.steps;
    }
  };
  if (n_threads <= 1) {
    worker();
  } else {
    std::vector<std::thread> th;
    for (int i = 0; i < n_threads; ++i) th.emplace_back(worker);
    for (auto& x : th) x.join();
  }
}

// The track-finding restatement on host arrays in ck_find_tracks's layout.
void kfo_find_tracks(const ck_options* opt, int n_surfaces, const ck_surface* surfaces,
                     const ck_field* field, const ck_ckf_options* ck, const ck_ckf_in* in,
                     ck_ckf_out* out, int n_threads) {
  Ctx ctx;
  for (int i = 0; i < n_surfaces; ++i) ctx.surfaces.push_back(Surface<double>::fromCk(surfaces[i]));
  ctx.fitter.surfaces = &ctx.surfaces;
  ctx.fitter.field = Field<double>::make(*field);
  ctx.fitter.mc = MatConst::make();
  ctx.fitter.o = Options::fromCk(*opt, true);
  using F = Fitter<double>;
  F::CkfCuts cuts{ck->chi2_cut,        ck->chi2_cut_outlier, ck->max_candidates,
                  ck->min_measurements, ck->max_holes,        ck->max_outliers,
                  ck->max_holes_and_outliers, ck->target_surface, ck->max_states,
                  ck->max_tracks,      ck->max_branches, ck->end_of_world != 0,
                  0.0,                 0.0,                  0.0};
  if (ck->target_surface >= 0 && ck->target_surface < n_surfaces) {
    const ck_surface& t = surfaces[ck->target_surface];
    cuts.targetHalfX = t.half_x;
    cuts.targetHalfY = t.half_y;
    cuts.targetHalfZ = t.half_length_z;
  }
  F::CkfMeas M{in->surf_meas_offsets, in->meas_values, in->meas_cov, in->meas_subspace};
  const int n = in->n_seeds, S = ck->max_states, T = ck->max_tracks;
  std::atomic<int> next{0};
  auto worker = [&]() {
    std::vector<F::CkfState> states;
    std::vector<F::CkfBranch> tracks;
    while (true) {
      const int s = next.fetch_add(1);
      if (s >= n) break;
      int st = CK_TRACK_OK;
      const int ev = in->seed_event ? in->seed_event[s] : 0;
      if (ev < 0 || ev >= std::max(in->n_events, 1)) st = CK_TRACK_INVALID_INPUT;
      F::CkfMeas Me = M;  // the seed's event's measurements
      Me.offsets = in->surf_meas_offsets + (size_t)std::max(ev, 0) * n_surfaces;
      for (int k = in->seq_offsets[s]; k < in->seq_offsets[s + 1]; ++k) {
        const int sid = in->seq_surfaces[k];
        if (sid < 0 || sid >= n_surfaces || ctx.surfaces[sid].type == CK_SURFACE_LINE)
          st = CK_TRACK_INVALID_INPUT;
      }
      states.clear();
      tracks.clear();
      if (st == CK_TRACK_OK) {
        const Surface<double> start = Surface<double>::plane(in->start_frames + 12 * (size_t)s);
        st = ctx.fitter.ckfSeed(start, get6<double>(in->start_params + 6 * (size_t)s),
                                get36<double>(in->start_cov + 36 * (size_t)s),
                                in->particle[2 * (size_t)s], in->particle[2 * (size_t)s + 1],
                                in->particle_pdg ? in->particle_pdg[s] : 211,
                                in->seq_surfaces + in->seq_offsets[s],
                                in->seq_offsets[s + 1] - in->seq_offsets[s], Me, cuts, states,
                                tracks);
      }
      out->status[s] = st;
      out->n_tracks[s] = st == CK_TRACK_OK ? (int)tracks.size() : 0;
      out->n_states[s] = st == CK_TRACK_OK ? (int)states.size() : 0;
      if (st != CK_TRACK_OK) continue;
      for (int k = 0; k < (int)tracks.size(); ++k) {
        const F::CkfBranch& b = tracks[k];
        const size_t i = (size_t)s * T + k;
        out->track_tip[i] = b.tip;
        out->track_n_measurements[i] = b.nMeas;
        out->track_n_holes[i] = b.nHoles;
        out->track_n_outliers[i] = b.nOutliers;
        out->track_ndf[i] = b.ndf;
        out->track_chi2[i] = b.chi2;
        for (int c = 0; c < 6; ++c)
          out->track_params[i * 6 + c] = b.hasParams ? b.params[c] : std::nan("");
        for (int r = 0, c = 0; r < 6; ++r)
          for (int q = r; q < 6; ++q, ++c)
            out->track_cov[i * 21 + c] = b.hasParams ? b.cov.a[r][q] : std::nan("");
      }
      for (int k = 0; k < (int)states.size(); ++k) {
        const F::CkfState& x = states[k];
        const size_t i = (size_t)s * S + k;
        out->state_prev[i] = x.prev;
        out->state_surface[i] = x.surface;
        out->state_flags[i] = x.flags;
        out->state_measurement[i] = x.meas;
        out->state_chi2[i] = x.chi2;
        out->state_path_length[i] = x.pathLength;
        for (int c = 0; c < 6; ++c) {
          out->predicted[i * 6 + c] = x.pred[c];
          out->filtered[i * 6 + c] = x.filt[c];
        }
        for (int r = 0, c = 0; r < 6; ++r)
          for (int q = r; q < 6; ++q, ++c) {
            out->predicted_cov[i * 21 + c] = x.predCov.a[r][q];
            out->filtered_cov[i * 21 + c] = x.filtCov.a[r][q];
          }
        for (int r = 0; r < 6; ++r)
          for (int q = 0; q < 6; ++q) out->jacobian[i * 36 + r * 6 + q] = x.jac.a[r][q];
      }
    }
  };
  if (n_threads <= 1) {
    worker();
  } else {
    std::vector<std::thread> th;
    for (int i = 0; i < n_threads; ++i) th.emplace_back(worker);
    for (auto& x : th) x.join();
  }
}

// Counts how often glibc logf differs from the correctly rounded float
// logarithm used by both implementations, over n inputs.
int kfo_logf_mismatch(int n, const float* x) {
  int bad = 0;
  for (int i = 0; i < n; ++i)
    if (std::log(x[i]) != ck_logf(x[i])) ++bad;
  return bad;
}

int kfo_hardware_threads() { return (int)std::thread::hardware_concurrency(); }

}  // extern "C"
