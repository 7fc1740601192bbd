// Exercises the C++ facade ActsPlugins::CudaKalman the way a reference user
// calls KalmanFitter::fit: per track (iterator range of source links, start
// parameters, options, surface sequence, track container) and batched; and
// CombinatorialKalmanFilter::findTracks over the same event's measurements.
// Exit code 0 on success. Needs a GPU.
#include <cmath>
#include <cstdio>
#include <vector>

#include "ActsPlugins/CudaKalman.hpp"
#include "ckgen.h"

using namespace ActsPlugins;

int main() {
  std::vector<ck_surface> surfaces(32);
  const int ns = ckg_geometry(CKG_TELESCOPE, surfaces.data(), 32);
  surfaces.resize(ns);
  ck_field field{};
  ckg_field(CKG_TELESCOPE, nullptr, &field, 1);

  const int n = 64, cap = 16;
  std::vector<int32_t> so(n + 1), ss(n * cap), mo(n + 1), msf(n * cap), pdg(n);
  std::vector<double> mv(2 * n * cap), mc(4 * n * cap), sp(6 * n), sc(36 * n), fr(12 * n);
  std::vector<float> part(2 * n);
  ckg_out g{};
  g.max_per_track = cap;
  g.seq_offsets = so.data();
  g.seq_surfaces = ss.data();
  g.meas_offsets = mo.data();
  g.meas_surfaces = msf.data();
  g.meas_values = mv.data();
  g.meas_cov = mc.data();
  g.start_params = sp.data();
  g.start_cov = sc.data();
  g.start_frames = fr.data();
  g.particle = part.data();
  g.particle_pdg = pdg.data();
  if (ckg_generate(CKG_TELESCOPE, 17, 0, n, surfaces.data(), ns, &field, 2, &g) < 0) return 2;

  CudaKalman::Config cfg;
  cfg.surfaces = surfaces;
  cfg.field = field;
  CudaKalman fitter(cfg);
  KalmanFitterOptions opts;

  std::vector<TrackInput> inputs(n);
  std::vector<std::vector<SourceLink>> links(n);
  std::vector<std::vector<int>> seqs(n);
  for (int t = 0; t < n; ++t) {
    for (int m = mo[t]; m < mo[t + 1]; ++m) {
      SourceLink sl;
      sl.surface = msf[m];
      sl.value = {mv[2 * m], mv[2 * m + 1]};
      sl.covariance = {mc[4 * m], mc[4 * m + 1], mc[4 * m + 2], mc[4 * m + 3]};
      links[t].push_back(sl);
    }
    for (int k = so[t]; k < so[t + 1]; ++k) seqs[t].push_back(ss[k]);
    BoundTrackParameters start;
    for (int i = 0; i < 6; ++i) start.parameters[i] = sp[6 * t + i];
    for (int i = 0; i < 36; ++i) start.covariance[i] = sc[36 * t + i];
    for (int i = 0; i < 9; ++i) start.planeRotation[i] = fr[12 * t + i];
    for (int i = 0; i < 3; ++i) start.planeCenter[i] = fr[12 * t + 9 + i];
    start.mass = part[2 * t];
    start.absCharge = part[2 * t + 1];
    start.absPdg = pdg[t];
    inputs[t].sourceLinks = links[t].data();
    inputs[t].nSourceLinks = links[t].size();
    inputs[t].start = start;
    inputs[t].surfaceSequence = seqs[t].data();
    inputs[t].nSurfaces = seqs[t].size();
  }

  // per-track calls
  TrackContainer single;
  for (int t = 0; t < n; ++t) {
    Result<size_t> r = fitter.fit(links[t].begin(), links[t].end(), inputs[t].start, opts,
                                  seqs[t], single);
    if (!r.ok()) {
      std::printf("track %d failed: %s\n", t, r.errorName());
      return 1;
    }
  }
  // batched call
  TrackContainer batch;
  std::vector<Result<size_t>> rs = fitter.fitBatch(inputs.data(), n, opts, batch);
  double chi2 = 0;
  size_t ndf = 0;
  for (int t = 0; t < n; ++t) {
    if (!rs[t].ok()) return 3;
    const Track& a = single.tracks[t];
    const Track& b = batch.tracks[rs[t].value()];
    if (a.nMeasurements != 10 || b.nMeasurements != 10 || a.nHoles || a.nOutliers) return 4;
    const TrackState* sa = single.trackStates(t);
    const TrackState* sb = batch.trackStates(rs[t].value());
    for (size_t k = 0; k < a.nStates; ++k)
      for (int i = 0; i < 6; ++i)
        if (sa[k].smoothed[i] != sb[k].smoothed[i]) return 5;  // same inputs -> same bits
    chi2 += b.chi2;
    ndf += b.nDoF;
  }
  // reverse filtering: smoothed parameters on the first and the last
  // measurement state only (TrackStateProxy::hasSmoothed)
  {
    KalmanFitterOptions rev = opts;
    rev.options.reverse_filtering = 1;
    TrackContainer tc;
    std::vector<Result<size_t>> rr = fitter.fitBatch(inputs.data(), n, rev, tc);
    for (int t = 0; t < n; ++t) {
      if (!rr[t].ok()) return 7;
      const Track& tr = tc.tracks[rr[t].value()];
      const TrackState* s = tc.trackStates(rr[t].value());
      size_t first = tr.nStates, last = 0;
      for (size_t k = 0; k < tr.nStates; ++k)
        if (s[k].isMeasurement()) {
          if (first == tr.nStates) first = k;
          last = k;
        }
      for (size_t k = 0; k < tr.nStates; ++k)
        if (s[k].hasSmoothed() != (k == first || k == last)) return 8;
      if (tr.nMeasurements != batch.tracks[rs[t].value()].nMeasurements) return 9;
    }
  }
  // an option outside the declared extension set is rejected, not emulated
  KalmanFitterOptions bad;
  bad.options.smoother = 7;
  bool threw = false;
  try {
    TrackContainer tc;
    fitter.fitBatch(inputs.data(), 1, bad, tc);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  if (!threw) return 6;
  // track finding: every track's start parameters as a seed among all the
  // event's measurements (CombinatorialKalmanFilter::findTracks)
  {
    std::vector<SourceLink> all;
    std::vector<int> owner;
    for (int t = 0; t < n; ++t)
      for (const SourceLink& sl : links[t]) {
        all.push_back(sl);
        owner.push_back(t);
      }
    std::vector<SeedInput> seeds(n);
    for (int t = 0; t < n; ++t) {
      seeds[t].start = inputs[t].start;
      seeds[t].surfaceSequence = seqs[t].data();
      seeds[t].nSurfaces = seqs[t].size();
    }
    CombinatorialKalmanFilterOptions co;
    co.ckf.chi2_cut = 15.0;
    TrackContainer found;
    std::vector<Result<std::vector<size_t>>> fr =
        fitter.findTracks(seeds.data(), n, all.data(), all.size(), co, found);
    size_t own = 0, hits = 0;
    for (int t = 0; t < n; ++t) {
      if (!fr[t].ok() || fr[t].value().size() != 1) return 10;
      const size_t k = fr[t].value()[0];
      const TrackState* st = found.trackStates(k);
      for (size_t i = 0; i < found.tracks[k].nStates; ++i) {
        if (st[i].sourceLink < 0) continue;
        ++hits;
        own += owner[st[i].sourceLink] == t ? 1 : 0;
        if (!(st[i].filteredCovariance[0] > 0) || st[i].hasSmoothed()) return 11;
      }
    }
    if (hits < 9 * static_cast<size_t>(n) || own < hits * 95 / 100) return 12;
    std::printf("findTracks ok: %d seeds, %zu of %zu hits their own\n", n, own, hits);
  }
  std::printf("facade ok: %d tracks, chi2/ndf %.3f\n", n, chi2 / ndf);
  return 0;
}
