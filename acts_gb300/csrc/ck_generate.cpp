// ck_generate.cpp — synthetic detector, field and track generator.
//
// Builds the inputs of the five benchmark workloads: the surface tables,
// the field map and, per track, the truth simulation of ck_simulate.h (run
// here on host threads; ck_simulate.cu runs the same source on the GPU).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "ck_simulate.h"
#include "ckgen.h"

using cks::basePreset;
using cks::mix;
using cks::Rng;

namespace {

// ------------------------------------------------------------- geometry
void setIdentity(ck_surface& s) {
  std::memset(s.rotation, 0, sizeof(s.rotation));
  s.rotation[0] = s.rotation[4] = s.rotation[8] = 1.0;
}

void setSilicon(ck_surface& s, float thickness) {
  // Silicon as in Tests/CommonHelpers/.../PredefinedMaterials.hpp:23-27:
  // X0 = 9.370 cm, L0 = 46.52 cm, Ar = 28.0855, Z = 14, rho = 2.329 g/cm3
  s.mat_thickness = thickness;
  s.mat_x0 = (float)93.70;
  s.mat_l0 = (float)465.2;
  s.mat_ar = (float)28.0855;
  s.mat_z = 14.0f;
  s.mat_molar_rho = (float)((2.329 / 28.0855) * 1.0 / 1000.0);
  s.mat_molar_electron_rho = s.mat_z * s.mat_molar_rho;
  // approximateMeanExcitationEnergy: 16 eV * Z^0.9 (Material.cpp:34-39)
  s.mat_mean_excitation = (float)(16 * 1e-9 * std::pow(s.mat_z, 0.9f));
  s.split_factor = 1.0f;
  s.flags |= CK_SURF_MATERIAL;
}

const double kBarrelRadii[10] = {32, 72, 116, 172, 260, 360, 500, 660, 820, 1020};

int barrelRadii(int preset, double* r) {
  if (preset == CKG_UNEVEN || preset == CKG_SERVING) {
    // the ten radii plus ten midpoints (the first between the beam line and
    // the innermost layer)
    int n = 0;
    double prev = 0;
    for (int i = 0; i < 10; ++i) {
      r[n++] = 0.5 * (prev + kBarrelRadii[i]);
      r[n++] = kBarrelRadii[i];
      prev = kBarrelRadii[i];
    }
    return n;
  }
  for (int i = 0; i < 10; ++i) r[i] = kBarrelRadii[i];
  return 10;
}

// Solenoid-like synthetic map: Bz = 2 T (1 + (z / 2.5 m)^2)^-1.5 for
// r < 1.2 m, falling linearly to 0 at r = 1.5 m; Br from div B = 0.
void gridFieldAt(double x, double y, double z, double* B) {
  const double a = 2500.0;
  const double u = 1.0 + (z / a) * (z / a);
  const double f = 2.0 * std::pow(u, -1.5);
  const double dfdz = 2.0 * (-1.5) * std::pow(u, -2.5) * (2.0 * z / (a * a));
  const double r = std::sqrt(x * x + y * y);
  double g, integ;  // g(r) and int_0^r r' g(r') dr'
  if (r < 1200.0) {
    g = 1.0;
    integ = 0.5 * r * r;
  } else if (r < 1500.0) {
    g = (1500.0 - r) / 300.0;
    auto prim = [](double s) { return (1500.0 * s * s / 2.0 - s * s * s / 3.0) / 300.0; };
    integ = 0.5 * 1200.0 * 1200.0 + prim(r) - prim(1200.0);
  } else {
    g = 0.0;
    auto prim = [](double s) { return (1500.0 * s * s / 2.0 - s * s * s / 3.0) / 300.0; };
    integ = 0.5 * 1200.0 * 1200.0 + prim(1500.0) - prim(1200.0);
  }
  const double Bz = f * g;
  double Br = (r > 0) ? -dfdz * integ / r : 0.0;
  B[0] = (r > 0) ? Br * x / r : 0.0;
  B[1] = (r > 0) ? Br * y / r : 0.0;
  B[2] = Bz;
}

// a track's rows, collected from the simulation
struct TrackRows {
  std::vector<int> seq, measSurf;
  std::vector<double> measVal, measCov, truth;
  std::vector<uint8_t> outlier;
  std::vector<int32_t> measSub;
  cks::TrackHeader hdr;
  void onSurface(int sid) { seq.push_back(sid); }
  void onMeasurement(int sid, int sub, const double* val, const double* cov, const double* tr, bool outl) {
    measSurf.push_back(sid);
    measSub.push_back(sub);
    measVal.push_back(val[0]);
    measVal.push_back(val[1]);
    for (int c = 0; c < 4; ++c) measCov.push_back(cov[c]);
    for (int c = 0; c < 6; ++c) truth.push_back(tr[c]);
    outlier.push_back(outl ? 1 : 0);
  }
};

}  // namespace

extern "C" {

int32_t ckg_geometry(int32_t preset, ck_surface* out, int32_t cap) {
  preset = basePreset(preset);
  std::vector<ck_surface> v;
  if (preset == CKG_TELESCOPE) {
    for (int i = 0; i < 10; ++i) {
      ck_surface s{};
      s.type = CK_SURFACE_PLANE;
      s.flags = CK_SURF_SENSITIVE;
      // local x = global y, local y = global z, normal = global x
      std::memset(s.rotation, 0, sizeof(s.rotation));
      s.rotation[0 * 3 + 2] = 1.0;
      s.rotation[1 * 3 + 0] = 1.0;
      s.rotation[2 * 3 + 1] = 1.0;
      s.center[0] = 30.0 * (i + 1);
      s.half_x = s.half_y = 250.0;
      s.split_factor = 1.0f;
      v.push_back(s);
    }
  } else if (preset >= CKG_BARREL && preset <= CKG_SERVING) {
    double r[20];
    int n = barrelRadii(preset, r);
    for (int i = 0; i < n; ++i) {
      ck_surface s{};
      s.type = CK_SURFACE_CYLINDER;
      s.flags = CK_SURF_SENSITIVE;
      setIdentity(s);
      s.radius = r[i];
      s.half_length_z = 1500.0;
      setSilicon(s, 0.3f);
      v.push_back(s);
    }
  } else {
    return -1;
  }
  int n = std::min<int>((int)v.size(), cap);
  for (int i = 0; i < n; ++i) out[i] = v[i];
  return n;
}

int64_t ckg_field_values(int32_t preset) {
  preset = basePreset(preset);
  if (preset == CKG_UNEVEN || preset == CKG_SERVING) return (int64_t)151 * 151 * 301 * 3;
  return 0;
}

void ckg_field(int32_t preset, float* values, ck_field* out, int32_t n_threads) {
  preset = basePreset(preset);
  std::memset(out, 0, sizeof(*out));
  if (preset != CKG_UNEVEN && preset != CKG_SERVING) {
    out->kind = CK_FIELD_CONSTANT;
    out->constant_tesla[2] = 2.0;
    return;
  }
  out->kind = CK_FIELD_GRID_XYZ;
  const int n[3] = {151, 151, 301};
  const double mn[3] = {-1500.0, -1500.0, -3000.0}, mx[3] = {1500.0, 1500.0, 3000.0};
  for (int i = 0; i < 3; ++i) {
    out->n[i] = n[i];
    out->min[i] = mn[i];
    out->max[i] = mx[i];
  }
  out->values_tesla = values;
  if (n_threads < 1) n_threads = 1;
  auto work = [&](int t) {
    for (int ix = t; ix < n[0]; ix += n_threads)
      for (int iy = 0; iy < n[1]; ++iy)
        for (int iz = 0; iz < n[2]; ++iz) {
          double x = mn[0] + ix * (mx[0] - mn[0]) / (n[0] - 1);
          double y = mn[1] + iy * (mx[1] - mn[1]) / (n[1] - 1);
          double z = mn[2] + iz * (mx[2] - mn[2]) / (n[2] - 1);
          double B[3];
          gridFieldAt(x, y, z, B);
          size_t id = ((size_t)ix * n[1] + iy) * n[2] + iz;
          for (int c = 0; c < 3; ++c) values[id * 3 + c] = (float)B[c];
        }
  };
  std::vector<std::thread> th;
  for (int t = 0; t < n_threads; ++t) th.emplace_back(work, t);
  for (auto& x : th) x.join();
}

int64_t ckg_generate(int32_t preset, uint64_t seed, int64_t first_track, int32_t n_tracks,
                     const ck_surface* surfaces, int32_t n_surfaces, const ck_field* field,
                     int32_t n_threads, ckg_out* out) {
  if (!surfaces || !field || !out || n_tracks < 0) return -1;
  std::vector<ck_surface> surf(surfaces, surfaces + n_surfaces);
  cks::FieldEval F;
  F.kind = field->kind;
  for (int i = 0; i < 3; ++i) F.b[i] = field->constant_tesla[i];
  if (F.kind == CK_FIELD_GRID_XYZ) {
    for (int i = 0; i < 3; ++i) {
      F.n[i] = field->n[i];
      F.mn[i] = field->min[i];
      F.step[i] = (field->max[i] - field->min[i]) / (F.n[i] - 1);
    }
    F.v = field->values_tesla;
    F.stride = 3;
  }
  std::vector<TrackRows> rows(n_tracks);
  if (n_threads < 1) n_threads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < n_threads; ++t)
    th.emplace_back([&, t]() {
      for (int i = t; i < n_tracks; i += n_threads)
        cks::simulateTrack(preset, seed, first_track + i, surf.data(), (int)surf.size(), F,
                           rows[i].hdr, rows[i]);
    });
  for (auto& x : th) x.join();
  int64_t ns = 0, nm = 0;
  out->seq_offsets[0] = 0;
  out->meas_offsets[0] = 0;
  const int cap = out->max_per_track;
  for (int i = 0; i < n_tracks; ++i) {
    TrackRows& r = rows[i];
    int nseq = std::min<int>((int)r.seq.size(), cap);
    int nmeas = std::min<int>((int)r.measSurf.size(), cap);
    for (int k = 0; k < nseq; ++k) out->seq_surfaces[ns + k] = r.seq[k];
    for (int k = 0; k < nmeas; ++k) {
      out->meas_surfaces[nm + k] = r.measSurf[k];
      for (int c = 0; c < 2; ++c) out->meas_values[2 * (nm + k) + c] = r.measVal[2 * k + c];
      for (int c = 0; c < 4; ++c) out->meas_cov[4 * (nm + k) + c] = r.measCov[4 * k + c];
      if (out->truth_meas)
        for (int c = 0; c < 6; ++c) out->truth_meas[6 * (nm + k) + c] = r.truth[6 * k + c];
      if (out->meas_outlier) out->meas_outlier[nm + k] = r.outlier[k];
      if (out->meas_subspace) out->meas_subspace[nm + k] = r.measSub[k];
    }
    ns += nseq;
    nm += nmeas;
    out->seq_offsets[i + 1] = (int32_t)ns;
    out->meas_offsets[i + 1] = (int32_t)nm;
    const cks::TrackHeader& hd = r.hdr;
    std::memcpy(out->start_params + 6 * (size_t)i, hd.startParams, sizeof(hd.startParams));
    std::memcpy(out->start_cov + 36 * (size_t)i, hd.startCov, sizeof(hd.startCov));
    std::memcpy(out->start_frames + 12 * (size_t)i, hd.frame, sizeof(hd.frame));
    if (out->truth_start)
      std::memcpy(out->truth_start + 6 * (size_t)i, hd.truthStart, sizeof(hd.truthStart));
    out->particle[2 * i] = hd.particle[0];
    out->particle[2 * i + 1] = hd.particle[1];
    out->particle_pdg[i] = hd.pdg;
  }
  return nm;
}

void ckg_event_sizes(uint64_t seed, int32_t n_events, double mean, int32_t lo, int32_t hi,
                     int32_t* sizes) {
  for (int e = 0; e < n_events; ++e) {
    Rng rng(mix(seed ^ 0x5EED5EEDull, (uint64_t)e));
    if (mean > 0) {
      // Poisson(mean) as a sum of Poisson(mean/k) draws by Knuth's method
      int chunks = (int)std::ceil(mean / 20.0);
      double lam = mean / chunks;
      const double L = std::exp(-lam);
      int64_t total = 0;
      for (int c = 0; c < chunks; ++c) {
        int k = 0;
        double p = 1.0;
        do {
          ++k;
          p *= rng.uniform();
        } while (p > L);
        total += k - 1;
      }
      sizes[e] = (int32_t)total;
    } else {
      double x = std::exp(rng.uniform(std::log((double)lo), std::log((double)hi)));
      sizes[e] = std::max(lo, std::min(hi, (int32_t)std::lround(x)));
    }
  }
}

}  // extern "C"
