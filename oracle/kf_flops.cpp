// kf_flops.cpp — algorithmic operation counts of the Kalman fit (test and
// measurement infrastructure).
//
// Instantiates the oracle's templated fit with a counting scalar that tallies
// every double-precision addition/subtraction, multiplication, division,
// square root and transcendental call the reference formulation performs
// (dense products as written in the reference, 8x8 free transport
// Jacobian). The float material physics is counted separately per call by
// its fixed per-call operation budget. bench.py uses the counts as the
// algorithmic work per track of its roofline.
#include <cmath>
#include <cstdint>

#include "kf_oracle.hpp"

namespace kfo {

struct FlopCounters {
  uint64_t add = 0, mul = 0, div = 0, sqrt = 0, trans = 0, cmp = 0;
};
thread_local FlopCounters g_fc;

struct Flop {
  double v = 0.0;
  Flop() = default;
  Flop(double x) : v(x) {}
  explicit operator double() const { return v; }
  explicit operator float() const { return (float)v; }
  explicit operator int() const { return (int)v; }
};

inline Flop operator+(Flop a, Flop b) {
  ++g_fc.add;
  return Flop(a.v + b.v);
}
inline Flop operator-(Flop a, Flop b) {
  ++g_fc.add;
  return Flop(a.v - b.v);
}
inline Flop operator*(Flop a, Flop b) {
  ++g_fc.mul;
  return Flop(a.v * b.v);
}
inline Flop operator/(Flop a, Flop b) {
  ++g_fc.div;
  return Flop(a.v / b.v);
}
inline Flop operator-(Flop a) { return Flop(-a.v); }
inline bool operator<(Flop a, Flop b) {
  ++g_fc.cmp;
  return a.v < b.v;
}
inline bool operator>(Flop a, Flop b) {
  ++g_fc.cmp;
  return a.v > b.v;
}
inline bool operator<=(Flop a, Flop b) {
  ++g_fc.cmp;
  return a.v <= b.v;
}
inline bool operator>=(Flop a, Flop b) {
  ++g_fc.cmp;
  return a.v >= b.v;
}
inline bool operator==(Flop a, Flop b) { return a.v == b.v; }
inline bool operator!=(Flop a, Flop b) { return a.v != b.v; }
inline Flop sqrt(Flop a) {
  ++g_fc.sqrt;
  return Flop(std::sqrt(a.v));
}
inline Flop abs(Flop a) { return Flop(std::abs(a.v)); }
inline Flop floor(Flop a) { return Flop(std::floor(a.v)); }
inline Flop atan2(Flop a, Flop b) {
  ++g_fc.trans;
  return Flop(std::atan2(a.v, b.v));
}
inline Flop sin(Flop a) {
  ++g_fc.trans;
  return Flop(std::sin(a.v));
}
inline Flop cos(Flop a) {
  ++g_fc.trans;
  return Flop(std::cos(a.v));
}
inline bool isnan(Flop a) { return std::isnan(a.v); }

}  // namespace kfo

using namespace kfo;

extern "C" {

// Fits tracks [first, first+count) of a host batch single-threaded with the
// counting scalar. out: add/sub, mul, div, sqrt, transcendental, compare
// counts (FP64) summed over the tracks; returns the number of tracks fitted
// successfully.
int kfo_count_flops(const ck_options* opt, int n_surfaces, const ck_surface* surfaces,
                    const ck_field* field, const ck_batch_in* in, int first, int count,
                    uint64_t* out) {
  std::vector<Surface<Flop>> surf;
  for (int i = 0; i < n_surfaces; ++i) surf.push_back(Surface<Flop>::fromCk(surfaces[i]));
  Fitter<Flop> f;
  f.surfaces = &surf;
  f.field = Field<Flop>::make(*field);
  f.mc = MatConst::make();
  f.o = Options::fromCk(*opt, opt->early_termination == 0);
  g_fc = FlopCounters();
  int okCount = 0;
  for (int tr = first; tr < first + count && tr < in->n_tracks; ++tr) {
    std::vector<MeasRec<Flop>> meas;
    for (int m = in->meas_offsets[tr]; m < in->meas_offsets[tr + 1]; ++m) {
      MeasRec<Flop> r;
      r.surface = in->meas_surfaces[m];
      r.sub = in->meas_subspace ? in->meas_subspace[m] : CK_MEAS_LOC01;
      r.v[0] = in->meas_values[2 * m];
      r.v[1] = in->meas_values[2 * m + 1];
      for (int c = 0; c < 4; ++c) r.cov[c] = in->meas_cov[4 * m + c];
      meas.push_back(r);
    }
    Surface<Flop> start = Surface<Flop>::plane(in->start_frames + 12 * (size_t)tr);
    Vec<Flop, 6> sp = get6<Flop>(in->start_params + 6 * (size_t)tr);
    Mat<Flop, 6, 6> sc = get36<Flop>(in->start_cov + 36 * (size_t)tr);
    TrackOut t;
    const int s0 = in->seq_offsets[tr], s1 = in->seq_offsets[tr + 1];
    f.fit(start, sp, sc, in->particle[2 * tr], in->particle[2 * tr + 1],
          in->particle_pdg ? in->particle_pdg[tr] : 211, in->seq_surfaces + s0, s1 - s0, meas, t);
    okCount += t.status == CK_TRACK_OK;
  }
  out[0] = g_fc.add;
  out[1] = g_fc.mul;
  out[2] = g_fc.div;
  out[3] = g_fc.sqrt;
  out[4] = g_fc.trans;
  out[5] = g_fc.cmp;
  return okCount;
}

}  // extern "C"
