// ck_simulate.h — the truth simulation of one generated track, shared by the
// host generator (ck_generate.cpp, one thread per track) and the device
// generator (ck_simulate.cu, one CUDA thread per track): the same source
// evaluates the same expressions on both.
//
// A fixed-step RK4 integration of the Lorentz force with crossing
// refinement, Highland multiple-scattering kicks and mean Bethe energy loss
// at each silicon layer (the roles Fatras plays for the reference's
// truth-tracking examples, Fatras/include/ActsFatras/Kernel/
// SingleParticleSimulation.hpp:34-67), then Gaussian smearing of the local
// hit positions (digitisation) and of the start parameters.
//
// Random numbers: SplitMix64 (G. Steele, D. Lea, C. Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) seeded per track, uniform
// doubles from the top 53 bits, Gaussians by the Box-Muller transform.
#pragma once

#include <cmath>
#include <cstdint>

#include "ckgen.h"

#ifdef __CUDACC__
#define CKS_HD __host__ __device__ inline
#else
#define CKS_HD inline
#endif

namespace cks {

constexpr double kPi = 3.14159265358979323846;
constexpr double kT = 0.000299792458;  // 1 T in GeV/(e mm)
constexpr double kNs = 299.792458;     // 1 ns in mm/c
constexpr double kMuonMass = 0.1056583755;
constexpr double kPionMass = 0.13957039;

struct Rng {
  uint64_t s;
  CKS_HD explicit Rng(uint64_t seed) : s(seed) {}
  CKS_HD uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  CKS_HD double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  CKS_HD double uniform(double a, double b) { return a + (b - a) * uniform(); }
  CKS_HD double gauss() {
    double u1 = uniform();
    double u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return sqrt(-2.0 * log(u1)) * cos(2.0 * kPi * u2);
  }
};

CKS_HD uint64_t mix(uint64_t a, uint64_t b) {
  Rng r(a ^ (b * 0xD6E8FEB86659FD93ull));
  r.next();
  return r.next();
}

// the geometry / field / kinematics preset a preset shares
CKS_HD int basePreset(int preset) { return preset == CKG_STRIPS ? CKG_BARREL : preset; }

// The field in GeV/(e mm): constant, or the plain trilinear interpolation of
// a grid whose node c-th component is v[node * stride + c] (stride 3 for the
// generator's float triplets, 4 for the fitter's device float4 nodes)
struct FieldEval {
  int kind = CK_FIELD_CONSTANT;
  double b[3] = {0, 0, 0};  // Tesla
  int n[3] = {0, 0, 0};
  double mn[3] = {0, 0, 0}, step[3] = {1, 1, 1};
  const float* v = nullptr;
  int stride = 3;
  CKS_HD void get(const double* p, double* out) const {
    if (kind == CK_FIELD_CONSTANT) {
      for (int i = 0; i < 3; ++i) out[i] = b[i] * kT;
      return;
    }
    int idx[3];
    double f[3];
    for (int i = 0; i < 3; ++i) {
      double u = (p[i] - mn[i]) / step[i];
      int k = (int)floor(u);
      k = (n[i] - 2 < k) ? n[i] - 2 : k;  // (std::max(0, std::min(k, n - 2)))
      k = (0 < k) ? k : 0;
      idx[i] = k;
      const double fu = u - k;
      const double lo = (0.0 < fu) ? fu : 0.0;  // (std::min(1.0, std::max(0.0, fu)))
      f[i] = (lo < 1.0) ? lo : 1.0;
    }
    for (int c = 0; c < 3; ++c) {
      double acc = 0;
      for (int corner = 0; corner < 8; ++corner) {
        int dx = (corner >> 2) & 1, dy = (corner >> 1) & 1, dz = corner & 1;
        double w = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
        size_t id = ((size_t)(idx[0] + dx) * n[1] + (idx[1] + dy)) * n[2] + (idx[2] + dz);
        acc += w * v[id * stride + c];
      }
      out[c] = acc * kT;
    }
  }
};

// --------------------------------------------------------- truth physics
struct Particle {
  int pdg;
  double mass;
  double q;
};

// Highland formula (PDG review, passage of particles through matter)
CKS_HD double highlandTheta0(double xOverX0, double p, double beta) {
  if (xOverX0 <= 0) return 0;
  return 13.6e-3 / (beta * p) * sqrt(xOverX0) * (1.0 + 0.038 * log(xOverX0 / (beta * beta)));
}

// Mean Bethe energy loss (PDG review eq. 34.5 form, no shell correction)
CKS_HD double betheLoss(const ck_surface& s, double thick, double m, double p) {
  const double me = 0.5109989461e-3;
  const double K = 0.307075e-3 * 100.0;  // GeV mm^2 / mol
  const double E = sqrt(m * m + p * p);
  const double beta2 = p * p / (E * E);
  const double bg = p / m;
  const double gamma = E / m;
  const double I = s.mat_mean_excitation;
  const double Ne = s.mat_molar_electron_rho;
  const double wmax = 2 * me * bg * bg / (1 + 2 * gamma * me / m + (me / m) * (me / m));
  double delta = 0;
  if (bg >= 10.0) {
    const double plasma = 28.816e-9 * sqrt(Ne * 1000.0);
    delta = 2.0 * (log(bg) + log(plasma / I) - 0.5);
  }
  const double eps = 0.5 * K * Ne * thick / beta2;
  return eps * (log(2 * me * bg * bg / I) + log(wmax / I) - 2 * beta2 - delta);
}

struct TState {
  double pos[3], dir[3];
  double p, t;
};

CKS_HD void rhs(const FieldEval& F, double qop, const double* pos, const double* dir,
                double* dpos, double* ddir) {
  double B[3];
  F.get(pos, B);
  for (int i = 0; i < 3; ++i) dpos[i] = dir[i];
  ddir[0] = qop * (dir[1] * B[2] - dir[2] * B[1]);
  ddir[1] = qop * (dir[2] * B[0] - dir[0] * B[2]);
  ddir[2] = qop * (dir[0] * B[1] - dir[1] * B[0]);
}

CKS_HD TState rk4(const FieldEval& F, const Particle& pa, const TState& s, double h) {
  const double qop = pa.q / s.p;
  double k1p[3], k1d[3], k2p[3], k2d[3], k3p[3], k3d[3], k4p[3], k4d[3], pp[3], dd[3];
  rhs(F, qop, s.pos, s.dir, k1p, k1d);
  for (int i = 0; i < 3; ++i) {
    pp[i] = s.pos[i] + 0.5 * h * k1p[i];
    dd[i] = s.dir[i] + 0.5 * h * k1d[i];
  }
  rhs(F, qop, pp, dd, k2p, k2d);
  for (int i = 0; i < 3; ++i) {
    pp[i] = s.pos[i] + 0.5 * h * k2p[i];
    dd[i] = s.dir[i] + 0.5 * h * k2d[i];
  }
  rhs(F, qop, pp, dd, k3p, k3d);
  for (int i = 0; i < 3; ++i) {
    pp[i] = s.pos[i] + h * k3p[i];
    dd[i] = s.dir[i] + h * k3d[i];
  }
  rhs(F, qop, pp, dd, k4p, k4d);
  TState o = s;
  double n2 = 0;
  for (int i = 0; i < 3; ++i) {
    o.pos[i] = s.pos[i] + h / 6.0 * (k1p[i] + 2 * k2p[i] + 2 * k3p[i] + k4p[i]);
    o.dir[i] = s.dir[i] + h / 6.0 * (k1d[i] + 2 * k2d[i] + 2 * k3d[i] + k4d[i]);
    n2 += o.dir[i] * o.dir[i];
  }
  const double n = sqrt(n2);
  for (int i = 0; i < 3; ++i) o.dir[i] /= n;
  const double E = sqrt(pa.mass * pa.mass + s.p * s.p);
  o.t = s.t + h * E / s.p;
  return o;
}

// signed distance of a point to a surface of the ordered detector
CKS_HD double sdist(const ck_surface& s, const double* p) {
  if (s.type == CK_SURFACE_CYLINDER) return sqrt(p[0] * p[0] + p[1] * p[1]) - s.radius;
  double d = 0;
  for (int i = 0; i < 3; ++i) d += s.rotation[i * 3 + 2] * (p[i] - s.center[i]);
  return d;
}

CKS_HD void toLocal(const ck_surface& s, const double* p, double* loc) {
  double d[3], l[3];
  for (int i = 0; i < 3; ++i) d[i] = p[i] - s.center[i];
  for (int j = 0; j < 3; ++j)
    l[j] = s.rotation[0 * 3 + j] * d[0] + s.rotation[1 * 3 + j] * d[1] + s.rotation[2 * 3 + j] * d[2];
  if (s.type == CK_SURFACE_CYLINDER) {
    loc[0] = s.radius * atan2(l[1], l[0]);
    loc[1] = l[2];
  } else {
    loc[0] = l[0];
    loc[1] = l[1];
  }
}

CKS_HD double cosIncidence(const ck_surface& s, const double* p, const double* dir) {
  double n[3];
  if (s.type == CK_SURFACE_CYLINDER) {
    double r = sqrt(p[0] * p[0] + p[1] * p[1]);
    n[0] = p[0] / r;
    n[1] = p[1] / r;
    n[2] = 0;
  } else {
    for (int i = 0; i < 3; ++i) n[i] = s.rotation[i * 3 + 2];
  }
  return fabs(n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2]);
}

CKS_HD bool inBounds(const ck_surface& s, const double* p) {
  if (s.type == CK_SURFACE_CYLINDER) return fabs(p[2]) < s.half_length_z;
  double loc[2];
  toLocal(s, p, loc);
  return fabs(loc[0]) < s.half_x && fabs(loc[1]) < s.half_y;
}

// kinematics and detector response of a preset
struct Preset {
  Particle pa;
  double sigma0, sigma1;
  int minHits, maxHits;
  double holeProb, outlierProb, outlierSigma;
  bool barrel;
};

CKS_HD Preset presetOf(int preset) {
  Preset p{};
  if (preset == CKG_TELESCOPE) {
    p.pa = {13, kMuonMass, 1};
    p.sigma0 = p.sigma1 = 0.050;
    p.minHits = p.maxHits = 0;
    p.barrel = false;
  } else {
    p.pa = {211, kPionMass, 1};
    p.sigma0 = 0.020;
    p.sigma1 = 0.050;
    p.barrel = true;
    if (preset == CKG_UNEVEN || preset == CKG_SERVING) {
      p.minHits = 4;
      p.maxHits = 20;
      p.holeProb = 0.1;
      p.outlierProb = 0.05;
      p.outlierSigma = 10.0;
    }
  }
  return p;
}

// the per-track results that are not rows
struct TrackHeader {
  double startParams[6], startCov[36], frame[12], truthStart[6];
  float particle[2];
  int pdg;
};

// Simulates track `id` of a preset through the ordered surfaces. `sink`
// receives the sequence (sink.onSurface(surface)) and the measurements
// (sink.onMeasurement(surface, subspace, value[2], covariance[4], truth[6],
// outlier)).
template <class Sink>
CKS_HD void simulateTrack(int preset, uint64_t seed, int64_t id, const ck_surface* surf,
                          int nSurf, const FieldEval& F, TrackHeader& out, Sink& sink) {
  const bool stripPreset = preset == CKG_STRIPS;
  preset = basePreset(preset);
  Preset P = presetOf(preset);
  Rng rng(mix(seed, (uint64_t)id * 0x2545F4914F6CDD1Dull + (uint64_t)preset));
  Particle pa = P.pa;
  pa.q = (rng.uniform() < 0.5) ? -1.0 : 1.0;
  double pT, eta, phi, vz = 0;
  if (preset == CKG_TELESCOPE) {
    pT = rng.uniform(1.0, 10.0);
    phi = rng.uniform(-0.1, 0.1);
    eta = rng.uniform(-0.1, 0.1);
  } else {
    eta = rng.uniform(-1.5, 1.5);
    phi = rng.uniform(-kPi, kPi);
    pT = exp(rng.uniform(log(0.5), log(100.0)));
    vz = 50.0 * rng.gauss();
  }
  const double theta = 2.0 * atan(exp(-eta));
  TState s;
  s.pos[0] = 0;
  s.pos[1] = 0;
  s.pos[2] = vz;
  s.dir[0] = cos(phi) * sin(theta);
  s.dir[1] = sin(phi) * sin(theta);
  s.dir[2] = cos(theta);
  s.p = pT / sin(theta);
  s.t = 0;
  const double qop0 = pa.q / s.p;

  // curvilinear start frame (CurvilinearSurface.cpp:25-39): U = z x T, V = T x U
  {
    double T[3] = {s.dir[0], s.dir[1], s.dir[2]};
    double U[3] = {-T[1], T[0], 0.0};  // z x T
    double un = sqrt(U[0] * U[0] + U[1] * U[1]);
    for (int i = 0; i < 3; ++i) U[i] /= un;
    double V[3] = {T[1] * U[2] - T[2] * U[1], T[2] * U[0] - T[0] * U[2], T[0] * U[1] - T[1] * U[0]};
    for (int i = 0; i < 3; ++i) {
      out.frame[i * 3 + 0] = U[i];
      out.frame[i * 3 + 1] = V[i];
      out.frame[i * 3 + 2] = T[i];
      out.frame[9 + i] = s.pos[i];
    }
  }
  out.truthStart[0] = 0;
  out.truthStart[1] = 0;
  out.truthStart[2] = phi;
  out.truthStart[3] = theta;
  out.truthStart[4] = qop0;
  out.truthStart[5] = 0;
  // smeared start: 10 um loc, 1 mrad angles, 1 % q/p, 1 ns time
  const double sl = 0.010, sa = 0.001, sq = 0.01 * fabs(qop0), st = kNs;
  out.startParams[0] = sl * rng.gauss();
  out.startParams[1] = sl * rng.gauss();
  double sphi = phi + sa * rng.gauss();
  if (sphi >= kPi) sphi -= 2 * kPi;
  if (sphi < -kPi) sphi += 2 * kPi;
  out.startParams[2] = sphi;
  out.startParams[3] = theta + sa * rng.gauss();
  out.startParams[4] = qop0 * (1.0 + 0.01 * rng.gauss());
  out.startParams[5] = st * rng.gauss();
  for (int i = 0; i < 36; ++i) out.startCov[i] = 0.0;
  out.startCov[0] = sl * sl;
  out.startCov[7] = sl * sl;
  out.startCov[14] = sa * sa;
  out.startCov[21] = sa * sa;
  out.startCov[28] = sq * sq;
  out.startCov[35] = st * st;
  out.particle[0] = (float)pa.mass;
  out.particle[1] = 1.0f;
  out.pdg = pa.pdg;

  int nHitsMax = 1 << 30;
  if (P.maxHits > 0) nHitsMax = P.minHits + (int)(rng.uniform() * (P.maxHits - P.minHits + 1));
  if (nHitsMax > P.maxHits && P.maxHits > 0) nHitsMax = P.maxHits;

  // propagate through the ordered surfaces
  const double h = 5.0;
  int next = 0;
  double path = 0;
  const double maxPath = 20000.0;
  int nCrossed = 0;
  while (next < nSurf && path < maxPath && nCrossed < nHitsMax) {
    if (fabs(s.pos[2]) > 3000.0) break;
    const ck_surface& S = surf[next];
    double d0 = sdist(S, s.pos);
    TState s1 = rk4(F, pa, s, h);
    double d1 = sdist(S, s1.pos);
    if (!(d0 < 0 && d1 >= 0)) {
      // barrel loopers that turn back never reach the next layer
      if (P.barrel) {
        double r0 = hypot(s.pos[0], s.pos[1]), r1 = hypot(s1.pos[0], s1.pos[1]);
        if (r1 < r0 && path > 100.0) break;
      }
      s = s1;
      path += h;
      continue;
    }
    // refine the crossing with the secant (Illinois) method on the step length
    double a = 0, b = h, fa = d0, fb = d1;
    TState sc = s1;
    double cstep = h;
    int side = 0;
    for (int it = 0; it < 60; ++it) {
      double c = (a * fb - b * fa) / (fb - fa);
      cstep = c;
      sc = rk4(F, pa, s, c);
      double fc = sdist(S, sc.pos);
      if (fabs(fc) < 1e-12) {
        a = b = c;
        break;
      }
      if ((fc < 0) == (fa < 0)) {
        a = c;
        fa = fc;
        if (side == -1) fb *= 0.5;
        side = -1;
      } else {
        b = c;
        fb = fc;
        if (side == 1) fa *= 0.5;
        side = 1;
      }
      if (b - a < 1e-13) break;
    }
    path += cstep;
    s = sc;
    const int sid = next;
    ++next;
    if (!inBounds(S, s.pos)) continue;
    ++nCrossed;
    sink.onSurface(sid);
    // truth at the surface
    double loc[2];
    toLocal(S, s.pos, loc);
    const double tphi = atan2(s.dir[1], s.dir[0]);
    const double ttheta = atan2(hypot(s.dir[0], s.dir[1]), s.dir[2]);
    const bool hole = P.holeProb > 0 && rng.uniform() < P.holeProb;
    const bool outl = P.outlierProb > 0 && rng.uniform() < P.outlierProb;
    const double sgn0 = rng.uniform() < 0.5 ? -1.0 : 1.0;
    const double sgn1 = rng.uniform() < 0.5 ? -1.0 : 1.0;
    const double g0 = rng.gauss();
    const double g1 = rng.gauss();
    // strip layers (CKG_STRIPS, layers 4-9): one local coordinate
    int sub = CK_MEAS_LOC01;
    if (stripPreset && sid >= 4) sub = (sid % 2 == 0) ? CK_MEAS_LOC0 : CK_MEAS_LOC1;
    const double truth[6] = {loc[0], loc[1], tphi, ttheta, pa.q / s.p, s.t};
    if (!hole && sub != CK_MEAS_LOC01) {
      const int hh = sub == CK_MEAS_LOC0 ? 0 : 1;
      const double sg = hh == 0 ? 0.100 : 0.150;
      double m = loc[hh] + sg * (hh == 0 ? g0 : g1);
      if (outl) m += (hh == 0 ? sgn0 : sgn1) * P.outlierSigma * sg;
      const double val[2] = {m, 0.0};
      const double cov[4] = {sg * sg, 0.0, 0.0, 0.0};
      sink.onMeasurement(sid, sub, val, cov, truth, outl);
    }
    double m0 = loc[0] + P.sigma0 * g0;
    double m1 = loc[1] + P.sigma1 * g1;
    if (!hole && sub == CK_MEAS_LOC01) {
      if (outl) {
        m0 += sgn0 * P.outlierSigma * P.sigma0;
        m1 += sgn1 * P.outlierSigma * P.sigma1;
      }
      const double val[2] = {m0, m1};
      const double cov[4] = {P.sigma0 * P.sigma0, 0.0, 0.0, P.sigma1 * P.sigma1};
      sink.onMeasurement(sid, sub, val, cov, truth, outl);
    }
    // material: Highland kick and mean Bethe loss
    if (S.flags & CK_SURF_MATERIAL) {
      const double cosA = cosIncidence(S, s.pos, s.dir);
      const double thick = S.mat_thickness / cosA;
      const double E = sqrt(pa.mass * pa.mass + s.p * s.p);
      const double beta = s.p / E;
      const double th0 = highlandTheta0(thick / S.mat_x0, s.p, beta);
      double u[3], v[3];
      {
        const double* T = s.dir;
        double a2[3] = {-T[1], T[0], 0.0};
        double n = hypot(a2[0], a2[1]);
        if (n < 1e-12) {
          a2[0] = 1;
          a2[1] = 0;
          n = 1;
        }
        for (int i = 0; i < 3; ++i) u[i] = a2[i] / n;
        v[0] = T[1] * u[2] - T[2] * u[1];
        v[1] = T[2] * u[0] - T[0] * u[2];
        v[2] = T[0] * u[1] - T[1] * u[0];
      }
      const double k1 = th0 * rng.gauss(), k2 = th0 * rng.gauss();
      double nn = 0;
      for (int i = 0; i < 3; ++i) {
        s.dir[i] += k1 * u[i] + k2 * v[i];
        nn += s.dir[i] * s.dir[i];
      }
      nn = sqrt(nn);
      for (int i = 0; i < 3; ++i) s.dir[i] /= nn;
      const double dE = betheLoss(S, thick, pa.mass, s.p);
      const double E2 = E - dE;
      s.p = (E2 > pa.mass) ? sqrt(E2 * E2 - pa.mass * pa.mass) : 0.01;
    }
  }
}

}  // namespace cks
