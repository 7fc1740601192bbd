// ck_generate.cpp — synthetic detector, field and track generator.
//
// Builds the inputs of the five benchmark workloads. The truth simulation is
// independent of the fitter: a fixed-step RK4 integration of the Lorentz
// force with crossing refinement, Highland multiple-scattering kicks and
// mean Bethe energy loss at each silicon layer (the roles Fatras plays for
// the reference's truth-tracking examples), then Gaussian smearing of the
// local hit positions (digitisation) and of the start parameters.
//
// Random numbers: SplitMix64 (G. Steele, D. Lea, C. Flood, "Fast splittable
// pseudorandom number generators", OOPSLA 2014) seeded per track, uniform
// doubles from the top 53 bits, Gaussians by the Box-Muller transform.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "ckgen.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kT = 0.000299792458;  // 1 T in GeV/(e mm)
constexpr double kNs = 299.792458;     // 1 ns in mm/c
constexpr double kMuonMass = 0.1056583755;
constexpr double kPionMass = 0.13957039;

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(seed) {}
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  double uniform(double a, double b) { return a + (b - a) * uniform(); }
  double gauss() {
    double u1 = uniform();
    double u2 = uniform();
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
  }
};

uint64_t mix(uint64_t a, uint64_t b) {
  Rng r(a ^ (b * 0xD6E8FEB86659FD93ull));
  r.next();
  return r.next();
}

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

// the geometry / field / kinematics preset a preset shares
int basePreset(int preset) { return preset == CKG_STRIPS ? CKG_BARREL : preset; }

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

// ---------------------------------------------------------------- field
struct FieldEval {
  int kind = CK_FIELD_CONSTANT;
  double b[3] = {0, 0, 0};  // Tesla
  int n[3] = {0, 0, 0};
  double mn[3] = {0, 0, 0}, step[3] = {1, 1, 1};
  const float* v = nullptr;
  explicit FieldEval(const ck_field& f) {
    kind = f.kind;
    for (int i = 0; i < 3; ++i) b[i] = f.constant_tesla[i];
    if (kind == CK_FIELD_GRID_XYZ) {
      for (int i = 0; i < 3; ++i) {
        n[i] = f.n[i];
        mn[i] = f.min[i];
        step[i] = (f.max[i] - f.min[i]) / (n[i] - 1);
      }
      v = f.values_tesla;
    }
  }
  // field in GeV/(e mm); plain trilinear interpolation of the node values
  void get(const double* p, double* out) const {
    if (kind == CK_FIELD_CONSTANT) {
      for (int i = 0; i < 3; ++i) out[i] = b[i] * kT;
      return;
    }
    int idx[3];
    double f[3];
    for (int i = 0; i < 3; ++i) {
      double u = (p[i] - mn[i]) / step[i];
      int k = (int)std::floor(u);
      k = std::max(0, std::min(k, n[i] - 2));
      idx[i] = k;
      f[i] = std::min(1.0, std::max(0.0, u - k));
    }
    for (int c = 0; c < 3; ++c) {
      double acc = 0;
      for (int corner = 0; corner < 8; ++corner) {
        int dx = (corner >> 2) & 1, dy = (corner >> 1) & 1, dz = corner & 1;
        double w = (dx ? f[0] : 1 - f[0]) * (dy ? f[1] : 1 - f[1]) * (dz ? f[2] : 1 - f[2]);
        size_t id = ((size_t)(idx[0] + dx) * n[1] + (idx[1] + dy)) * n[2] + (idx[2] + dz);
        acc += w * v[id * 3 + c];
      }
      out[c] = acc * kT;
    }
  }
};

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

// --------------------------------------------------------- truth physics
struct Particle {
  int pdg;
  double mass;
  double q;
};

// Highland formula (PDG review, passage of particles through matter)
double highlandTheta0(double xOverX0, double p, double beta) {
  if (xOverX0 <= 0) return 0;
  return 13.6e-3 / (beta * p) * std::sqrt(xOverX0) * (1.0 + 0.038 * std::log(xOverX0 / (beta * beta)));
}

// Mean Bethe energy loss (PDG review eq. 34.5 form, no shell correction)
double betheLoss(const ck_surface& s, double thick, double m, double p) {
  const double me = 0.5109989461e-3;
  const double K = 0.307075e-3 * 100.0;  // GeV mm^2 / mol
  const double E = std::sqrt(m * m + p * p);
  const double beta2 = p * p / (E * E);
  const double bg = p / m;
  const double gamma = E / m;
  const double I = s.mat_mean_excitation;
  const double Ne = s.mat_molar_electron_rho;
  const double wmax = 2 * me * bg * bg / (1 + 2 * gamma * me / m + (me / m) * (me / m));
  double delta = 0;
  if (bg >= 10.0) {
    const double plasma = 28.816e-9 * std::sqrt(Ne * 1000.0);
    delta = 2.0 * (std::log(bg) + std::log(plasma / I) - 0.5);
  }
  const double eps = 0.5 * K * Ne * thick / beta2;
  return eps * (std::log(2 * me * bg * bg / I) + std::log(wmax / I) - 2 * beta2 - delta);
}

struct TState {
  double pos[3], dir[3];
  double p, t;
};

void rhs(const FieldEval& F, double qop, const double* pos, const double* dir, double* dpos,
         double* ddir) {
  double B[3];
  F.get(pos, B);
  for (int i = 0; i < 3; ++i) dpos[i] = dir[i];
  ddir[0] = qop * (dir[1] * B[2] - dir[2] * B[1]);
  ddir[1] = qop * (dir[2] * B[0] - dir[0] * B[2]);
  ddir[2] = qop * (dir[0] * B[1] - dir[1] * B[0]);
}

TState rk4(const FieldEval& F, const Particle& pa, const TState& s, double h) {
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
  const double n = std::sqrt(n2);
  for (int i = 0; i < 3; ++i) o.dir[i] /= n;
  const double E = std::sqrt(pa.mass * pa.mass + s.p * s.p);
  o.t = s.t + h * E / s.p;
  return o;
}

// signed distance of a point to a surface of the ordered detector
double sdist(const ck_surface& s, const double* p) {
  if (s.type == CK_SURFACE_CYLINDER) return std::sqrt(p[0] * p[0] + p[1] * p[1]) - s.radius;
  double d = 0;
  for (int i = 0; i < 3; ++i) d += s.rotation[i * 3 + 2] * (p[i] - s.center[i]);
  return d;
}

void toLocal(const ck_surface& s, const double* p, double* loc) {
  double d[3], l[3];
  for (int i = 0; i < 3; ++i) d[i] = p[i] - s.center[i];
  for (int j = 0; j < 3; ++j)
    l[j] = s.rotation[0 * 3 + j] * d[0] + s.rotation[1 * 3 + j] * d[1] + s.rotation[2 * 3 + j] * d[2];
  if (s.type == CK_SURFACE_CYLINDER) {
    loc[0] = s.radius * std::atan2(l[1], l[0]);
    loc[1] = l[2];
  } else {
    loc[0] = l[0];
    loc[1] = l[1];
  }
}

double cosIncidence(const ck_surface& s, const double* p, const double* dir) {
  double n[3];
  if (s.type == CK_SURFACE_CYLINDER) {
    double r = std::sqrt(p[0] * p[0] + p[1] * p[1]);
    n[0] = p[0] / r;
    n[1] = p[1] / r;
    n[2] = 0;
  } else {
    for (int i = 0; i < 3; ++i) n[i] = s.rotation[i * 3 + 2];
  }
  return std::abs(n[0] * dir[0] + n[1] * dir[1] + n[2] * dir[2]);
}

bool inBounds(const ck_surface& s, const double* p) {
  if (s.type == CK_SURFACE_CYLINDER) return std::abs(p[2]) < s.half_length_z;
  double loc[2];
  toLocal(s, p, loc);
  return std::abs(loc[0]) < s.half_x && std::abs(loc[1]) < s.half_y;
}

// kinematics and detector response of a preset
struct Preset {
  Particle pa;
  double sigma0, sigma1;
  int minHits, maxHits;
  double holeProb, outlierProb, outlierSigma;
  bool barrel;
};

Preset presetOf(int preset) {
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

struct TrackRows {
  std::vector<int> seq, measSurf;
  std::vector<double> measVal, measCov, truth;
  std::vector<uint8_t> outlier;
  std::vector<int32_t> measSub;
  double startParams[6], startCov[36], frame[12], truthStart[6];
  float particle[2];
  int pdg;
};

void generateTrack(int preset, uint64_t seed, int64_t id, const std::vector<ck_surface>& surf,
                   const FieldEval& F, TrackRows& out) {
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
    pT = std::exp(rng.uniform(std::log(0.5), std::log(100.0)));
    vz = 50.0 * rng.gauss();
  }
  const double theta = 2.0 * std::atan(std::exp(-eta));
  TState s;
  s.pos[0] = 0;
  s.pos[1] = 0;
  s.pos[2] = vz;
  s.dir[0] = std::cos(phi) * std::sin(theta);
  s.dir[1] = std::sin(phi) * std::sin(theta);
  s.dir[2] = std::cos(theta);
  s.p = pT / std::sin(theta);
  s.t = 0;
  const double qop0 = pa.q / s.p;

  // curvilinear start frame (CurvilinearSurface.cpp:25-39): U = z x T, V = T x U
  {
    double T[3] = {s.dir[0], s.dir[1], s.dir[2]};
    double U[3] = {-T[1], T[0], 0.0};  // z x T
    double un = std::sqrt(U[0] * U[0] + U[1] * U[1]);
    for (double& u : U) u /= un;
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
  const double sl = 0.010, sa = 0.001, sq = 0.01 * std::abs(qop0), st = kNs;
  out.startParams[0] = sl * rng.gauss();
  out.startParams[1] = sl * rng.gauss();
  double sphi = phi + sa * rng.gauss();
  if (sphi >= kPi) sphi -= 2 * kPi;
  if (sphi < -kPi) sphi += 2 * kPi;
  out.startParams[2] = sphi;
  out.startParams[3] = theta + sa * rng.gauss();
  out.startParams[4] = qop0 * (1.0 + 0.01 * rng.gauss());
  out.startParams[5] = st * rng.gauss();
  std::memset(out.startCov, 0, sizeof(out.startCov));
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
  size_t next = 0;
  double path = 0;
  const double maxPath = 20000.0;
  int nCrossed = 0;
  while (next < surf.size() && path < maxPath && nCrossed < nHitsMax) {
    if (std::abs(s.pos[2]) > 3000.0) break;
    const ck_surface& S = surf[next];
    double d0 = sdist(S, s.pos);
    TState s1 = rk4(F, pa, s, h);
    double d1 = sdist(S, s1.pos);
    if (!(d0 < 0 && d1 >= 0)) {
      // barrel loopers that turn back never reach the next layer
      if (P.barrel) {
        double r0 = std::hypot(s.pos[0], s.pos[1]), r1 = std::hypot(s1.pos[0], s1.pos[1]);
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
      if (std::abs(fc) < 1e-12) {
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
    ++next;
    if (!inBounds(S, s.pos)) continue;
    ++nCrossed;
    const int sid = (int)(&S - surf.data());
    out.seq.push_back(sid);
    // truth at the surface
    double loc[2];
    toLocal(S, s.pos, loc);
    const double tphi = std::atan2(s.dir[1], s.dir[0]);
    const double ttheta = std::atan2(std::hypot(s.dir[0], s.dir[1]), s.dir[2]);
    const bool hole = P.holeProb > 0 && rng.uniform() < P.holeProb;
    const bool outl = P.outlierProb > 0 && rng.uniform() < P.outlierProb;
    const double sgn0 = rng.uniform() < 0.5 ? -1.0 : 1.0;
    const double sgn1 = rng.uniform() < 0.5 ? -1.0 : 1.0;
    const double g0 = rng.gauss();
    const double g1 = rng.gauss();
    // strip layers (CKG_STRIPS, layers 4-9): one local coordinate
    int sub = CK_MEAS_LOC01;
    if (stripPreset && sid >= 4) sub = (sid % 2 == 0) ? CK_MEAS_LOC0 : CK_MEAS_LOC1;
    if (!hole && sub != CK_MEAS_LOC01) {
      const int h = sub == CK_MEAS_LOC0 ? 0 : 1;
      const double sg = h == 0 ? 0.100 : 0.150;
      double m = loc[h] + sg * (h == 0 ? g0 : g1);
      if (outl) m += (h == 0 ? sgn0 : sgn1) * P.outlierSigma * sg;
      out.measSurf.push_back(sid);
      out.measSub.push_back(sub);
      out.measVal.push_back(m);
      out.measVal.push_back(0.0);
      out.measCov.push_back(sg * sg);
      out.measCov.push_back(0.0);
      out.measCov.push_back(0.0);
      out.measCov.push_back(0.0);
    }
    double m0 = loc[0] + P.sigma0 * g0;
    double m1 = loc[1] + P.sigma1 * g1;
    if (!hole && sub == CK_MEAS_LOC01) {
      if (outl) {
        m0 += sgn0 * P.outlierSigma * P.sigma0;
        m1 += sgn1 * P.outlierSigma * P.sigma1;
      }
      out.measSurf.push_back(sid);
      out.measSub.push_back(sub);
      out.measVal.push_back(m0);
      out.measVal.push_back(m1);
      out.measCov.push_back(P.sigma0 * P.sigma0);
      out.measCov.push_back(0.0);
      out.measCov.push_back(0.0);
      out.measCov.push_back(P.sigma1 * P.sigma1);
    }
    if (!hole) {
      out.truth.push_back(loc[0]);
      out.truth.push_back(loc[1]);
      out.truth.push_back(tphi);
      out.truth.push_back(ttheta);
      out.truth.push_back(pa.q / s.p);
      out.truth.push_back(s.t);
      out.outlier.push_back(outl ? 1 : 0);
    }
    // material: Highland kick and mean Bethe loss
    if (S.flags & CK_SURF_MATERIAL) {
      const double cosA = cosIncidence(S, s.pos, s.dir);
      const double thick = S.mat_thickness / cosA;
      const double E = std::sqrt(pa.mass * pa.mass + s.p * s.p);
      const double beta = s.p / E;
      const double th0 = highlandTheta0(thick / S.mat_x0, s.p, beta);
      double u[3], v[3];
      {
        const double* T = s.dir;
        double a2[3] = {-T[1], T[0], 0.0};
        double n = std::hypot(a2[0], a2[1]);
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
      nn = std::sqrt(nn);
      for (double& x : s.dir) x /= nn;
      const double dE = betheLoss(S, thick, pa.mass, s.p);
      const double E2 = E - dE;
      s.p = (E2 > pa.mass) ? std::sqrt(E2 * E2 - pa.mass * pa.mass) : 0.01;
    }
  }
}

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
  FieldEval F(*field);
  std::vector<TrackRows> rows(n_tracks);
  if (n_threads < 1) n_threads = 1;
  std::vector<std::thread> th;
  for (int t = 0; t < n_threads; ++t)
    th.emplace_back([&, t]() {
      for (int i = t; i < n_tracks; i += n_threads)
        generateTrack(preset, seed, first_track + i, surf, F, rows[i]);
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
    std::memcpy(out->start_params + 6 * (size_t)i, r.startParams, sizeof(r.startParams));
    std::memcpy(out->start_cov + 36 * (size_t)i, r.startCov, sizeof(r.startCov));
    std::memcpy(out->start_frames + 12 * (size_t)i, r.frame, sizeof(r.frame));
    if (out->truth_start) std::memcpy(out->truth_start + 6 * (size_t)i, r.truthStart, sizeof(r.truthStart));
    out->particle[2 * i] = r.particle[0];
    out->particle[2 * i + 1] = r.particle[1];
    out->particle_pdg[i] = r.pdg;
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
