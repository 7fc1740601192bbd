// kf_oracle.hpp — CPU restatement of the reference Kalman track fit.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: it is linked into
// oracle/_build/libkforacle.so, which only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference legs load. The product
// (acts_gb300/) never includes or calls it.
//
// It restates, in plain scalar C++ (no Eigen, which is absent here), the
// algorithm of
//   Acts::KalmanFitter<Propagator<EigenStepper<>, DirectNavigator>,
//                      VectorMultiTrajectory>::fit
// with GainMatrixUpdater and GainMatrixSmoother, following the reference
// files cited at each function (paths relative to the acts repository).
// Matrix products are evaluated as written in the reference, left to right,
// with sequential inner sums; the 8x8 free transport Jacobian is kept in
// full as the reference does (EigenStepper.ipp:310-352).
//
// Parity pinning: the reference cannot be compiled in this environment
// (Eigen >= 3.4 and Boost >= 1.78 are absent), so the restatement is pinned
// against the reference's own known-answer unit tests (GainMatrixUpdater,
// GainMatrixSmoother, Interactions, interpolated field map, KF structural
// tests) in tests/test_oracle_pins.py.
//
// Deliberate, documented deviations from the reference:
//  * logf: the reference evaluates std::log on floats (glibc logf). Both this
//    oracle and the CUDA kernels use ck_logf(x) = (float)log((double)x), the
//    correctly rounded float logarithm except in ~2^-29 of cases, so that
//    the float material physics is reproducible across CPU and GPU.
//  * Field cell cache: InterpolatedBFieldMap caches the last cell; results
//    differ from a fresh cell lookup only by rounding at cell borders. The
//    oracle always looks the cell up afresh.
//  * Affine inverse: globalToLocal uses R^T (p - c) instead of Eigen's
//    general affine inverse (identical up to rounding for rotations).
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "cudakalman.h"

namespace kfo {

// ------------------------------------------------------------------ units
// Core/include/Acts/Definitions/Units.hpp:85-174 (long double literals are
// evaluated in long double and returned as double, as the reference's
// ACTS_DEFINE_UNIT_LITERAL does).
constexpr double kMeV = 1e-3;
constexpr double kEV = 1e-9;
constexpr double kMM2 = 1.0;
constexpr double kCM3 = 10.0 * 10.0 * 10.0;
constexpr double kTesla = 0.000299792458;
constexpr double kOnSurfaceTolerance = 1e-4;  // Tolerance.hpp:25
constexpr double kPi = 3.14159265358979323846;

inline double lit_MeV(long double x) { return (double)(kMeV * x); }
inline double lit_eV(long double x) { return (double)(kEV * x); }

// Float logarithm shared with the device code (see header note).
inline float ck_logf(float x) { return (float)std::log((double)x); }

// ------------------------------------------------------ small matrix types
template <typename S, int R, int C>
struct Mat {
  S a[R][C];
  S* operator[](int i) { return a[i]; }
  const S* operator[](int i) const { return a[i]; }
  static Mat zero() {
    Mat m;
    for (int i = 0; i < R; ++i)
      for (int j = 0; j < C; ++j) m.a[i][j] = S(0.0);
    return m;
  }
  static Mat identity() {
    Mat m = zero();
    for (int i = 0; i < R && i < C; ++i) m.a[i][i] = S(1.0);
    return m;
  }
};

template <typename S, int N>
struct Vec {
  S v[N];
  S& operator[](int i) { return v[i]; }
  const S& operator[](int i) const { return v[i]; }
  static Vec zero() {
    Vec x;
    for (int i = 0; i < N; ++i) x.v[i] = S(0.0);
    return x;
  }
};

template <typename S, int R, int K, int C>
Mat<S, R, C> mul(const Mat<S, R, K>& A, const Mat<S, K, C>& B) {
  Mat<S, R, C> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) {
      S s = A.a[i][0] * B.a[0][j];
      for (int k = 1; k < K; ++k) s = s + A.a[i][k] * B.a[k][j];
      out.a[i][j] = s;
    }
  return out;
}

template <typename S, int R, int C>
Vec<S, R> mulv(const Mat<S, R, C>& A, const Vec<S, C>& x) {
  Vec<S, R> out;
  for (int i = 0; i < R; ++i) {
    S s = A.a[i][0] * x.v[0];
    for (int k = 1; k < C; ++k) s = s + A.a[i][k] * x.v[k];
    out.v[i] = s;
  }
  return out;
}

template <typename S, int R, int C>
Mat<S, C, R> transpose(const Mat<S, R, C>& A) {
  Mat<S, C, R> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) out.a[j][i] = A.a[i][j];
  return out;
}

template <typename S, int R, int C>
Mat<S, R, C> add(const Mat<S, R, C>& A, const Mat<S, R, C>& B) {
  Mat<S, R, C> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) out.a[i][j] = A.a[i][j] + B.a[i][j];
  return out;
}

template <typename S, int R, int C>
Mat<S, R, C> sub(const Mat<S, R, C>& A, const Mat<S, R, C>& B) {
  Mat<S, R, C> out;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j) out.a[i][j] = A.a[i][j] - B.a[i][j];
  return out;
}

template <typename S, int R, int C>
bool hasNaN(const Mat<S, R, C>& A) {
  using std::isnan;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < C; ++j)
      if (isnan(A.a[i][j])) return true;
  return false;
}

// 6x6 inverse by LU with partial pivoting (the algorithm Eigen 3.4's
// fixed-size inverse() uses for N > 4).
template <typename S, int N>
Mat<S, N, N> inverse(const Mat<S, N, N>& A) {
  using std::abs;
  Mat<S, N, N> lu = A;
  int perm[N];
  for (int i = 0; i < N; ++i) perm[i] = i;
  for (int k = 0; k < N; ++k) {
    int p = k;
    S best = abs(lu.a[k][k]);
    for (int i = k + 1; i < N; ++i) {
      S v = abs(lu.a[i][k]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    if (p != k) {
      for (int j = 0; j < N; ++j) std::swap(lu.a[k][j], lu.a[p][j]);
      std::swap(perm[k], perm[p]);
    }
    S piv = lu.a[k][k];
    for (int i = k + 1; i < N; ++i) {
      S l = lu.a[i][k] / piv;
      lu.a[i][k] = l;
      for (int j = k + 1; j < N; ++j) lu.a[i][j] = lu.a[i][j] - l * lu.a[k][j];
    }
  }
  Mat<S, N, N> inv;
  for (int c = 0; c < N; ++c) {
    // solve L U x = P e_c
    S y[N];
    for (int i = 0; i < N; ++i) {
      S s = (perm[i] == c) ? S(1.0) : S(0.0);
      for (int j = 0; j < i; ++j) s = s - lu.a[i][j] * y[j];
      y[i] = s;
    }
    for (int i = N - 1; i >= 0; --i) {
      S s = y[i];
      for (int j = i + 1; j < N; ++j) s = s - lu.a[i][j] * inv.a[j][c];
      inv.a[i][c] = s / lu.a[i][i];
    }
  }
  return inv;
}

// 2x2 inverse by the adjugate (Eigen's compute_inverse for size 2).
template <typename S>
Mat<S, 2, 2> inverse2(const Mat<S, 2, 2>& m) {
  S det = m.a[0][0] * m.a[1][1] - m.a[0][1] * m.a[1][0];
  S invdet = S(1.0) / det;
  Mat<S, 2, 2> r;
  r.a[0][0] = m.a[1][1] * invdet;
  r.a[1][0] = -m.a[1][0] * invdet;
  r.a[0][1] = -m.a[0][1] * invdet;
  r.a[1][1] = m.a[0][0] * invdet;
  return r;
}

template <typename S>
using V3 = Vec<S, 3>;

template <typename S>
V3<S> cross(const V3<S>& a, const V3<S>& b) {
  V3<S> r;
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
  return r;
}
template <typename S>
S dot(const V3<S>& a, const V3<S>& b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <typename S>
S norm(const V3<S>& a) {
  using std::sqrt;
  return sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
}
template <typename S>
V3<S> normalized(const V3<S>& a) {
  using std::sqrt;
  S n2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
  V3<S> r = a;
  if (n2 > S(0.0)) {
    S n = sqrt(n2);
    r[0] = a[0] / n;
    r[1] = a[1] / n;
    r[2] = a[2] / n;
  }
  return r;
}
template <typename S>
S perp(const V3<S>& a) {
  using std::sqrt;
  return sqrt(a[0] * a[0] + a[1] * a[1]);
}

// ------------------------------------------------------------- periodic
// Core/include/Acts/Utilities/detail/periodic.hpp:19-93
template <typename S>
S wrap_periodic(S value, S start, S range) {
  using std::floor;
  S diff = value - start;
  return ((S(0.0) <= diff) && (diff < range)) ? value
                                               : (value - range * floor(diff / range));
}
template <typename S>
S radian_pos(S x) {
  return wrap_periodic<S>(x, S(0.0), S(2 * kPi));
}
template <typename S>
S radian_sym(S x) {
  return wrap_periodic<S>(x, S(-kPi), S(2 * kPi));
}
template <typename S>
void normalizePhiTheta(S& phi, S& theta) {
  theta = radian_pos(theta);
  if (S(kPi) < theta) {
    phi = phi + S(kPi);
    theta = S(2 * kPi) - theta;
  }
  phi = radian_sym(phi);
}
// TrackParameterHelpers.hpp:51-83
template <typename S>
Vec<S, 6> normalizeBoundParameters(Vec<S, 6> p) {
  normalizePhiTheta(p[2], p[3]);
  return p;
}
template <typename S>
Vec<S, 6> subtractBoundParameters(const Vec<S, 6>& a, const Vec<S, 6>& b) {
  Vec<S, 6> r;
  for (int i = 0; i < 6; ++i) r[i] = a[i] - b[i];
  r[2] = radian_sym(r[2]);
  r[3] = radian_sym(r[3]);
  return r;
}

// ------------------------------------------------- direction helpers
// VectorHelpers.hpp:165-178, MathHelpers.hpp:94-180
template <typename S>
struct Trig {
  S cosPhi, sinPhi, cosTheta, sinTheta;
};
template <typename S>
Trig<S> evaluateTrigonomics(const V3<S>& d) {
  using std::abs;
  using std::sqrt;
  Trig<S> t;
  t.cosTheta = d[2];
  S az = abs(d[2]);
  t.sinTheta = sqrt((S(1.0) - az) * (S(1.0) + az));
  S invSinTheta = S(1.0) / t.sinTheta;
  t.cosPhi = d[0] * invSinTheta;
  t.sinPhi = d[1] * invSinTheta;
  return t;
}
// JacobianHelpers.hpp:26-64
template <typename S>
Mat<S, 3, 2> sphericalToFreeDirectionJacobian(const V3<S>& d) {
  Trig<S> t = evaluateTrigonomics(d);
  Mat<S, 3, 2> j;
  j.a[0][0] = -d[1];
  j.a[0][1] = t.cosTheta * t.cosPhi;
  j.a[1][0] = d[0];
  j.a[1][1] = t.cosTheta * t.sinPhi;
  j.a[2][0] = S(0.0);
  j.a[2][1] = -t.sinTheta;
  return j;
}
template <typename S>
Mat<S, 2, 3> freeToSphericalDirectionJacobian(const V3<S>& d) {
  Trig<S> t = evaluateTrigonomics(d);
  S invSinTheta = S(1.0) / t.sinTheta;
  Mat<S, 2, 3> j;
  j.a[0][0] = -t.sinPhi * invSinTheta;
  j.a[0][1] = t.cosPhi * invSinTheta;
  j.a[0][2] = S(0.0);
  j.a[1][0] = t.cosPhi * t.cosTheta;
  j.a[1][1] = t.sinPhi * t.cosTheta;
  j.a[1][2] = -t.sinTheta;
  return j;
}

// ---------------------------------------------------------------- surfaces
enum class IStatus { unreachable = 0, reachable = 1, onSurface = 2 };

template <typename S>
struct Intersection {
  S pathLength;
  IStatus status;
  bool valid() const { return status != IStatus::unreachable; }
};

// Material slab with the reference's float fields
// (Core/include/Acts/Material/MaterialSlab.hpp:94-128, Material.hpp:135-145).
struct Slab {
  float X0 = 0, L0 = 0, Ar = 0, Z = 0, molarRho = 0, molarElectronRho = 0,
        meanExcitation = 0;
  float thickness = 0, thicknessInX0 = 0, thicknessInL0 = 0;
  bool vacuumMaterial = true;
  bool isVacuum() const { return vacuumMaterial || thickness <= 0.0f; }
  void scaleThickness(float s) {
    thickness *= s;
    thicknessInX0 *= s;
    thicknessInL0 *= s;
  }
  static Slab make(const ck_surface& cs) {
    Slab s;
    s.X0 = cs.mat_x0;
    s.L0 = cs.mat_l0;
    s.Ar = cs.mat_ar;
    s.Z = cs.mat_z;
    s.molarRho = cs.mat_molar_rho;
    s.molarElectronRho = cs.mat_molar_electron_rho;
    s.meanExcitation = cs.mat_mean_excitation;
    s.vacuumMaterial = !(cs.mat_ar > 0.0f);
    const float eps = 2 * std::numeric_limits<float>::epsilon();
    s.thickness = cs.mat_thickness;
    s.thicknessInX0 = (eps < s.X0) ? (cs.mat_thickness / s.X0) : 0.0f;
    s.thicknessInL0 = (eps < s.L0) ? (cs.mat_thickness / s.L0) : 0.0f;
    return s;
  }
};

template <typename S>
struct Surface {
  int type = CK_SURFACE_PLANE;
  bool sensitive = false;
  bool hasMaterial = false;
  S R[3][3];
  S c[3];
  S radius = S(0.0);
  Slab slab;
  float splitFactor = 1.0f;

  static Surface fromCk(const ck_surface& cs) {
    Surface s;
    s.type = cs.type;
    s.sensitive = (cs.flags & CK_SURF_SENSITIVE) != 0;
    s.hasMaterial = (cs.flags & CK_SURF_MATERIAL) != 0;
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) s.R[i][j] = S(cs.rotation[i * 3 + j]);
      s.c[i] = S(cs.center[i]);
    }
    s.radius = S(cs.radius);
    s.slab = Slab::make(cs);
    s.splitFactor = cs.split_factor;
    return s;
  }
  static Surface plane(const double* frame12) {
    Surface s;
    s.type = CK_SURFACE_PLANE;
    for (int i = 0; i < 3; ++i) {
      for (int j = 0; j < 3; ++j) s.R[i][j] = S(frame12[i * 3 + j]);
      s.c[i] = S(frame12[9 + i]);
    }
    return s;
  }

  V3<S> col(int j) const {
    V3<S> v;
    for (int i = 0; i < 3; ++i) v[i] = R[i][j];
    return v;
  }
  V3<S> toLocal3(const V3<S>& p) const {  // R^T (p - c)
    V3<S> d, l;
    for (int i = 0; i < 3; ++i) d[i] = p[i] - c[i];
    for (int j = 0; j < 3; ++j) l[j] = R[0][j] * d[0] + R[1][j] * d[1] + R[2][j] * d[2];
    return l;
  }
  V3<S> toGlobal3(const V3<S>& l) const {  // R l + c
    V3<S> g;
    for (int i = 0; i < 3; ++i) g[i] = (R[i][0] * l[0] + R[i][1] * l[1] + R[i][2] * l[2]) + c[i];
    return g;
  }

  // PlanarHelper.hpp:56-77 ; CylinderSurface.cpp:199-277 ;
  // RealQuadraticEquation.hpp:47-67. Boundary tolerance is Infinite for the
  // DirectNavigator (DirectNavigator.hpp:266-269), so bounds are not checked.
  int intersect(const V3<S>& pos, const V3<S>& dir, S tol, Intersection<S> out[2]) const {
    using std::abs;
    using std::sqrt;
    if (type == CK_SURFACE_LINE) {
      // LineSurface::intersect (LineSurface.cpp:141-185): closest approach of
      // the straight track to the line; no bounds (a PerigeeSurface)
      V3<S> eb = col(2);
      V3<S> mab;
      for (int i = 0; i < 3; ++i) mab[i] = c[i] - pos[i];
      S eaTeb = dot(dir, eb);
      S denom = S(1.0) - eaTeb * eaTeb;
      if (abs(denom) < abs(tol)) {
        out[0] = Intersection<S>{S(std::numeric_limits<double>::infinity()), IStatus::unreachable};
        return 0;
      }
      S u = (dot(mab, dir) - dot(mab, eb) * eaTeb) / denom;
      out[0] = Intersection<S>{u, abs(u) > abs(tol) ? IStatus::reachable : IStatus::onSurface};
      return 1;
    }
    if (type == CK_SURFACE_PLANE) {
      V3<S> n = col(2);
      S denom = dot(dir, n);
      if (denom == S(0.0)) {
        out[0] = {S(0.0), IStatus::unreachable};
        return 1;
      }
      V3<S> cp;
      for (int i = 0; i < 3; ++i) cp[i] = c[i] - pos[i];
      S path = dot(n, cp) / denom;
      out[0] = {path, abs(path) < abs(tol) ? IStatus::onSurface : IStatus::reachable};
      return 1;
    }
    V3<S> axis = col(2);
    V3<S> pc;
    for (int i = 0; i < 3; ++i) pc[i] = pos[i] - c[i];
    V3<S> pcXcd = cross(pc, axis);
    V3<S> ldXcd = cross(dir, axis);
    S a = dot(ldXcd, ldXcd);
    S b = S(2.0) * dot(ldXcd, pcXcd);
    S cc = dot(pcXcd, pcXcd) - radius * radius;
    S disc = b * b - S(4.0) * a * cc;
    if (!(disc >= S(0.0))) {
      out[0] = {S(0.0), IStatus::unreachable};
      out[1] = {S(0.0), IStatus::unreachable};
      return 2;
    }
    int nsol = (disc == S(0.0)) ? 1 : 2;
    S sq = sqrt(disc);
    S q = S(-0.5) * (b + (b > S(0.0) ? sq : -sq));
    S first = q / a;
    S second = cc / q;
    Intersection<S> i1{first, abs(first) < abs(tol) ? IStatus::onSurface : IStatus::reachable};
    if (nsol == 1) {
      out[0] = i1;
      out[1] = i1;
      return 2;
    }
    Intersection<S> i2{second, abs(second) < abs(tol) ? IStatus::onSurface : IStatus::reachable};
    if (i1.pathLength <= i2.pathLength) {
      out[0] = i1;
      out[1] = i2;
    } else {
      out[0] = i2;
      out[1] = i1;
    }
    return 2;
  }

  // PlaneSurface.cpp:77-86 ; CylinderSurface.cpp:125-145 ;
  // LineSurface.cpp:70-96 (the line frame depends on the direction)
  bool globalToLocal(const V3<S>& pos, const V3<S>& dir, S tol, S loc[2]) const {
    using std::abs;
    using std::atan2;
    if (type == CK_SURFACE_LINE) {
      Mat<S, 3, 3> f = referenceFrame(pos, dir);
      V3<S> d;
      for (int i = 0; i < 3; ++i) d[i] = pos[i] - c[i];
      S lz = f.a[0][2] * d[0] + f.a[1][2] * d[1] + f.a[2][2] * d[2];
      if (abs(lz) > abs(tol)) return false;
      loc[0] = f.a[0][0] * d[0] + f.a[1][0] * d[1] + f.a[2][0] * d[2];
      loc[1] = f.a[0][1] * d[0] + f.a[1][1] * d[1] + f.a[2][1] * d[2];
      return true;
    }
    V3<S> l = toLocal3(pos);
    if (type == CK_SURFACE_PLANE) {
      if (abs(l[2]) > abs(tol)) return false;
      loc[0] = l[0];
      loc[1] = l[1];
      return true;
    }
    S inttol = tol;
    if (tol == S(kOnSurfaceTolerance)) inttol = radius * S(0.0001);
    if (inttol < S(0.01)) inttol = S(0.01);
    if (abs(perp(l) - radius) > inttol) return false;
    loc[0] = radius * atan2(l[1], l[0]);
    loc[1] = l[2];
    return true;
  }

  // PlaneSurface.cpp:72-75 ; CylinderSurface.cpp:116-123 ; LineSurface.cpp:57-68
  V3<S> localToGlobal(const S loc[2], const V3<S>& dir) const {
    using std::cos;
    using std::sin;
    V3<S> l;
    if (type == CK_SURFACE_LINE) {
      V3<S> r = normalized(cross(col(2), dir));
      V3<S> z;
      for (int i = 0; i < 3; ++i) z[i] = R[i][2] * loc[1] + c[i];
      V3<S> g;
      for (int i = 0; i < 3; ++i) g[i] = z[i] + loc[0] * r[i];
      return g;
    }
    if (type == CK_SURFACE_PLANE) {
      l[0] = loc[0];
      l[1] = loc[1];
      l[2] = S(0.0);
    } else {
      S phi = loc[0] / radius;
      l[0] = radius * cos(phi);
      l[1] = radius * sin(phi);
      l[2] = loc[1];
    }
    return toGlobal3(l);
  }

  // CylinderSurface.cpp:154-163
  V3<S> normal(const V3<S>& pos) const {
    if (type == CK_SURFACE_PLANE) return col(2);
    V3<S> p3 = toLocal3(pos);
    p3[2] = S(0.0);
    V3<S> n = normalized(p3);
    V3<S> g;
    for (int i = 0; i < 3; ++i) g[i] = R[i][0] * n[0] + R[i][1] * n[1] + R[i][2] * n[2];
    return g;
  }

  // PlaneSurface.cpp:63-66 ; CylinderSurface.cpp:93-110 ; LineSurface.cpp:102-115
  Mat<S, 3, 3> referenceFrame(const V3<S>& pos, const V3<S>& dir) const {
    Mat<S, 3, 3> f;
    if (type == CK_SURFACE_LINE) {
      V3<S> z0 = col(2);
      V3<S> d0 = normalized(cross(z0, dir));
      V3<S> dist = cross(d0, z0);
      for (int i = 0; i < 3; ++i) {
        f.a[i][0] = d0[i];
        f.a[i][1] = z0[i];
        f.a[i][2] = dist[i];
      }
      return f;
    }
    if (type == CK_SURFACE_PLANE) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) f.a[i][j] = R[i][j];
      return f;
    }
    V3<S> measY = col(2);
    V3<S> measDepth = normal(pos);
    V3<S> measX = normalized(cross(measY, measDepth));
    for (int i = 0; i < 3; ++i) {
      f.a[i][0] = measX[i];
      f.a[i][1] = measY[i];
      f.a[i][2] = measDepth[i];
    }
    return f;
  }

  // PlaneSurface.cpp:155-160 ; CylinderSurface.cpp:165-171
  S pathCorrection(const V3<S>& pos, const V3<S>& dir) const {
    using std::abs;
    if (type == CK_SURFACE_PLANE) return S(1.0) / abs(dot(col(2), dir));
    V3<S> n = normal(pos);
    S cosAlpha = dot(n, dir);
    return abs(S(1.0) / cosAlpha);
  }

  // Surface.cpp:249-268
  Mat<S, 8, 6> boundToFreeJacobian(const V3<S>& pos, const V3<S>& dir) const {
    Mat<S, 3, 3> rf = referenceFrame(pos, dir);
    Mat<S, 8, 6> j = Mat<S, 8, 6>::zero();
    for (int i = 0; i < 3; ++i) {
      j.a[i][0] = rf.a[i][0];
      j.a[i][1] = rf.a[i][1];
    }
    j.a[3][5] = S(1.0);
    Mat<S, 3, 2> sj = sphericalToFreeDirectionJacobian(dir);
    for (int i = 0; i < 3; ++i) {
      j.a[4 + i][2] = sj.a[i][0];
      j.a[4 + i][3] = sj.a[i][1];
    }
    j.a[7][4] = S(1.0);
    return j;
  }

  // Surface.cpp:270-291
  Mat<S, 6, 8> freeToBoundJacobian(const V3<S>& pos, const V3<S>& dir) const {
    Mat<S, 3, 3> rf = referenceFrame(pos, dir);
    Mat<S, 6, 8> j = Mat<S, 6, 8>::zero();
    for (int k = 0; k < 3; ++k) {
      j.a[0][k] = rf.a[k][0];
      j.a[1][k] = rf.a[k][1];
    }
    j.a[5][3] = S(1.0);
    Mat<S, 2, 3> fj = freeToSphericalDirectionJacobian(dir);
    for (int k = 0; k < 3; ++k) {
      j.a[2][4 + k] = fj.a[0][k];
      j.a[3][4 + k] = fj.a[1][k];
    }
    j.a[4][7] = S(1.0);
    return j;
  }

  // Surface.cpp:293-306 ; LineSurface.cpp:224-251
  Vec<S, 8> freeToPathDerivative(const V3<S>& pos, const V3<S>& dir) const {
    if (type == CK_SURFACE_LINE) {
      V3<S> pc, z = col(2);
      for (int i = 0; i < 3; ++i) pc[i] = pos[i] - c[i];
      S pz = dot(pc, z);
      S dz = dot(z, dir);
      S nrm = S(1.0) / (S(1.0) - dz * dz);
      Vec<S, 8> f = Vec<S, 8>::zero();
      for (int i = 0; i < 3; ++i) {
        f[i] = nrm * (dz * z[i] - dir[i]);
        f[4 + i] = nrm * (pz * z[i] - pc[i]);
      }
      return f;
    }
    Mat<S, 3, 3> rf = referenceFrame(pos, dir);
    V3<S> z;
    for (int i = 0; i < 3; ++i) z[i] = rf.a[i][2];
    S dz = dot(z, dir);
    Vec<S, 8> f = Vec<S, 8>::zero();
    for (int i = 0; i < 3; ++i) f[i] = (S(-1.0) * z[i]) / dz;
    return f;
  }
};

// ------------------------------------------------------ bound <-> free
// Core/src/EventData/TransformationHelpers.cpp:17-63 ; UnitVectors.hpp:50-57
template <typename S>
Vec<S, 8> boundToFree(const Surface<S>& s, const Vec<S, 6>& b) {
  using std::cos;
  using std::sin;
  S sinTheta = sin(b[3]);
  V3<S> dir;
  dir[0] = cos(b[2]) * sinTheta;
  dir[1] = sin(b[2]) * sinTheta;
  dir[2] = cos(b[3]);
  S loc[2] = {b[0], b[1]};
  V3<S> pos = s.localToGlobal(loc, dir);
  Vec<S, 8> f;
  f[0] = pos[0];
  f[1] = pos[1];
  f[2] = pos[2];
  f[3] = b[5];
  f[4] = dir[0];
  f[5] = dir[1];
  f[6] = dir[2];
  f[7] = b[4];
  return f;
}

template <typename S>
bool freeToBound(const Vec<S, 8>& f, const Surface<S>& s, Vec<S, 6>& b) {
  using std::atan2;
  V3<S> pos{{f[0], f[1], f[2]}};
  V3<S> dir{{f[4], f[5], f[6]}};
  S loc[2];
  if (!s.globalToLocal(pos, dir, S(kOnSurfaceTolerance), loc)) return false;
  b[0] = loc[0];
  b[1] = loc[1];
  b[5] = f[3];
  b[2] = atan2(dir[1], dir[0]);
  b[3] = atan2(perp(dir), dir[2]);
  b[4] = f[7];
  return true;
}

// ---------------------------------------------------------------- field
template <typename S>
struct Field {
  int kind = CK_FIELD_CONSTANT;
  V3<S> b;  // internal units
  // XYZ grid (BFieldMapUtils.cpp:106-186, Helpers.hpp:289-310, Axis.hpp:232-276)
  int n[3] = {0, 0, 0};
  double mn[3], width[3], upper[3];
  const float* values = nullptr;

  static Field make(const ck_field& f) {
    Field F;
    F.kind = f.kind;
    for (int i = 0; i < 3; ++i) F.b[i] = S(f.constant_tesla[i] * kTesla);
    if (f.kind == CK_FIELD_GRID_XYZ) {
      for (int i = 0; i < 3; ++i) {
        F.n[i] = f.n[i];
        double xmin = f.min[i], xmax = f.max[i];
        double step = (xmax - xmin) / static_cast<double>(f.n[i] - 1);
        xmax += step;
        F.mn[i] = xmin;
        F.width[i] = (xmax - xmin) / static_cast<double>(f.n[i]);
        // m_upperRight = lower-left edge of the last bin
        F.upper[i] = xmin + static_cast<double>(f.n[i] - 1) * F.width[i];
      }
      F.values = f.values_tesla;
    }
    return F;
  }

  // grid value at local bin (i,j,k), 1-based; the overflow bin holds zero
  V3<S> node(int i, int j, int k) const {
    V3<S> v;
    if (i > n[0] || j > n[1] || k > n[2]) {
      v[0] = v[1] = v[2] = S(0.0);
      return v;
    }
    size_t idx = ((size_t)(i - 1) * n[1] + (j - 1)) * n[2] + (k - 1);
    for (int c = 0; c < 3; ++c) v[c] = S((double)values[idx * 3 + c] * kTesla);
    return v;
  }

  // InterpolatedBFieldMap::getField (InterpolatedBFieldMap.hpp:238-264,
  // 354-366) with the trilinear interpolate (Interpolation.hpp:96-120).
  bool get(const V3<S>& p, V3<S>& out) const {
    using std::floor;
    if (kind == CK_FIELD_CONSTANT) {
      out = b;
      return true;
    }
    for (int i = 0; i < 3; ++i)
      if (p[i] < S(mn[i]) || p[i] >= S(upper[i])) return false;
    int bin[3];
    S ll[3], ur[3];
    for (int i = 0; i < 3; ++i) {
      int bb = static_cast<int>(floor((p[i] - S(mn[i])) / S(width[i])) + S(1.0));
      bb = std::max(0, std::min(bb, n[i] + 1));
      bin[i] = bb;
      ll[i] = S(mn[i]) + S(static_cast<double>(bb - 1)) * S(width[i]);
      ur[i] = S(mn[i]) + S(static_cast<double>(bb)) * S(width[i]);
    }
    V3<S> v[8];
    for (int c = 0; c < 8; ++c)
      v[c] = node(bin[0] + ((c >> 2) & 1), bin[1] + ((c >> 1) & 1), bin[2] + (c & 1));
    // reduce z, then y, then x
    int cnt = 8;
    for (int d = 2; d >= 0; --d) {
      S f = (p[d] - ll[d]) / (ur[d] - ll[d]);
      for (int i = 0; i < cnt / 2; ++i)
        for (int c = 0; c < 3; ++c)
          v[i][c] = (S(1.0) - f) * v[2 * i][c] + f * v[2 * i + 1][c];
      cnt /= 2;
    }
    out = v[0];
    return true;
  }
};

// ------------------------------------------------------------- material
// Core/src/Material/Interactions.cpp:23-198,313-329,484-530 (float physics)
struct MatConst {
  float Me, K, PlasmaEnergyScale, invCm3;
  double highland;  // 13.6_MeV
  static MatConst make() {
    MatConst c;
    c.Me = (float)lit_MeV(0.5109989461L);
    c.K = (float)(lit_MeV(30.7075L) * kMM2);
    c.PlasmaEnergyScale = (float)lit_eV(28.816L);
    c.invCm3 = static_cast<float>(1 / kCM3);
    c.highland = lit_MeV(13.6L);
    return c;
  }
};

struct RelQ {
  float q2OverBeta2, beta2, betaGamma, gamma;
  RelQ(float mass, float qOverP, float absQ) {
    q2OverBeta2 = absQ * absQ + (mass * qOverP) * (mass * qOverP);
    const float mOverP = mass * std::abs(qOverP / absQ);
    const float pOverM = 1.0f / mOverP;
    beta2 = 1.0f / (1.0f + mOverP * mOverP);
    betaGamma = pOverM;
    gamma = std::sqrt(1.0f * 1.0f + pOverM * pOverM);
  }
};

inline float computeEpsilon(const MatConst& C, float Ne, float thickness, const RelQ& rq) {
  return 0.5f * C.K * Ne * thickness * rq.q2OverBeta2;
}
inline float computeDeltaHalf(const MatConst& C, float I, float Ne, const RelQ& rq) {
  if (rq.betaGamma < 10.0f) return 0.0f;
  const float plasmaEnergy = C.PlasmaEnergyScale * std::sqrt(Ne / C.invCm3);
  return ck_logf(rq.betaGamma) + ck_logf(plasmaEnergy / I) - 0.5f;
}
inline float computeMassTerm(float mass, const RelQ& rq) {
  return 2 * mass * rq.betaGamma * rq.betaGamma;
}
inline float computeWMax(const MatConst& C, float mass, const RelQ& rq) {
  const float mfrac = C.Me / mass;
  const float nominator = 2 * C.Me * rq.betaGamma * rq.betaGamma;
  const float denonimator = 1.0f + 2 * rq.gamma * mfrac + mfrac * mfrac;
  return nominator / denonimator;
}

inline float computeEnergyLossBethe(const MatConst& C, const Slab& slab, float m, float qOverP,
                                    float absQ) {
  if (slab.isVacuum()) return 0.0f;
  const RelQ rq{m, qOverP, absQ};
  const float I = slab.meanExcitation;
  const float Ne = slab.molarElectronRho;
  const float thickness = slab.thickness;
  const float eps = computeEpsilon(C, Ne, thickness, rq);
  const float dhalf = computeDeltaHalf(C, I, Ne, rq);
  const float u = computeMassTerm(C.Me, rq);
  const float wmax = computeWMax(C, m, rq);
  const float running = ck_logf(u / I) + ck_logf(wmax / I) - 2.0f * rq.beta2 - 2.0f * dhalf;
  return eps * running;
}

inline float computeEnergyLossLandau(const MatConst& C, const Slab& slab, float m, float qOverP,
                                     float absQ) {
  if (slab.isVacuum()) return 0.0f;
  const RelQ rq{m, qOverP, absQ};
  const float I = slab.meanExcitation;
  const float Ne = slab.molarElectronRho;
  const float eps = computeEpsilon(C, Ne, slab.thickness, rq);
  const float dhalf = computeDeltaHalf(C, I, Ne, rq);
  const float u = computeMassTerm(C.Me, rq);
  const float running = ck_logf(u / I) + ck_logf(eps / I) + 0.2f - rq.beta2 - 2 * dhalf;
  return eps * running;
}

inline float computeEnergyLossLandauFwhm(const MatConst& C, const Slab& slab, const RelQ& rq) {
  if (slab.isVacuum()) return 0.0f;
  return 4 * computeEpsilon(C, slab.molarElectronRho, slab.thickness, rq);
}

inline float computeEnergyLossLandauSigmaQOverP(const MatConst& C, const Slab& slab, float m,
                                                float qOverP, float absQ) {
  const RelQ rq{m, qOverP, absQ};
  const float fwhm = computeEnergyLossLandauFwhm(C, slab, rq);
  const float sigmaE = fwhm * 0.42466090014400953f;
  const float pInv = qOverP / absQ;
  const float qOverBeta = std::sqrt(rq.q2OverBeta2);
  return qOverBeta * pInv * pInv * sigmaE;
}

inline float computeMultipleScatteringTheta0(const MatConst& C, const Slab& slab, int absPdg,
                                             float m, float qOverP, float absQ) {
  if (slab.isVacuum()) return 0.0f;
  const float xOverX0 = slab.thicknessInX0;
  const float momentumInv = std::abs(qOverP / absQ);
  const float q2OverBeta2 = RelQ(m, qOverP, absQ).q2OverBeta2;
  const float t = std::sqrt(xOverX0 * q2OverBeta2);
  if (absPdg == 11) {
    // Rossi-Greisen: 17.5 MeV, log10 (Interactions.cpp:490-495)
    return (float)(lit_MeV(17.5L) * momentumInv * t *
                   (1.0f + 0.125f * (ck_logf(10.0f * xOverX0) / ck_logf(10.0f))));
  }
  return (float)(C.highland * momentumInv * t * (1.0f + 0.038f * 2 * ck_logf(t)));
}

struct MatEffects {
  double eLoss = 0, variancePhi = 0, varianceTheta = 0, varianceQoverP = 0;
};

// PointwiseMaterialInteraction.cpp:49-90
template <typename S>
MatEffects computeMaterialEffects(const MatConst& C, const Slab& slab, int absPdg, double mass,
                                  double absQ, const V3<S>& dir, float qOverP, bool ms, bool el) {
  MatEffects r;
  if (el) r.eLoss = computeEnergyLossBethe(C, slab, (float)mass, qOverP, (float)absQ);
  if (ms) {
    const double theta0 =
        computeMultipleScatteringTheta0(C, slab, absPdg, (float)mass, qOverP, (float)absQ);
    const double sigmaPhi = theta0 * ((double)norm(dir) / (double)perp(dir));
    r.variancePhi = sigmaPhi * sigmaPhi;
    r.varianceTheta = theta0 * theta0;
  }
  if (el) {
    const double s = computeEnergyLossLandauSigmaQOverP(C, slab, (float)mass, qOverP, (float)absQ);
    r.varianceQoverP = s * s;
  }
  return r;
}

// ------------------------------------------------------------ stepper
// EigenStepper state (EigenStepper.hpp / EigenStepper.ipp:37-70) and
// ConstrainedStep (ConstrainedStep.hpp:44-173)
struct ConstrainedStep {
  static constexpr double kNotSet = std::numeric_limits<double>::max();
  double values[3] = {kNotSet, kNotSet, kNotSet};  // navigator, actor, user
  double accuracy = kNotSet;
  double value() const {
    double mn = std::min(values[0], std::min(values[1], values[2]));
    double result = std::min(std::abs(mn), accuracy);
    return std::signbit(mn) ? -result : result;
  }
  void release(int t) { values[t] = kNotSet; }
  void update(double v, int t) {
    if (std::abs(v) < std::abs(values[t])) values[t] = v;
  }
};
enum { kNav = 0, kActor = 1, kUser = 2 };

template <typename S>
struct Stepper {
  Vec<S, 8> pars;
  Mat<S, 6, 6> cov;
  Mat<S, 6, 6> jacobian;
  Mat<S, 8, 8> jacTransport;
  Vec<S, 8> derivative;
  Mat<S, 8, 6> jacToGlobal;
  S pathAccumulated = S(0.0);
  ConstrainedStep stepSize;
  int nSteps = 0;
  float mass = 0, absQ = 1;
  int absPdg = 0;
  // step data
  V3<S> B_first, B_middle, B_last, k1, k2, k3, k4;

  S qop() const { return pars[7]; }
  V3<S> pos() const { return V3<S>{{pars[0], pars[1], pars[2]}}; }
  V3<S> dir() const { return V3<S>{{pars[4], pars[5], pars[6]}}; }
  // ChargeHypothesis.hpp:70-90
  S absoluteMomentum() const {
    using std::copysign;
    float q = (float)copysign((double)absQ, (double)qop());
    return S((double)q) / qop();
  }
};

struct Options {
  double stepTolerance, stepSizeCutOff, initialStepSize, maxStepSize;
  unsigned maxRungeKuttaStepTrials, maxSteps, maxTargetSkipping;
  bool loopProtection;
  double pathLimit, loopFraction, surfaceTolerance, nearLimit;
  bool multipleScattering, energyLoss, josephs;
  double outlierChi2Cut;
  bool coastAfterLastMeasurement;  // faithful reference termination
  int smoother;                    // CK_SMOOTHER_*
  int referenceSurface;            // -1 or a table index
  int referenceStrategy;           // CK_EXTRAPOLATE_*
  bool freeToBoundCorrection;      // KalmanFitterOptions::freeToBoundCorrection
  bool reverseFiltering;           // KalmanFitterOptions::reverseFiltering
  double reverseCovScaling;        // reverseFilteringCovarianceScaling
  double reverseMomThreshold;      // the examples' reverseFilteringLogic threshold
  static Options fromCk(const ck_options& o, bool coast) {
    Options r;
    r.reverseFiltering = o.reverse_filtering != 0;
    r.reverseCovScaling = o.reverse_filtering_cov_scaling;
    r.reverseMomThreshold = o.reverse_filtering_mom_threshold;
    r.freeToBoundCorrection = o.free_to_bound_correction != 0;
    r.smoother = o.smoother;
    r.referenceSurface = o.reference_surface;
    r.referenceStrategy = o.reference_strategy;
    r.stepTolerance = o.step_tolerance;
    r.stepSizeCutOff = o.step_size_cutoff;
    r.initialStepSize = o.initial_step_size;
    r.maxStepSize = o.max_step_size;
    r.maxRungeKuttaStepTrials = o.max_rk_step_trials;
    r.maxSteps = o.max_steps;
    r.maxTargetSkipping = o.max_target_skipping;
    r.loopProtection = o.loop_protection != 0;
    r.pathLimit = o.path_limit;
    r.loopFraction = o.loop_fraction;
    r.surfaceTolerance = o.surface_tolerance;
    r.nearLimit = o.near_limit;
    r.multipleScattering = o.multiple_scattering != 0;
    r.energyLoss = o.energy_loss != 0;
    r.josephs = o.use_joseph != 0;
    r.outlierChi2Cut = o.outlier_chi2_cut;
    r.coastAfterLastMeasurement = coast;
    return r;
  }
};

// Result of one stepper step: EigenStepper::step (EigenStepper.ipp:168-388)
// with EigenStepperDefaultExtension (EigenStepperDefaultExtension.hpp:40-228).
enum StepErr { kStepOk = 0, kStepField = 1, kStepStalled = 2, kStepAdjust = 3 };

template <typename S>
int eigenStep(Stepper<S>& st, const Field<S>& field, const Options& o, S& hOut,
              int propDir = 1) {
  using std::abs;
  using std::sqrt;
  V3<S> pos = st.pos();
  V3<S> dir = st.dir();
  S qop = st.qop();
  if (!field.get(pos, st.B_first)) return kStepField;
  // k<0>
  {
    V3<S> c = cross(dir, st.B_first);
    for (int i = 0; i < 3; ++i) st.k1[i] = qop * c[i];
  }
  S errorEstimate = S(0.0), h2 = S(0.0), half_h = S(0.0);
  auto scaling = [&](S err) -> S {
    S x = S(o.stepTolerance) / err;
    x = sqrt(sqrt(x));
    return std::clamp(x, S(0.25), S(4.0));
  };
  auto tryStep = [&](S h, bool& ok) -> bool {
    h2 = h * h;
    half_h = h * S(0.5);
    V3<S> pos1;
    for (int i = 0; i < 3; ++i) pos1[i] = pos[i] + half_h * dir[i] + h2 * S(0.125) * st.k1[i];
    if (!field.get(pos1, st.B_middle)) return false;
    V3<S> t;
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + half_h * st.k1[i];
    V3<S> c = cross(t, st.B_middle);
    for (int i = 0; i < 3; ++i) st.k2[i] = qop * c[i];
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + half_h * st.k2[i];
    c = cross(t, st.B_middle);
    for (int i = 0; i < 3; ++i) st.k3[i] = qop * c[i];
    V3<S> pos2;
    for (int i = 0; i < 3; ++i) pos2[i] = pos[i] + h * dir[i] + h2 * S(0.5) * st.k3[i];
    if (!field.get(pos2, st.B_last)) return false;
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + h * st.k3[i];
    c = cross(t, st.B_last);
    for (int i = 0; i < 3; ++i) st.k4[i] = qop * c[i];
    S l1 = S(0.0);
    for (int i = 0; i < 3; ++i) l1 = l1 + abs(((st.k1[i] - st.k2[i]) - st.k3[i]) + st.k4[i]);
    // kQoP is zero in the default extension
    errorEstimate = h2 * (l1 + abs(((S(0.0) - S(0.0)) - S(0.0)) + S(0.0)));
    errorEstimate = std::max(S(1e-20), errorEstimate);
    ok = errorEstimate <= S(4.0) * S(o.stepTolerance);
    return true;
  };
  const S initialH = S(st.stepSize.value() * propDir);  // EigenStepper.ipp:272
  S h = initialH;
  unsigned nStepTrials = 0;
  while (true) {
    ++nStepTrials;
    bool ok = false;
    if (!tryStep(h, ok)) return kStepField;
    if (ok) break;
    h = h * scaling(errorEstimate);
    if (abs(h) < abs(S(o.stepSizeCutOff))) return kStepStalled;
    if (nStepTrials > o.maxRungeKuttaStepTrials) return kStepAdjust;
  }
  // finalize: propagateTime + transportMatrix (DefaultExtension :86-228)
  const S m = S((double)st.mass);
  const S p = st.absoluteMomentum();
  {
    S mp = m / p;
    S dtds = sqrt(S(1.0) * S(1.0) + mp * mp);
    st.pars[3] = st.pars[3] + h * dtds;
    st.derivative[3] = dtds;
  }
  {
    S mp = m / p;
    S dtds = sqrt(S(1.0) * S(1.0) + mp * mp);
    Mat<S, 8, 8> D = Mat<S, 8, 8>::identity();
    S hh = h * S(0.5);
    Mat<S, 3, 3> dk1dT = Mat<S, 3, 3>::zero();
    Mat<S, 3, 3> dk2dT = Mat<S, 3, 3>::identity();
    Mat<S, 3, 3> dk3dT = Mat<S, 3, 3>::identity();
    Mat<S, 3, 3> dk4dT = Mat<S, 3, 3>::identity();
    V3<S> dk1dL = cross(dir, st.B_first);
    V3<S> t, c1, c2;
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * st.k1[i];
    c1 = cross(t, st.B_middle);
    c2 = cross(dk1dL, st.B_middle);
    V3<S> dk2dL;
    for (int i = 0; i < 3; ++i) dk2dL[i] = c1[i] + (qop * hh) * c2[i];
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + hh * st.k2[i];
    c1 = cross(t, st.B_middle);
    c2 = cross(dk2dL, st.B_middle);
    V3<S> dk3dL;
    for (int i = 0; i < 3; ++i) dk3dL[i] = c1[i] + (qop * hh) * c2[i];
    for (int i = 0; i < 3; ++i) t[i] = dir[i] + h * st.k3[i];
    c1 = cross(t, st.B_last);
    c2 = cross(dk3dL, st.B_last);
    V3<S> dk4dL;
    for (int i = 0; i < 3; ++i) dk4dL[i] = c1[i] + (qop * h) * c2[i];

    const V3<S>& B1 = st.B_first;
    dk1dT.a[0][1] = B1[2];
    dk1dT.a[0][2] = -B1[1];
    dk1dT.a[1][0] = -B1[2];
    dk1dT.a[1][2] = B1[0];
    dk1dT.a[2][0] = B1[1];
    dk1dT.a[2][1] = -B1[0];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dk1dT.a[i][j] = dk1dT.a[i][j] * qop;
    auto crossM = [](const Mat<S, 3, 3>& Mx, const V3<S>& v) {
      Mat<S, 3, 3> r;
      for (int j = 0; j < 3; ++j) {
        V3<S> cj{{Mx.a[0][j], Mx.a[1][j], Mx.a[2][j]}};
        V3<S> x = cross(cj, v);
        for (int i = 0; i < 3; ++i) r.a[i][j] = x[i];
      }
      return r;
    };
    auto axpyM = [](Mat<S, 3, 3>& Y, S a, const Mat<S, 3, 3>& X) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Y.a[i][j] = Y.a[i][j] + a * X.a[i][j];
    };
    auto scaleM = [](S a, const Mat<S, 3, 3>& X) {
      Mat<S, 3, 3> r;
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.a[i][j] = a * X.a[i][j];
      return r;
    };
    axpyM(dk2dT, hh, dk1dT);
    dk2dT = scaleM(qop, crossM(dk2dT, st.B_middle));
    axpyM(dk3dT, hh, dk2dT);
    dk3dT = scaleM(qop, crossM(dk3dT, st.B_middle));
    axpyM(dk4dT, h, dk3dT);
    dk4dT = scaleM(qop, crossM(dk4dT, st.B_last));

    // dFdT = (I + h/6 (dk1dT + dk2dT + dk3dT)) * h
    S h6 = h / S(6.0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        S id = (i == j) ? S(1.0) : S(0.0);
        S v = id + h6 * ((dk1dT.a[i][j] + dk2dT.a[i][j]) + dk3dT.a[i][j]);
        D.a[i][4 + j] = v * h;
      }
    S hh6 = (h * h) / S(6.0);
    for (int i = 0; i < 3; ++i) D.a[i][7] = hh6 * ((dk1dL[i] + dk2dL[i]) + dk3dL[i]);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        S v = ((dk1dT.a[i][j] + S(2.0) * (dk2dT.a[i][j] + dk3dT.a[i][j])) + dk4dT.a[i][j]);
        D.a[4 + i][4 + j] = D.a[4 + i][4 + j] + h6 * v;
      }
    for (int i = 0; i < 3; ++i)
      D.a[4 + i][7] = h6 * ((dk1dL[i] + S(2.0) * (dk2dL[i] + dk3dL[i])) + dk4dL[i]);
    D.a[3][7] = h * m * m / (p * p * qop * dtds);

    // blocked update of jacTransport (EigenStepper.ipp:310-352)
    Mat<S, 4, 4> D12, D22, J12, J22;
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        D12.a[i][j] = D.a[i][4 + j];
        D22.a[i][j] = D.a[4 + i][4 + j];
        J12.a[i][j] = st.jacTransport.a[i][4 + j];
        J22.a[i][j] = st.jacTransport.a[4 + i][4 + j];
      }
    Mat<S, 4, 4> t12 = mul(D12, J22);
    Mat<S, 4, 4> t22 = mul(D22, J22);
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        st.jacTransport.a[i][4 + j] = J12.a[i][j] + t12.a[i][j];
        st.jacTransport.a[4 + i][4 + j] = t22.a[i][j];
      }
  }
  // parameter update (EigenStepper.ipp:354-366)
  S hh6 = h2 / S(6.0);
  S h6 = h / S(6.0);
  for (int i = 0; i < 3; ++i)
    st.pars[i] = st.pars[i] + (h * dir[i] + hh6 * ((st.k1[i] + st.k2[i]) + st.k3[i]));
  for (int i = 0; i < 3; ++i)
    st.pars[4 + i] =
        st.pars[4 + i] + h6 * ((st.k1[i] + S(2.0) * (st.k2[i] + st.k3[i])) + st.k4[i]);
  {
    V3<S> d = st.dir();
    d = normalized(d);
    st.pars[4] = d[0];
    st.pars[5] = d[1];
    st.pars[6] = d[2];
  }
  st.derivative[0] = st.pars[4];
  st.derivative[1] = st.pars[5];
  st.derivative[2] = st.pars[6];
  st.derivative[4] = st.k4[0];
  st.derivative[5] = st.k4[1];
  st.derivative[6] = st.k4[2];
  st.pathAccumulated = st.pathAccumulated + h;
  ++st.nSteps;
  // step size accuracy update (EigenStepper.ipp:379-385)
  const S nextAccuracy = abs(h * scaling(errorEstimate));
  const S previousAccuracy = S(std::abs(st.stepSize.accuracy));
  const S initialStepLength = abs(initialH);
  if (nextAccuracy < initialStepLength || nextAccuracy > previousAccuracy)
    st.stepSize.accuracy = (double)nextAccuracy;
  hOut = h;
  return kStepOk;
}

// Eigen decomposition of a symmetric 8x8 matrix by cyclic Jacobi rotations
// (the free covariance is symmetric positive semi-definite, so its SVD
// U S U^T is this decomposition; Eigen::JacobiSVD is not available here).
// On return A holds the eigenvalues on its diagonal, V the eigenvectors in
// its columns.
template <typename S>
void jacobiEigen8(Mat<S, 8, 8>& A, Mat<S, 8, 8>& V) {
  using std::abs;
  using std::sqrt;
  V = Mat<S, 8, 8>::identity();
  for (int sweep = 0; sweep < 60; ++sweep) {
    S off = S(0.0), diag = S(0.0);
    for (int p = 0; p < 8; ++p) {
      diag = diag + A.a[p][p] * A.a[p][p];
      for (int q = p + 1; q < 8; ++q) off = off + A.a[p][q] * A.a[p][q];
    }
    if (!(off > S(1e-60) * diag)) break;
    for (int p = 0; p < 7; ++p)
      for (int q = p + 1; q < 8; ++q) {
        const S apq = A.a[p][q];
        if (apq == S(0.0)) continue;
        const S theta = (A.a[q][q] - A.a[p][p]) / (S(2.0) * apq);
        const S t = (theta >= S(0.0) ? S(1.0) : S(-1.0)) /
                    (abs(theta) + sqrt(theta * theta + S(1.0)));
        const S c = S(1.0) / sqrt(t * t + S(1.0)), sn = t * c;
        for (int k = 0; k < 8; ++k) {  // A <- A R (columns p, q)
          const S akp = A.a[k][p], akq = A.a[k][q];
          A.a[k][p] = c * akp - sn * akq;
          A.a[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 8; ++k) {  // A <- R^T A (rows p, q)
          const S apk = A.a[p][k], aqk = A.a[q][k];
          A.a[p][k] = c * apk - sn * aqk;
          A.a[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 8; ++k) {
          const S vkp = V.a[k][p], vkq = V.a[k][q];
          V.a[k][p] = c * vkp - sn * vkq;
          V.a[k][q] = sn * vkp + c * vkq;
        }
      }
  }
}

// detail::CorrectedFreeToBoundTransformer::operator()
// (Core/src/EventData/CorrectedTransformationFreeToBound.cpp:51-183) with the
// FreeToBoundCorrection defaults (alpha 0.1, beta 2, incidence cut-offs
// 1e-5 / 0.99500417; CorrectedTransformationFreeToBound.hpp:22-35): an
// unscented transform of the free covariance through free-to-bound, each
// shifted sigma point put back on the surface along its direction. False
// (no correction) outside the incidence window or when a transformation
// fails.
template <typename S>
bool correctedFreeToBound(const Vec<S, 8>& fp, const Mat<S, 8, 8>& freeCov, const Surface<S>& s,
                          Vec<S, 6>& mean, Mat<S, 6, 6>& cov) {
  using std::abs;
  using std::sqrt;
  const double alpha = 0.1, beta = 2.0, cosMin = 1e-5, cosMax = 0.99500417;
  V3<S> pos{{fp[0], fp[1], fp[2]}}, dir{{fp[4], fp[5], fp[6]}};
  const S absCos = abs(dot(dir, s.normal(pos)));
  if (absCos < S(cosMin) || absCos > S(cosMax)) return false;
  Mat<S, 8, 8> A = freeCov, U;
  jacobiEigen8(A, U);
  Mat<S, 8, 8> covSqrt;
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) covSqrt.a[i][j] = A.a[j][j] > S(0.0) ? U.a[i][j] * sqrt(A.a[j][j]) : S(0.0);
  const double kappa = alpha * alpha * 8.0, lambda = kappa - 8.0, gamma = std::sqrt(kappa);
  Vec<S, 6> b[17];
  double wm[17], wc[17];
  if (!freeToBound(fp, s, b[0])) return false;
  wm[0] = lambda / kappa;
  wc[0] = lambda / kappa + (1.0 - alpha * alpha + beta);
  for (int i = 0; i < 8; ++i)
    for (int sg = 0; sg < 2; ++sg) {
      const int k = 1 + 2 * i + sg;
      Vec<S, 8> p = fp;
      for (int r = 0; r < 8; ++r)
        p[r] = sg == 0 ? p[r] + covSqrt.a[r][i] * S(gamma) : p[r] - covSqrt.a[r][i] * S(gamma);
      // re-intersect along the sample's direction (forward), no bounds
      V3<S> pp{{p[0], p[1], p[2]}}, pd{{p[4], p[5], p[6]}};
      Intersection<S> is[2];
      const int n = s.intersect(pp, pd, S(kOnSurfaceTolerance), is);
      int best = -1;
      for (int j = 0; j < n; ++j) {
        if (is[j].status == IStatus::unreachable) continue;
        if (best < 0 || abs(is[j].pathLength) < abs(is[best].pathLength)) best = j;
      }
      if (best < 0) return false;
      for (int r = 0; r < 3; ++r) p[r] = pp[r] + is[best].pathLength * pd[r];
      if (!freeToBound(p, s, b[k])) return false;
      wm[k] = 0.5 / kappa;
      wc[k] = 0.5 / kappa;
    }
  for (int r = 0; r < 6; ++r) mean[r] = S(0.0);
  for (int k = 0; k < 17; ++k)
    for (int r = 0; r < 6; ++r) mean[r] = mean[r] + S(wm[k]) * b[k][r];
  cov = Mat<S, 6, 6>::zero();
  for (int k = 0; k < 17; ++k) {
    Vec<S, 6> d;
    for (int r = 0; r < 6; ++r) d[r] = b[k][r] - mean[r];
    for (int r = 0; r < 6; ++r)
      for (int c = 0; c < 6; ++c) cov.a[r][c] = cov.a[r][c] + S(wc[k]) * d[r] * d[c];
  }
  return true;
}

// CovarianceEngine.cpp:102-165 + JacobianEngine.cpp:19-45,122-141
template <typename S>
void transportCovarianceToBound(Stepper<S>& st, const Surface<S>& s, bool correction = false) {
  V3<S> pos = st.pos(), dir = st.dir();
  Vec<S, 8> fTP = s.freeToPathDerivative(pos, dir);
  Mat<S, 6, 8> F2B = s.freeToBoundJacobian(pos, dir);
  Mat<S, 8, 8> M = Mat<S, 8, 8>::identity();
  for (int i = 0; i < 8; ++i)
    for (int j = 0; j < 8; ++j) M.a[i][j] = M.a[i][j] + st.derivative[i] * fTP[j];
  Mat<S, 6, 8> A = mul(F2B, M);
  Mat<S, 6, 8> B = mul(A, st.jacTransport);
  st.jacobian = mul(B, st.jacToGlobal);
  bool corrected = false;
  if (correction) {
    // CovarianceEngine.cpp:120-144: the free covariance through the
    // unscented transform; the free parameters move to the corrected mean
    Mat<S, 8, 6> T = mul(st.jacTransport, st.jacToGlobal);
    Mat<S, 8, 8> freeCov = mul(mul(T, st.cov), transpose(T));
    Vec<S, 6> mean;
    Mat<S, 6, 6> bc;
    if (correctedFreeToBound(st.pars, freeCov, s, mean, bc)) {
      st.pars = boundToFree(s, mean);
      st.cov = bc;
      corrected = true;
      pos = st.pos();
      dir = st.dir();
    }
  }
  if (!corrected) st.cov = mul(mul(st.jacobian, st.cov), transpose(st.jacobian));
  // reinitializeJacobians: identity, zero, and the new boundToFree (only if
  // the position is on the surface; the result is ignored otherwise)
  st.jacTransport = Mat<S, 8, 8>::identity();
  st.derivative = Vec<S, 8>::zero();
  S loc[2];
  // (after the extrapolation to a line surface nothing steps on, so its
  // bound-to-free Jacobian, LineSurface.cpp:187-222, is not needed)
  if (s.type != CK_SURFACE_LINE && s.globalToLocal(pos, dir, S(kOnSurfaceTolerance), loc))
    st.jacToGlobal = s.boundToFreeJacobian(pos, dir);
}

// ------------------------------------------------------------ propagation
// Propagator<EigenStepper<>, VoidNavigator>::propagate(start[, target],
// options) (Propagator.ipp:25-260): EigenStepper::initialize from bound
// parameters on a plane, the stepping loop without navigation targets and
// actors, the aborters in list order after every step — SurfaceReached on
// the target (StandardAborters.hpp:66-155; its near limit -100 um) and
// PathLimitReached (StandardAborters.hpp:24-62) with the loop protection of
// LoopProtection.hpp:19-72 — and makeResult: the bound state on the target
// (CovarianceEngine.cpp:29-63) or the curvilinear state at the end point
// (CovarianceEngine.cpp:65-99, JacobianEngine.cpp:61-82, UnitVectors.hpp:
// 94-150). The direction is Direction::fromScalar(pathLimit).
struct PropResult {
  int status = CK_TRACK_OK;
  Vec<double, 6> params;
  Mat<double, 6, 6> cov, jacobian;
  double frame[12] = {0};  // the curvilinear end plane (no target)
  double pathLength = 0;
  int steps = 0;
};

template <typename S>
PropResult propagate(const Field<S>& field, const Options& o, const Surface<S>& start,
                     const Vec<S, 6>& startParams, const Mat<S, 6, 6>& startCov, float mass,
                     float absQ, const Surface<S>* target, double pathLimit) {
  using std::abs;
  PropResult r;
  const int propDir = pathLimit < 0 ? -1 : 1;
  Stepper<S> st;
  st.mass = mass;
  st.absQ = absQ;
  st.pars = boundToFree(start, startParams);
  st.cov = startCov;
  st.jacToGlobal = start.boundToFreeJacobian(st.pos(), st.dir());
  st.jacobian = Mat<S, 6, 6>::identity();
  st.jacTransport = Mat<S, 8, 8>::identity();
  st.derivative = Vec<S, 8>::zero();
  st.stepSize = ConstrainedStep();
  st.stepSize.accuracy = o.initialStepSize;
  st.stepSize.values[kUser] = o.maxStepSize;
  double limit = pathLimit;
  if (o.loopProtection) {
    V3<S> B;
    if (field.get(st.pos(), B)) {
      const double Bn = (double)norm(B);
      if (Bn != 0) {
        const double helix = propDir * 2 * kPi * (double)st.absoluteMomentum() / Bn;
        const double loop = o.loopFraction * helix;
        if (std::abs(loop) < std::abs(limit)) limit = loop;
      }
    }
  }
  auto checkAbort = [&]() -> bool {
    if (target) {
      V3<S> d = st.dir();
      for (int i = 0; i < 3; ++i) d[i] = S(double(propDir)) * d[i];
      Intersection<S> is[2];
      int n = target->intersect(st.pos(), d, S(o.surfaceTolerance), is);
      if (target->type == CK_SURFACE_LINE && n == 0) {
        is[0] = Intersection<S>{S(0.0), IStatus::unreachable};
        n = 1;
      }
      // MultiIntersection::closest (Intersection::closestOrder)
      int best = -1;
      for (int i = 0; i < n; ++i)
        if (is[i].valid() && (best < 0 || abs(is[i].pathLength) < abs(is[best].pathLength)))
          best = i;
      const bool reached = best >= 0 && is[best].status == IStatus::onSurface;
      for (int i = 0; i < n; ++i) {
        const double pl = (double)is[i].pathLength;
        if (is[i].valid() && pl > -0.1 &&
            pl < std::numeric_limits<double>::max() + kOnSurfaceTolerance) {
          // updateSingleSurfaceStatus (SteppingHelper.hpp:41-78)
          st.stepSize.release(kActor);
          st.stepSize.update(pl, kActor);
          break;
        }
      }
      if (reached) return true;
    }
    const double dist = std::abs(limit) - std::abs((double)st.pathAccumulated);
    if (std::abs(dist) < std::abs(o.surfaceTolerance)) return true;
    st.stepSize.update(dist, kActor);
    return false;
  };
  if (!checkAbort()) {
    bool terminated = false;
    for (unsigned s = 0; s < o.maxSteps; ++s) {
      S h;
      const int se = eigenStep(st, field, o, h, propDir);
      if (se != kStepOk) {
        r.status = se == kStepField ? CK_TRACK_FIELD_OUT_OF_BOUNDS
                                    : (se == kStepStalled ? CK_TRACK_STEP_SIZE_STALLED
                                                          : CK_TRACK_STEP_ADJUST_FAILED);
        return r;
      }
      st.stepSize.release(kNav);
      st.stepSize.release(kActor);
      if (checkAbort()) {
        terminated = true;
        break;
      }
    }
    if (!terminated) {
      r.status = CK_TRACK_STEP_COUNT_LIMIT;
      return r;
    }
  }
  Surface<S> end;
  bool curvilinear = false;
  if (target) {
    end = *target;
  } else {
    // the curvilinear frame (UnitVectors.hpp:94-150) at the end point
    const V3<S> d = st.dir();
    V3<S> u{{-d[1], d[0], S(0.0)}};
    const S sc = std::sqrt(u[0] * u[0] + u[1] * u[1]);
    if (sc < S(16.0 * std::numeric_limits<double>::epsilon())) {
      u[0] = S(1.0);
      u[1] = S(0.0);
    } else {
      u[0] = u[0] / sc;
      u[1] = u[1] / sc;
    }
    V3<S> v = normalized(cross(d, u));
    end.type = CK_SURFACE_PLANE;
    for (int i = 0; i < 3; ++i) {
      end.R[i][0] = u[i];
      end.R[i][1] = v[i];
      end.R[i][2] = d[i];
      end.c[i] = st.pars[i];
      r.frame[i * 3 + 0] = (double)u[i];
      r.frame[i * 3 + 1] = (double)v[i];
      r.frame[i * 3 + 2] = (double)d[i];
      r.frame[9 + i] = (double)st.pars[i];
    }
    curvilinear = true;
  }
  Vec<S, 6> bp;
  if (!freeToBound(st.pars, end, bp)) {
    r.status = CK_TRACK_NOT_ON_SURFACE;
    return r;
  }
  transportCovarianceToBound(st, end);
  if (curvilinear) bp[0] = bp[1] = S(0.0);
  for (int i = 0; i < 6; ++i) r.params[i] = (double)bp[i];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      r.cov.a[i][j] = (double)st.cov.a[i][j];
      r.jacobian.a[i][j] = (double)st.jacobian.a[i][j];
    }
  r.pathLength = (double)st.pathAccumulated;
  r.steps = st.nSteps;
  return r;
}

// -------------------------------------------------------------- KF output
struct TrackOut {
  int status = CK_TRACK_NOT_PROCESSED;
  int nStates = 0, nMeasurements = 0, nHoles = 0, nOutliers = 0, ndf = 0;
  double chi2 = 0;
  bool hasTrackParams = false;  // parameters at the reference surface
  double trackParams[6], trackCov[36];
  struct St {
    int surface;
    uint32_t flags;
    double pathLength, chi2;
    double pred[6], predCov[36], filt[6], filtCov[36], smth[6], smthCov[36], jac[36];
  };
  std::vector<St> states;
};

template <typename S>
struct MeasRec {
  int surface;
  int sub = CK_MEAS_LOC01;  // measured bound parameters (CK_MEAS_*)
  double v[2];              // measured values, packed (1D: v[0])
  double cov[4];            // covariance, packed row-major (1D: cov[0])
};

// Projector indices of a subspace mask (the measured local coordinates in
// increasing order) and its dimension.
inline int subspaceIndices(int sub, int idx[2]) {
  int n = 0;
  for (int i = 0; i < 2; ++i)
    if (sub & (1 << i)) idx[n++] = i;
  return n;
}

template <typename S>
void put6(double* d, const Vec<S, 6>& v) {
  for (int i = 0; i < 6; ++i) d[i] = (double)v[i];
}
template <typename S>
void put36(double* d, const Mat<S, 6, 6>& m) {
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) d[i * 6 + j] = (double)m.a[i][j];
}
template <typename S>
Vec<S, 6> get6(const double* d) {
  Vec<S, 6> v;
  for (int i = 0; i < 6; ++i) v[i] = S(d[i]);
  return v;
}
template <typename S>
Mat<S, 6, 6> get36(const double* d) {
  Mat<S, 6, 6> m;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) m.a[i][j] = S(d[i * 6 + j]);
  return m;
}

// Inverse of a 1x1 / 2x2 matrix as Eigen's fixed-size inverse computes it
// (reciprocal; adjugate over determinant).
template <typename S>
Mat<S, 1, 1> inverseSmall(const Mat<S, 1, 1>& m) {
  Mat<S, 1, 1> r;
  r.a[0][0] = S(1.0) / m.a[0][0];
  return r;
}
template <typename S>
Mat<S, 2, 2> inverseSmall(const Mat<S, 2, 2>& m) {
  return inverse2(m);
}

// Projector H (N x 6) with rows e_idx[k] (FixedBoundSubspaceHelper::projector)
template <typename S, int N>
Mat<S, N, 6> projector(const int idx[N]) {
  Mat<S, N, 6> H = Mat<S, N, 6>::zero();
  for (int k = 0; k < N; ++k) H.a[k][idx[k]] = S(1.0);
  return H;
}

template <typename S, int N>
Mat<S, N, N> measCovN(const double* mcov) {
  Mat<S, N, N> V;
  for (int r = 0; r < N; ++r)
    for (int c = 0; c < N; ++c) V.a[r][c] = S(mcov[r * N + c]);
  return V;
}

// GainMatrixUpdater::visitMeasurementImpl<N> (GainMatrixUpdaterImpl.hpp:21-91)
// for an N-dimensional measurement of the bound parameters idx[0..N-1];
// meas / mcov hold the N values and the N x N covariance, packed.
template <typename S, int N>
bool gainMatrixUpdateN(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const int idx[N],
                       const double* meas, const double* mcov, bool joseph, Vec<S, 6>& filt,
                       Mat<S, 6, 6>& F, S& chi2) {
  const Mat<S, N, 6> H = projector<S, N>(idx);
  const Mat<S, 6, N> Ht = transpose(H);
  const Mat<S, N, N> V = measCovN<S, N>(mcov);
  Mat<S, N, N> Sm = add(mul(mul(H, P), Ht), V);
  Mat<S, 6, N> K = mul(mul(P, Ht), inverseSmall(Sm));
  if (hasNaN(K)) return false;
  Vec<S, N> m;
  for (int k = 0; k < N; ++k) m[k] = S(meas[k]);
  Vec<S, N> Hp = mulv(H, pred);
  Vec<S, N> r;
  for (int k = 0; k < N; ++k) r[k] = m[k] - Hp[k];
  Vec<S, 6> Kr = mulv(K, r);
  for (int i = 0; i < 6; ++i) filt[i] = pred[i] + Kr[i];
  filt = normalizeBoundParameters(filt);
  Mat<S, 6, 6> tmp = sub(Mat<S, 6, 6>::identity(), mul(K, H));
  if (!joseph) {
    F = mul(tmp, P);
  } else {
    F = add(mul(mul(tmp, P), transpose(tmp)), mul(mul(K, V), transpose(K)));
  }
  Vec<S, N> Hf = mulv(H, filt);
  Vec<S, N> res;
  for (int k = 0; k < N; ++k) res[k] = m[k] - Hf[k];
  Mat<S, N, N> mm = mul(sub(Mat<S, N, N>::identity(), mul(H, K)), V);
  Mat<S, N, N> mi = inverseSmall(mm);
  // (r^T mi) r
  chi2 = S(0.0);
  for (int c = 0; c < N; ++c) {
    S t = S(0.0);
    for (int k = 0; k < N; ++k) t = t + res[k] * mi.a[k][c];
    chi2 = chi2 + t * res[c];
  }
  return true;
}

// the (loc0, loc1) case
template <typename S>
bool gainMatrixUpdate(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const double meas[2],
                      const double mcov[4], bool joseph, Vec<S, 6>& filt, Mat<S, 6, 6>& F,
                      S& chi2) {
  const int idx[2] = {0, 1};
  return gainMatrixUpdateN<S, 2>(pred, P, idx, meas, mcov, joseph, filt, F, chi2);
}

// the update of a source link of any supported subspace
template <typename S>
bool gainMatrixUpdateSub(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const MeasRec<S>& m,
                         bool joseph, Vec<S, 6>& filt, Mat<S, 6, 6>& F, S& chi2) {
  int idx[2] = {0, 1};
  if (subspaceIndices(m.sub, idx) == 1)
    return gainMatrixUpdateN<S, 1>(pred, P, idx, m.v, m.cov, joseph, filt, F, chi2);
  return gainMatrixUpdateN<S, 2>(pred, P, idx, m.v, m.cov, joseph, filt, F, chi2);
}

// calculatePredictedChi2 (TrackHelpers.hpp:563-694): residual m - H pred,
// residual covariance V + H P H^T, chi2 = (r^T R^-1) r
template <typename S, int N>
S predictedChi2N(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const int idx[N],
                 const double* meas, const double* mcov) {
  Vec<S, N> r;
  Mat<S, N, N> Rc;
  for (int k = 0; k < N; ++k) {
    r[k] = S(meas[k]) - pred[idx[k]];
    for (int c = 0; c < N; ++c) Rc.a[k][c] = S(mcov[k * N + c]) + P.a[idx[k]][idx[c]];
  }
  Mat<S, N, N> ri = inverseSmall(Rc);
  S chi2 = S(0.0);
  for (int c = 0; c < N; ++c) {
    S t = S(0.0);
    for (int k = 0; k < N; ++k) t = t + r[k] * ri.a[k][c];
    chi2 = chi2 + t * r[c];
  }
  return chi2;
}

template <typename S>
S predictedChi2(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const double meas[2],
                const double mcov[4]) {
  const int idx[2] = {0, 1};
  return predictedChi2N<S, 2>(pred, P, idx, meas, mcov);
}

template <typename S>
S predictedChi2Sub(const Vec<S, 6>& pred, const Mat<S, 6, 6>& P, const MeasRec<S>& m) {
  int idx[2] = {0, 1};
  if (subspaceIndices(m.sub, idx) == 1) return predictedChi2N<S, 1>(pred, P, idx, m.v, m.cov);
  return predictedChi2N<S, 2>(pred, P, idx, m.v, m.cov);
}

// GainMatrixSmoother::calculate (GainMatrixSmoother.cpp:18-97)
template <typename S>
bool smoothStep(const Vec<S, 6>& filt, const Mat<S, 6, 6>& Pf, const Vec<S, 6>& prevPred,
                const Mat<S, 6, 6>& prevPpred, const Mat<S, 6, 6>& prevJac,
                const Vec<S, 6>& prevSmth, const Mat<S, 6, 6>& prevPsmth, Vec<S, 6>& smth,
                Mat<S, 6, 6>& Psmth) {
  Mat<S, 6, 6> G = mul(mul(Pf, transpose(prevJac)), inverse(prevPpred));
  if (hasNaN(G)) return false;
  Vec<S, 6> d = subtractBoundParameters(prevSmth, prevPred);
  Vec<S, 6> Gd = mulv(G, d);
  for (int i = 0; i < 6; ++i) smth[i] = filt[i] + Gd[i];
  smth = normalizeBoundParameters(smth);
  Psmth = add(Pf, mul(mul(G, sub(prevPsmth, prevPpred)), transpose(G)));
  return true;
}

// MbfSmoother (modified Bryson-Frazier): MbfSmoother::calculateSmoothed
// (MbfSmoother.cpp:17-29) — smoothed covariance P_f - P_f Lambda P_f,
// smoothed parameters x_f - P_f lambda (normalised). When the state's
// smoothed storage is shared with its filtered storage (the last measurement
// state), the covariance is written first and the parameter update then
// reads the already smoothed covariance through the shared storage.
template <typename S>
void mbfSmoothed(const Vec<S, 6>& filt, const Mat<S, 6, 6>& Pf, const Mat<S, 6, 6>& L,
                 const Vec<S, 6>& l, bool shared, Vec<S, 6>& smth, Mat<S, 6, 6>& Ps) {
  Ps = sub(Pf, mul(mul(Pf, L), Pf));
  Vec<S, 6> Pl = mulv(shared ? Ps : Pf, l);
  for (int i = 0; i < 6; ++i) smth[i] = filt[i] - Pl[i];
  smth = normalizeBoundParameters(smth);
}

// MbfSmoother::visitNonMeasurement (MbfSmoother.cpp:31-38): holes, outliers
// and material states carry the lambdas through their Jacobian only.
template <typename S>
void mbfVisitNonMeasurement(const Mat<S, 6, 6>& F, Mat<S, 6, 6>& L, Vec<S, 6>& l) {
  L = mul(mul(transpose(F), L), F);
  l = mulv(transpose(F), l);
}

// MbfSmoother::visitMeasurementImpl<N> (MbfSmootherImpl.hpp:17-58) for an
// N-dimensional measurement of the bound parameters idx[0..N-1].
template <typename S, int N>
void mbfVisitMeasurementN(const Mat<S, 6, 6>& F, const Vec<S, 6>& pred, const Mat<S, 6, 6>& Pp,
                          const int idx[N], const double* meas, const double* mcov,
                          Mat<S, 6, 6>& L, Vec<S, 6>& l) {
  const Mat<S, N, 6> H = projector<S, N>(idx);
  const Mat<S, 6, N> Ht = transpose(H);
  const Mat<S, N, N> V = measCovN<S, N>(mcov);
  Mat<S, N, N> Sm = add(mul(mul(H, Pp), Ht), V);
  Mat<S, N, N> Si = inverseSmall(Sm);
  Mat<S, 6, N> K = mul(mul(Pp, Ht), Si);
  Mat<S, 6, 6> C = sub(Mat<S, 6, 6>::identity(), mul(K, H));
  Vec<S, N> Hp = mulv(H, pred);
  Vec<S, N> y;
  for (int k = 0; k < N; ++k) y[k] = S(meas[k]) - Hp[k];
  Mat<S, 6, 6> Lt = add(mul(mul(Ht, Si), H), mul(mul(transpose(C), L), C));
  Vec<S, 6> a = mulv(mul(Ht, Si), y);
  Vec<S, 6> b = mulv(transpose(C), l);
  Vec<S, 6> lt;
  for (int i = 0; i < 6; ++i) lt[i] = -a[i] + b[i];
  L = mul(mul(transpose(F), Lt), F);
  l = mulv(transpose(F), lt);
}

// the (loc0, loc1) case
template <typename S>
void mbfVisitMeasurement(const Mat<S, 6, 6>& F, const Vec<S, 6>& pred, const Mat<S, 6, 6>& Pp,
                         const double meas[2], const double mcov[4], Mat<S, 6, 6>& L,
                         Vec<S, 6>& l) {
  const int idx[2] = {0, 1};
  mbfVisitMeasurementN<S, 2>(F, pred, Pp, idx, meas, mcov, L, l);
}

template <typename S>
void mbfVisitMeasurementSub(const Mat<S, 6, 6>& F, const Vec<S, 6>& pred,
                            const Mat<S, 6, 6>& Pp, const MeasRec<S>& m, Mat<S, 6, 6>& L,
                            Vec<S, 6>& l) {
  int idx[2] = {0, 1};
  if (subspaceIndices(m.sub, idx) == 1)
    mbfVisitMeasurementN<S, 1>(F, pred, Pp, idx, m.v, m.cov, L, l);
  else
    mbfVisitMeasurementN<S, 2>(F, pred, Pp, idx, m.v, m.cov, L, l);
}

// The whole fit for one track: KalmanFitter::fit_impl / filter_impl
// (KalmanFitter.hpp:795-984), Actor::act / filter (:337-671), the
// Propagator stepping loop (Propagator.ipp:25-210) with the DirectNavigator
// (DirectNavigator.hpp:178-348) and detail::updateSingleSurfaceStatus
// (SteppingHelper.hpp:41-78).
template <typename S>
struct Fitter {
  const std::vector<Surface<S>>* surfaces;
  Field<S> field;
  MatConst mc;
  Options o;

  // one internal track state (VectorMultiTrajectory entry)
  struct IState {
    int surface;
    uint32_t flags;
    S pathLength;
    S chi2;
    Vec<S, 6> pred, filt, smth;
    Mat<S, 6, 6> predCov, filtCov, smthCov, jac;
    bool smoothedSharesFiltered = false;
    int measDim = 0;  // dimension of the state's measurement (ndf)
  };

  // PropagatorPlainOptions / StepperPlainOptions defaults
  // (PropagatorOptions.hpp:28-51, StepperOptions.hpp:36-49): the options of
  // the extrapolation (KalmanFitter.hpp:960-961 builds them afresh)
  static Options defaultPropagation() {
    Options d{};
    d.stepTolerance = 1e-4;
    d.stepSizeCutOff = 0.0;
    d.initialStepSize = 10000.0;
    d.maxStepSize = std::numeric_limits<double>::max();
    d.maxRungeKuttaStepTrials = 10000;
    d.maxSteps = 1000;
    d.maxTargetSkipping = 100;
    d.loopProtection = true;
    d.pathLimit = std::numeric_limits<double>::max();
    d.loopFraction = 0.5;
    d.surfaceTolerance = kOnSurfaceTolerance;
    d.nearLimit = -0.1;
    return d;
  }

  // extrapolateTrackToReferenceSurface (TrackHelpers.hpp:339-381): the start
  // state by the strategy (findTrackStateForExtrapolation, :175-300; first /
  // last state with a non-outlier measurement, its smoothed parameters), then
  // Propagator::propagate with ForcedSurfaceReached and PathLimitReached
  // (Propagator.ipp:25-210, StandardAborters.hpp:66-164) in the direction of
  // the straight-line distance, and the bound state on the target with the
  // transported covariance (Propagator.ipp:342-380).
  int extrapolate(const std::vector<IState>& states, int tip, float mass, float absQ, int absPdg,
                  TrackOut& out) const {
    using std::abs;
    const std::vector<Surface<S>>& sf = *surfaces;
    const Surface<S>& target = sf[o.referenceSurface];
    int first = -1, last = -1;
    for (int k = 0; k <= tip; ++k)
      if ((states[k].flags & CK_FLAG_HAS_MEASUREMENT) && !(states[k].flags & CK_FLAG_IS_OUTLIER)) {
        if (first < 0) first = k;
        last = k;
      }
    if (first < 0) return CK_TRACK_NO_COMPATIBLE_STATE;
    auto intersectFrom = [&](int k, S& path) -> bool {
      Vec<S, 8> f = boundToFree(sf[states[k].surface], states[k].smth);
      V3<S> pos{{f[0], f[1], f[2]}}, dir{{f[4], f[5], f[6]}};
      Intersection<S> is[2];
      const int n = target.intersect(pos, dir, S(kOnSurfaceTolerance), is);
      path = is[0].pathLength;
      return n > 0 && is[0].status != IStatus::unreachable;
    };
    int k = -1;
    S distance = S(0.0);
    if (o.referenceStrategy == CK_EXTRAPOLATE_FIRST || o.referenceStrategy == CK_EXTRAPOLATE_LAST) {
      k = o.referenceStrategy == CK_EXTRAPOLATE_FIRST ? first : last;
      if (!intersectFrom(k, distance)) return CK_TRACK_REFERENCE_UNREACHABLE;
    } else {
      S pf, pl;
      const bool vf = intersectFrom(first, pf), vl = intersectFrom(last, pl);
      const S inf = S(std::numeric_limits<double>::infinity());
      const S df = vf ? abs(pf) : inf, dl = vl ? abs(pl) : inf;
      if (vf && df <= dl) {
        k = first;
        distance = pf;
      } else if (vl && dl <= df) {
        k = last;
        distance = pl;
      } else {
        return CK_TRACK_REFERENCE_UNREACHABLE;
      }
    }
    const int propDir = distance >= S(0.0) ? 1 : -1;  // Direction::fromScalarZeroAsPositive
    const Options eo = defaultPropagation();
    const Surface<S>& from = sf[states[k].surface];
    Stepper<S> st;
    st.mass = mass;
    st.absQ = absQ;
    st.absPdg = absPdg;
    st.pars = boundToFree(from, states[k].smth);
    st.pathAccumulated = S(0.0);
    st.nSteps = 0;
    st.stepSize = ConstrainedStep();
    st.stepSize.accuracy = eo.initialStepSize;
    st.stepSize.values[kUser] = eo.maxStepSize;
    st.cov = states[k].smthCov;
    st.jacToGlobal = from.boundToFreeJacobian(st.pos(), st.dir());
    st.jacobian = Mat<S, 6, 6>::identity();
    st.jacTransport = Mat<S, 8, 8>::identity();
    st.derivative = Vec<S, 8>::zero();
    // loop protection of the path aborter (LoopProtection.hpp:19-72)
    double pathLimit = eo.pathLimit;
    {
      V3<S> B;
      if (field.get(st.pos(), B)) {
        const double Bn = (double)norm(B);
        if (Bn != 0) {
          const double ll = eo.loopFraction * (2 * kPi * (double)st.absoluteMomentum() / Bn);
          if (std::abs(ll) < std::abs(pathLimit)) pathLimit = ll;
        }
      }
    }
    // the aborters in list order; the first that fires ends the propagation
    auto checkAbort = [&]() -> bool {
      V3<S> d = st.dir();
      for (int i = 0; i < 3; ++i) d[i] = S(double(propDir)) * d[i];
      Intersection<S> is[2];
      const int n = target.intersect(st.pos(), d, S(eo.surfaceTolerance), is);
      const bool reached = n > 0 && is[0].status == IStatus::onSurface;
      if (n > 0 && is[0].status != IStatus::unreachable) {
        // updateSingleSurfaceStatus (SteppingHelper.hpp:41-78), Actor type
        st.stepSize.release(kActor);
        st.stepSize.update((double)is[0].pathLength, kActor);
      }
      if (reached) return true;
      const double dist = std::abs(pathLimit) - std::abs((double)st.pathAccumulated);
      if (std::abs(dist) < std::abs(eo.surfaceTolerance)) return true;
      st.stepSize.update(dist, kActor);
      return false;
    };
    if (!checkAbort()) {
      bool terminated = false;
      for (unsigned s = 0; s < eo.maxSteps; ++s) {
        S h;
        const int se = eigenStep(st, field, eo, h, propDir);
        if (se != kStepOk)
          return se == kStepField ? CK_TRACK_FIELD_OUT_OF_BOUNDS
                                  : (se == kStepStalled ? CK_TRACK_STEP_SIZE_STALLED
                                                        : CK_TRACK_STEP_ADJUST_FAILED);
        st.stepSize.release(kNav);
        st.stepSize.release(kActor);
        if (checkAbort()) {
          terminated = true;
          break;
        }
      }
      if (!terminated) return CK_TRACK_STEP_COUNT_LIMIT;
    }
    transportCovarianceToBound(st, target);
    Vec<S, 6> bp;
    if (!freeToBound(st.pars, target, bp)) return CK_TRACK_NOT_ON_SURFACE;
    put6(out.trackParams, bp);
    put36(out.trackCov, st.cov);
    out.hasTrackParams = true;
    return CK_TRACK_OK;
  }

  // The outcome of one filter pass (KalmanFitter::filter_impl,
  // KalmanFitter.hpp:794-848): its track states, the index of the last state
  // with a measurement, the number of non-outlier measurement states, and the
  // bound state on the target surface when the pass reached it
  // (KalmanFitter.hpp:398-412).
  struct Pass {
    std::vector<IState> states;
    int lastMeasurementIndex = -1;
    int measurementStates = 0;
    bool fitted = false;
    Vec<S, 6> fittedPars;
    Mat<S, 6, 6> fittedCov;
  };

  // One propagation of the Kalman actor along the surface sequence: forward
  // (propDir +1) from a start surface outside the sequence (startSid -2), or
  // backward (propDir -1) from the sequence surface startSid, which the
  // first actor call filters with its own measurement (the DirectNavigator
  // starts on it, DirectNavigator.hpp:238-262). `target` >= 0 is the
  // reversed pass's target surface (Actor::targetReached, a SurfaceReached
  // with an unlimited near limit, KalmanFitter.hpp:292, :384-412).
  int filterPass(const Surface<S>& startSurface, int startSid, const Vec<S, 6>& startPars,
                 const Mat<S, 6, 6>& startCov, float mass, float absQ, int absPdg,
                 const int* seq, int nSeq, const std::vector<MeasRec<S>>& meas, int propDir,
                 int target, Pass& p) const {
    using std::abs;
    const std::vector<Surface<S>>& sf = *surfaces;
    // measurement map (first source link per surface wins, :750-755)
    auto findMeas = [&](int sid) -> int {
      for (size_t i = 0; i < meas.size(); ++i)
        if (meas[i].surface == sid) return (int)i;
      return -1;
    };
    int nDistinct = 0;
    for (size_t i = 0; i < meas.size(); ++i) {
      bool dup = false;
      for (size_t j = 0; j < i; ++j) dup |= (meas[j].surface == meas[i].surface);
      nDistinct += dup ? 0 : 1;
    }
    // surfaces of the sequence that carry a source link: the early
    // termination points used when not coasting
    int lastSlSeq = -1, firstSlSeq = -1;
    for (int k = 0; k < nSeq; ++k)
      if (findMeas(seq[k]) >= 0) {
        lastSlSeq = k;
        if (firstSlSeq < 0) firstSlSeq = k;
      }

    Stepper<S> st;
    st.mass = mass;
    st.absQ = absQ;
    st.absPdg = absPdg;
    st.pars = boundToFree(startSurface, startPars);
    st.pathAccumulated = S(0.0);
    st.nSteps = 0;
    st.stepSize = ConstrainedStep();
    st.stepSize.accuracy = o.initialStepSize;
    st.stepSize.values[kUser] = o.maxStepSize;  // setUser
    st.cov = startCov;
    st.jacToGlobal = startSurface.boundToFreeJacobian(st.pos(), st.dir());
    st.jacobian = Mat<S, 6, 6>::identity();
    st.jacTransport = Mat<S, 8, 8>::identity();
    st.derivative = Vec<S, 8>::zero();

    // loop protection (LoopProtection.hpp:19-72)
    auto loopLimit = [&](double previous, bool release) -> double {
      double limit = previous;
      if (!o.loopProtection) return limit;
      if (release) limit = std::numeric_limits<double>::max();
      V3<S> B;
      if (!field.get(st.pos(), B)) return limit;
      double Bn = (double)norm(B);
      if (Bn == 0) return limit;
      double p = (double)st.absoluteMomentum();
      double helixPath = 1.0 * 2 * kPi * p / Bn;
      double ll = o.loopFraction * helixPath;
      if (std::abs(ll) < std::abs(limit)) limit = ll;
      return limit;
    };
    double propPathLimit = loopLimit(o.pathLimit, false);
    double kfPathLimit = std::numeric_limits<double>::max();

    // navigator state (DirectNavigator::initialize, DirectNavigator.hpp:
    // 238-262): the index before the start surface in the direction of
    // travel, or one end of the sequence when the start surface is not in it
    int surfaceIndex = propDir > 0 ? -1 : nSeq;
    for (int k = 0; startSid >= 0 && k < nSeq; ++k)
      if (seq[k] == startSid) {
        surfaceIndex = k - propDir;
        break;
      }
    bool navigationBreak = false;
    int currentSurface = startSid;  // -2: start surface, -1: none, >= 0: table id
    int targetSurf = -1, targetIdx = 0;
    bool haveTarget = false;
    // the direction the navigator and the aborters intersect along
    auto navDir = [&]() -> V3<S> {
      V3<S> d = st.dir();
      if (propDir < 0)
        for (int i = 0; i < 3; ++i) d[i] = -d[i];
      return d;
    };

    std::vector<IState>& states = p.states;
    int lastTrackIndex = -1, lastMeasurementIndex = -1;
    int measurementStates = 0;
    int missedActive = 0;
    bool finished = false;
    int err = CK_TRACK_OK;

    auto pathLimitCheck = [&](double limit) -> bool {
      double distance = std::abs(limit) - std::abs((double)st.pathAccumulated);
      if (std::abs(distance) < std::abs(o.surfaceTolerance)) return true;
      st.stepSize.update(distance, kActor);
      return false;
    };

    // boundState (CovarianceEngine.cpp:29-63)
    auto boundState = [&](const Surface<S>& s, bool transportCov, Vec<S, 6>& bp) -> bool {
      if (!freeToBound(st.pars, s, bp)) return false;
      if (transportCov) transportCovarianceToBound(st, s, o.freeToBoundCorrection);
      return true;
    };

    // PointwiseMaterialInteraction.hpp:162-274 ; mode factors from
    // ISurfaceMaterial.cpp:18-27 by the direction of travel; on the start
    // surface only the post-update part applies
    // (PointwiseMaterialInteraction.cpp:16-29)
    auto material = [&](int sid, const Surface<S>& s, int mode) -> bool {
      // mode: 0 none, 1 pre, 2 post, 3 full
      if (sid == startSid) mode &= 2;
      if (!s.hasMaterial) return true;
      V3<S> pos = st.pos(), dir = st.dir();
      S pc = s.pathCorrection(pos, dir);
      S loc[2];
      if (!s.globalToLocal(pos, st.dir(), S(kOnSurfaceTolerance), loc)) return false;
      Slab slab = s.slab;
      if (!slab.isVacuum()) {
        const double split = (double)s.splitFactor;
        const bool pre = mode == 1;
        double factor = mode == 0   ? 0.0
                        : mode == 3 ? 1.0
                                    : ((pre == (propDir > 0)) ? 1.0 - split : split);
        if (factor == 0.0) return true;  // MaterialSlab::Nothing()
        slab.scaleThickness((float)factor);
      }
      slab.scaleThickness((float)(double)pc);
      if (slab.isVacuum()) return true;
      const float qOverPf = (float)(double)st.qop();
      MatEffects e = computeMaterialEffects<S>(mc, slab, st.absPdg, (double)st.mass,
                                               (double)st.absQ, dir, qOverPf,
                                               o.multipleScattering, o.energyLoss);
      const double massd = (double)st.mass;
      const double absQd = (double)st.absQ;
      const double momentum = (double)st.absoluteMomentum();
      const double nextE = std::sqrt(massd * massd + momentum * momentum) - e.eLoss * double(propDir);
      double nextP = 0.0;
      if (massd < nextE) {
        double am = std::abs(massd);
        nextP = std::sqrt((nextE - am) * (nextE + am));
      }
      nextP = std::max(10 * kMeV, nextP);
      const float signedQ = (float)std::copysign(absQd, (double)qOverPf);
      st.pars[7] = S((double)signedQ / nextP);
      auto upd = [](S var, double change) { return S(std::max(0.0, (double)var + std::copysign(change, 1.0))); };
      st.cov.a[2][2] = upd(st.cov.a[2][2], e.variancePhi);
      st.cov.a[3][3] = upd(st.cov.a[3][3], e.varianceTheta);
      st.cov.a[4][4] = upd(st.cov.a[4][4], e.varianceQoverP);
      return true;
    };

    auto filter = [&](int sid) -> int {
      const Surface<S>& s = sf[sid];
      const bool precedingMeasurementExists = measurementStates > 0;
      const int mi = findMeas(sid);
      if (mi >= 0) {
        transportCovarianceToBound(st, s, o.freeToBoundCorrection);
        if (!material(sid, s, 1)) return CK_TRACK_NOT_ON_SURFACE;
        IState ts;
        ts.surface = sid;
        Vec<S, 6> bp;
        if (!boundState(s, false, bp)) return CK_TRACK_NOT_ON_SURFACE;
        ts.pred = bp;
        ts.predCov = st.cov;
        ts.jac = st.jacobian;
        ts.pathLength = st.pathAccumulated;
        ts.chi2 = S(0.0);
        uint32_t flags = CK_FLAG_HAS_PARAMETERS;
        if (s.hasMaterial) flags |= CK_FLAG_HAS_MATERIAL;
        const MeasRec<S>& m = meas[mi];
        ts.measDim = (m.sub & 1) + ((m.sub >> 1) & 1);
        bool outlier = false;
        if (o.outlierChi2Cut < std::numeric_limits<double>::infinity()) {
          S c2 = predictedChi2Sub(ts.pred, ts.predCov, m);
          outlier = c2 > S(o.outlierChi2Cut);
        }
        if (!outlier) {
          S c2;
          if (!gainMatrixUpdateSub(ts.pred, ts.predCov, m, o.josephs, ts.filt, ts.filtCov, c2))
            return CK_TRACK_UPDATE_FAILED;
          ts.chi2 = c2;
          flags |= CK_FLAG_HAS_MEASUREMENT;
        } else {
          flags |= CK_FLAG_HAS_MEASUREMENT | CK_FLAG_IS_OUTLIER;
          ts.filt = ts.pred;
          ts.filtCov = ts.predCov;
        }
        ts.flags = flags;
        states.push_back(ts);
        lastTrackIndex = (int)states.size() - 1;
        if (!outlier) {
          // stepper.update (EigenStepper.ipp:128-138)
          st.pars = boundToFree(s, ts.filt);
          st.cov = ts.filtCov;
          st.jacToGlobal = s.boundToFreeJacobian(st.pos(), st.dir());
          ++measurementStates;
        }
        if (!material(sid, s, 2)) return CK_TRACK_NOT_ON_SURFACE;
        lastMeasurementIndex = lastTrackIndex;
      } else if ((precedingMeasurementExists && s.sensitive) || s.hasMaterial) {
        IState ts;
        ts.surface = sid;
        Vec<S, 6> bp;
        if (!boundState(s, true, bp)) return CK_TRACK_NOT_ON_SURFACE;
        ts.pred = bp;
        ts.predCov = st.cov;
        ts.jac = st.jacobian;
        ts.pathLength = st.pathAccumulated;
        ts.chi2 = S(0.0);
        ts.filt = ts.pred;
        ts.filtCov = ts.predCov;
        uint32_t flags = CK_FLAG_HAS_PARAMETERS;
        if (s.hasMaterial) flags |= CK_FLAG_HAS_MATERIAL;
        if (s.sensitive && precedingMeasurementExists) {
          flags |= CK_FLAG_IS_HOLE;
          ++missedActive;
        }
        ts.flags = flags;
        states.push_back(ts);
        lastTrackIndex = (int)states.size() - 1;
        if (!material(sid, s, 3)) return CK_TRACK_NOT_ON_SURFACE;
      }
      return CK_TRACK_OK;
    };

    // KalmanFitter::Actor::act (:337-422) + the propagator's own path aborter
    auto act = [&]() -> int {
      if (finished) return CK_TRACK_OK;
      if (kfPathLimit == std::numeric_limits<double>::max()) kfPathLimit = loopLimit(kfPathLimit, true);
      if (currentSurface >= 0) {
        int r = filter(currentSurface);
        if (r != CK_TRACK_OK) return r;
      }
      bool complete = measurementStates == nDistinct;
      if (!o.coastAfterLastMeasurement && !complete && lastSlSeq >= 0 && currentSurface >= 0 &&
          (propDir > 0 ? surfaceIndex >= lastSlSeq : surfaceIndex <= firstSlSeq))
        complete = true;  // early termination: later states cannot join the track
      bool pathReached = pathLimitCheck(kfPathLimit);
      bool targetReached = false;
      if (target >= 0) {
        // SurfaceReached::checkAbort (StandardAborters.hpp:94-155): the
        // closest intersection decides; the first valid one in the (unlimited)
        // path window steers the actor step size
        const Surface<S>& ts = sf[target];
        Intersection<S> is[2];
        const int ni = ts.intersect(st.pos(), navDir(), S(o.surfaceTolerance), is);
        // Intersection::closestOrder (Intersection.hpp:132-149)
        auto closer = [](const Intersection<S>& a, const Intersection<S>& b) {
          if (!a.valid() && b.valid()) return false;
          if (a.valid() && !b.valid()) return true;
          return abs(a.pathLength) < abs(b.pathLength);
        };
        int closest = 0;
        for (int i = 1; i < ni; ++i)
          if (closer(is[i], is[closest])) closest = i;
        targetReached = ni > 0 && is[closest].status == IStatus::onSurface;
        for (int i = 0; i < ni; ++i)
          if (is[i].valid() &&
              (double)is[i].pathLength < std::numeric_limits<double>::max() + kOnSurfaceTolerance) {
            // updateSingleSurfaceStatus (SteppingHelper.hpp:41-78), Actor
            // step size: on surface or reachable, the same constraint
            st.stepSize.release(kActor);
            st.stepSize.update((double)is[i].pathLength, kActor);
            break;
          }
      }
      if (targetReached) {
        // stepper.boundState on the target with covariance transport
        Vec<S, 6> bp;
        if (!freeToBound(st.pars, sf[target], bp)) return CK_TRACK_NOT_ON_SURFACE;
        transportCovarianceToBound(st, sf[target]);
        p.fitted = true;
        p.fittedPars = bp;
        p.fittedCov = st.cov;
      }
      if (complete || pathReached || targetReached) finished = true;
      return CK_TRACK_OK;
    };
    auto checkAbort = [&]() -> bool {
      if (finished) return true;
      return pathLimitCheck(propPathLimit);
    };

    auto nextTargetNav = [&]() -> bool {
      currentSurface = -1;
      if (navigationBreak) return false;
      surfaceIndex += propDir;
      while (surfaceIndex >= 0 && surfaceIndex < nSeq) {
        const Surface<S>& s = sf[seq[surfaceIndex]];
        Intersection<S> is[2];
        int ni = s.intersect(st.pos(), navDir(), S(o.surfaceTolerance), is);
        for (int i = 0; i < ni; ++i) {
          S pl = is[i].pathLength;
          if (is[i].valid() && pl > S(o.nearLimit) &&
              pl < S(std::numeric_limits<double>::max()) + S(kOnSurfaceTolerance)) {
            targetSurf = seq[surfaceIndex];
            targetIdx = i;
            return true;
          }
        }
        surfaceIndex += propDir;
      }
      navigationBreak = true;
      return false;
    };
    // updateSingleSurfaceStatus, boundary tolerance Infinite
    auto surfaceStatus = [&](int sid, int idx) -> IStatus {
      Intersection<S> is[2];
      sf[sid].intersect(st.pos(), navDir(), S(o.surfaceTolerance), is);
      Intersection<S> x = is[idx];
      if (x.status == IStatus::onSurface) {
        st.stepSize.release(kNav);
        st.stepSize.update((double)x.pathLength, kNav);
        return IStatus::onSurface;
      }
      if (x.valid()) {
        st.stepSize.release(kNav);
        st.stepSize.update((double)x.pathLength, kNav);
        return IStatus::reachable;
      }
      return IStatus::unreachable;
    };
    auto getNextTarget = [&](int& e) -> bool {
      e = CK_TRACK_OK;
      for (unsigned i = 0; i < o.maxTargetSkipping; ++i) {
        if (!nextTargetNav()) return false;
        IStatus stt = surfaceStatus(targetSurf, targetIdx);
        if (stt == IStatus::onSurface) continue;
        if (stt == IStatus::reachable) return true;
      }
      e = CK_TRACK_NEXT_TARGET_LIMIT;
      return false;
    };

    // ---- Propagator::propagate
    err = act();
    if (err == CK_TRACK_OK && !checkAbort()) {
      currentSurface = -1;  // (set below by nextTarget)
      int e;
      haveTarget = getNextTarget(e);
      if (e != CK_TRACK_OK) err = e;
      bool terminated = false;
      unsigned steps = 0;
      for (; err == CK_TRACK_OK && steps < o.maxSteps; ++steps) {
        S h;
        int se = eigenStep(st, field, o, h, propDir);
        if (se != kStepOk) {
          err = se == kStepField ? CK_TRACK_FIELD_OUT_OF_BOUNDS
                                 : (se == kStepStalled ? CK_TRACK_STEP_SIZE_STALLED
                                                       : CK_TRACK_STEP_ADJUST_FAILED);
          break;
        }
        st.stepSize.release(kNav);
        st.stepSize.release(kActor);
        if (haveTarget) {
          // a branch restart keeps the previous branch's target
          // (DirectNavigator::checkTargetValid is always true) while the
          // sequence index restarts; with the index before the sequence
          // start no current surface is set (the reference's navSurface()
          // would throw there)
          IStatus post = surfaceStatus(targetSurf, targetIdx);
          if (post == IStatus::onSurface && !navigationBreak && surfaceIndex >= 0 &&
              surfaceIndex < nSeq)
            currentSurface = seq[surfaceIndex];
          if (post != IStatus::reachable) haveTarget = false;
        }
        err = act();
        if (err != CK_TRACK_OK) break;
        if (checkAbort()) {
          terminated = true;
          break;
        }
        if (!haveTarget) {
          st.stepSize.release(kNav);
          haveTarget = getNextTarget(e);
          if (e != CK_TRACK_OK) {
            err = e;
            break;
          }
        }
      }
      if (err == CK_TRACK_OK && !terminated) err = CK_TRACK_STEP_COUNT_LIMIT;
    }
    (void)missedActive;
    p.lastMeasurementIndex = lastMeasurementIndex;
    p.measurementStates = measurementStates;
    return err;
  }

  // ---------------------------------------------------- track finding (CKF)
  // A track state of the CKF's trajectory and a branch (TrackProxy: its tip
  // and summary counters).
  struct CkfState {
    int surface = -1, prev = -1, meas = -1;
    uint32_t flags = 0;
    S chi2 = S(0.0), pathLength = S(0.0);
    Vec<S, 6> pred, filt;
    Mat<S, 6, 6> predCov, filtCov, jac;
  };
  struct CkfBranch {
    int tip = -1;
    int nMeas = 0, nHoles = 0, nOutliers = 0, ndf = 0;
    S chi2 = S(0.0);
    bool hasParams = false;
    Vec<S, 6> params;
    Mat<S, 6, 6> cov;
  };
  struct CkfCuts {
    double chi2Cut, chi2CutOutlier;
    int maxCandidates, minMeasurements, maxHoles, maxOutliers, maxHolesAndOutliers;
    int target, maxStates, maxTracks, maxBranches;
    // the end of the seed's sequence ends a branch as the end of the world
    // ends it with the geometry Navigator (EndOfWorldReached)
    bool endOfWorld;
    // the target's bounds (0: unbounded): rectangle half lengths of a
    // plane, the half length in z of a cylinder
    double targetHalfX, targetHalfY, targetHalfZ;
  };
  // the event's measurements grouped by surface
  struct CkfMeas {
    const int* offsets;  // [n_surfaces + 1]
    const double* values;
    const double* cov;
    const int* sub;  // or nullptr
    MeasRec<S> get(int m, int sid) const {
      MeasRec<S> r;
      r.surface = sid;
      r.sub = sub ? sub[m] : CK_MEAS_LOC01;
      for (int c = 0; c < 2; ++c) r.v[c] = values[2 * (size_t)m + c];
      for (int c = 0; c < 4; ++c) r.cov[c] = cov[4 * (size_t)m + c];
      return r;
    }
  };

  // CombinatorialKalmanFilter::findTracks
  // (CombinatorialKalmanFilter.hpp:1191-1335) with the DirectNavigator over
  // `seq`: the propagation loop of Propagator.ipp:25-210 with the CKF actor
  // (Actor::act :322-448, filter :548-822, processNewTrackStates :836-898,
  // addNonSourcelinkState :900-946, reset :460-531), the default
  // TrackStateCreator (TrackStateCreator.hpp:89-296) with the
  // MeasurementSelector (MeasurementSelector.ipp:19-124, single cut bin) and
  // the examples' branch stopper (TrackFindingAlgorithm.cpp:203-261). The
  // propagator's step counter runs over all branches of the seed; the CKF's
  // path aborter is the loop protection alone (a stub replaces the
  // propagator's own). Returns CK_TRACK_OK or the error of the search.
  int ckfSeed(const Surface<S>& startSurface, const Vec<S, 6>& startPars,
              const Mat<S, 6, 6>& startCov, float mass, float absQ, int absPdg, const int* seq,
              int nSeq, const CkfMeas& M, const CkfCuts& cuts, std::vector<CkfState>& states,
              std::vector<CkfBranch>& tracks) const {
    using std::abs;
    const std::vector<Surface<S>>& sf = *surfaces;
    states.clear();
    tracks.clear();
    Stepper<S> st;
    st.mass = mass;
    st.absQ = absQ;
    st.absPdg = absPdg;
    // EigenStepper::initialize (EigenStepper.ipp:37-70)
    auto initialize = [&](const Surface<S>& s, const Vec<S, 6>& bp, const Mat<S, 6, 6>& c) {
      st.pars = boundToFree(s, bp);
      st.pathAccumulated = S(0.0);
      st.nSteps = 0;
      st.stepSize = ConstrainedStep();
      st.stepSize.accuracy = o.initialStepSize;
      st.stepSize.values[kUser] = o.maxStepSize;
      st.cov = c;
      st.jacToGlobal = s.boundToFreeJacobian(st.pos(), st.dir());
      st.jacobian = Mat<S, 6, 6>::identity();
      st.jacTransport = Mat<S, 8, 8>::identity();
      st.derivative = Vec<S, 8>::zero();
    };
    initialize(startSurface, startPars, startCov);

    auto loopLimit = [&]() -> double {
      double limit = std::numeric_limits<double>::max();  // (release)
      if (!o.loopProtection) return limit;
      V3<S> B;
      if (!field.get(st.pos(), B)) return limit;
      double Bn = (double)norm(B);
      if (Bn == 0) return limit;
      double ll = o.loopFraction * (2 * kPi * (double)st.absoluteMomentum() / Bn);
      if (std::abs(ll) < std::abs(limit)) limit = ll;
      return limit;
    };
    double pathLimit = std::numeric_limits<double>::max();
    bool pathLimitSet = false;
    auto pathLimitCheck = [&]() -> bool {
      double distance = std::abs(pathLimit) - std::abs((double)st.pathAccumulated);
      if (std::abs(distance) < std::abs(o.surfaceTolerance)) return true;
      st.stepSize.update(distance, kActor);
      return false;
    };

    // navigator (DirectNavigator.hpp:222-348)
    int surfaceIndex = -1;
    bool navigationBreak = false;
    int currentSurface = -1;  // the seed's plane is not in the table
    int targetSurf = -1, targetIdx = 0;
    bool haveTarget = false;
    auto nextTargetNav = [&]() -> bool {
      currentSurface = -1;
      if (navigationBreak) return false;
      ++surfaceIndex;
      while (surfaceIndex >= 0 && surfaceIndex < nSeq) {
        Intersection<S> is[2];
        const int ni = sf[seq[surfaceIndex]].intersect(st.pos(), st.dir(), S(o.surfaceTolerance), is);
        for (int i = 0; i < ni; ++i) {
          S pl = is[i].pathLength;
          if (is[i].valid() && pl > S(o.nearLimit) &&
              pl < S(std::numeric_limits<double>::max()) + S(kOnSurfaceTolerance)) {
            targetSurf = seq[surfaceIndex];
            targetIdx = i;
            return true;
          }
        }
        ++surfaceIndex;
      }
      navigationBreak = true;
      return false;
    };
    auto surfaceStatus = [&](int sid, int idx) -> IStatus {
      Intersection<S> is[2];
      sf[sid].intersect(st.pos(), st.dir(), S(o.surfaceTolerance), is);
      Intersection<S> x = is[idx];
      if (x.valid()) {
        st.stepSize.release(kNav);
        st.stepSize.update((double)x.pathLength, kNav);
      }
      return x.status;
    };
    auto getNextTarget = [&](int& e) -> bool {
      e = CK_TRACK_OK;
      for (unsigned i = 0; i < o.maxTargetSkipping; ++i) {
        if (!nextTargetNav()) return false;
        IStatus stt = surfaceStatus(targetSurf, targetIdx);
        if (stt == IStatus::onSurface) continue;
        if (stt == IStatus::reachable) return true;
      }
      e = CK_TRACK_NEXT_TARGET_LIMIT;
      return false;
    };

    // PointwiseMaterialInteraction (forward; mode 1 pre, 2 post); on the
    // navigator's start surface (the surface a branch restarts from) only
    // the post-update part applies (PointwiseMaterialInteraction.cpp:16-29)
    int startSid = -1;
    auto material = [&](int sid, const Surface<S>& s, int mode) -> bool {
      if (sid == startSid) mode &= 2;
      if (mode == 0 || !s.hasMaterial) return true;
      V3<S> pos = st.pos(), dir = st.dir();
      S pc = s.pathCorrection(pos, dir);
      S loc[2];
      if (!s.globalToLocal(pos, dir, S(kOnSurfaceTolerance), loc)) return false;
      Slab slab = s.slab;
      if (!slab.isVacuum()) {
        const double split = (double)s.splitFactor;
        const double factor = mode == 1 ? 1.0 - split : split;
        if (factor == 0.0) return true;
        slab.scaleThickness((float)factor);
      }
      slab.scaleThickness((float)(double)pc);
      if (slab.isVacuum()) return true;
      const float qOverPf = (float)(double)st.qop();
      MatEffects e = computeMaterialEffects<S>(mc, slab, st.absPdg, (double)st.mass,
                                               (double)st.absQ, dir, qOverPf,
                                               o.multipleScattering, o.energyLoss);
      const double massd = (double)st.mass;
      const double momentum = (double)st.absoluteMomentum();
      const double nextE = std::sqrt(massd * massd + momentum * momentum) - e.eLoss;
      double nextP = 0.0;
      if (massd < nextE) {
        double am = std::abs(massd);
        nextP = std::sqrt((nextE - am) * (nextE + am));
      }
      nextP = std::max(10 * kMeV, nextP);
      const float signedQ = (float)std::copysign((double)st.absQ, (double)qOverPf);
      st.pars[7] = S((double)signedQ / nextP);
      auto upd = [](S var, double change) { return S(std::max(0.0, (double)var + change)); };
      st.cov.a[2][2] = upd(st.cov.a[2][2], e.variancePhi);
      st.cov.a[3][3] = upd(st.cov.a[3][3], e.varianceTheta);
      st.cov.a[4][4] = upd(st.cov.a[4][4], e.varianceQoverP);
      return true;
    };

    std::vector<CkfBranch> active(1);
    bool finished = false;
    int err = CK_TRACK_OK;

    auto store = [&]() -> int {
      if ((int)tracks.size() >= cuts.maxTracks) return CK_TRACK_TOO_MANY_STATES;
      tracks.push_back(active.back());
      return CK_TRACK_OK;
    };
    // the examples' branch stopper: 0 continue, 1 stop and keep, 2 stop and drop
    auto stopper = [&](const CkfBranch& b) -> int {
      const bool tooMany = b.nHoles > cuts.maxHoles || b.nOutliers > cuts.maxOutliers ||
                           b.nHoles + b.nOutliers > cuts.maxHolesAndOutliers;
      if (!tooMany) return 0;
      return b.nMeas >= cuts.minMeasurements ? 1 : 2;
    };
    auto targetCheck = [&](bool& reached) {
      // SurfaceReached with an unlimited near limit (the actor's
      // targetReached, CombinatorialKalmanFilter.hpp:259;
      // StandardAborters.hpp:94-155): reached when the navigator's current
      // surface is the target, else when the closest intersection within
      // the target's bounds (BoundaryTolerance::None) is on the surface
      reached = false;
      if (cuts.target < 0) return;
      if (currentSurface == cuts.target) {
        reached = true;
        return;
      }
      const Surface<S>& ts = sf[cuts.target];
      Intersection<S> is[2];
      const int ni = ts.intersect(st.pos(), st.dir(), S(o.surfaceTolerance), is);
      for (int i = 0; i < ni; ++i) {
        if (!is[i].valid()) continue;
        V3<S> p;
        for (int k = 0; k < 3; ++k) p[k] = st.pos()[k] + is[i].pathLength * st.dir()[k];
        const V3<S> l = ts.toLocal3(p);
        bool inside = true;
        if (ts.type == CK_SURFACE_CYLINDER && cuts.targetHalfZ > 0)
          inside = abs((double)l[2]) < abs(cuts.targetHalfZ + o.surfaceTolerance);
        else if (ts.type == CK_SURFACE_PLANE && cuts.targetHalfX > 0 && cuts.targetHalfY > 0)
          inside = (double)l[0] >= -cuts.targetHalfX && (double)l[0] <= cuts.targetHalfX &&
                   (double)l[1] >= -cuts.targetHalfY && (double)l[1] <= cuts.targetHalfY;
        if (!inside) is[i].status = IStatus::unreachable;
      }
      int best = -1;
      for (int i = 0; i < ni; ++i)
        if (is[i].valid() && (best < 0 || abs(is[i].pathLength) < abs(is[best].pathLength)))
          best = i;
      reached = best >= 0 && is[best].status == IStatus::onSurface;
      for (int i = 0; i < ni; ++i)
        if (is[i].valid() &&
            (double)is[i].pathLength < std::numeric_limits<double>::max() + kOnSurfaceTolerance) {
          st.stepSize.release(kActor);
          st.stepSize.update((double)is[i].pathLength, kActor);
          break;
        }
    };
    // Actor::reset: the next active branch from its outermost state
    auto reset = [&]() -> int {
      if (active.empty()) {
        finished = true;
        return CK_TRACK_OK;
      }
      const CkfState& cs = states[active.back().tip];
      const Surface<S>& s = sf[cs.surface];
      initialize(s, cs.filt, cs.filtCov);
      currentSurface = cs.surface;
      surfaceIndex = -1;
      for (int k = 0; k < nSeq; ++k)
        if (seq[k] == cs.surface) {
          surfaceIndex = k - 1;
          break;
        }
      navigationBreak = false;
      startSid = cs.surface;
      if (!material(cs.surface, s, 2)) return CK_TRACK_NOT_ON_SURFACE;
      pathLimit = loopLimit();
      bool dummy;
      targetCheck(dummy);
      return CK_TRACK_OK;
    };
    auto filter = [&](int sid) -> int {
      const Surface<S>& s = sf[sid];
      if (!s.sensitive && !s.hasMaterial) return CK_TRACK_OK;  // passive
      if (!s.sensitive) return CK_TRACK_INVALID_INPUT;          // material-only
      transportCovarianceToBound(st, s);
      if (!material(sid, s, 1)) return CK_TRACK_NOT_ON_SURFACE;
      Vec<S, 6> bp;
      if (!freeToBound(st.pars, s, bp)) return CK_TRACK_NOT_ON_SURFACE;
      const int prevTip = active.back().tip;
      // TrackStateCreator + MeasurementSelector
      const int m0 = M.offsets[sid], m1 = M.offsets[sid + 1];
      struct Cand {
        int m;
        S chi2;
      };
      std::vector<Cand> cands;
      for (int m = m0; m < m1; ++m) {
        const MeasRec<S> mr = M.get(m, sid);
        if (mr.sub < CK_MEAS_LOC0 || mr.sub > CK_MEAS_LOC01) return CK_TRACK_INVALID_INPUT;
        cands.push_back({m, predictedChi2Sub(bp, st.cov, mr)});
      }
      std::vector<Cand> sel;
      bool isOutlier = false;
      if (!cands.empty()) {
        S minChi2 = S(std::numeric_limits<double>::max());
        int minIndex = -1;
        std::vector<Cand> passed;
        for (size_t i = 0; i < cands.size(); ++i) {
          if (cands[i].chi2 < minChi2) {
            minChi2 = cands[i].chi2;
            minIndex = (int)i;
          }
          if (!(cands[i].chi2 >= S(cuts.chi2Cut))) passed.push_back(cands[i]);
        }
        if (passed.empty()) {
          if (minChi2 < S(cuts.chi2CutOutlier)) {
            sel.push_back(cands[minIndex]);
            isOutlier = true;
          }
        } else {
          std::stable_sort(passed.begin(), passed.end(),
                           [](const Cand& a, const Cand& b) { return a.chi2 < b.chi2; });
          const size_t k = std::min(passed.size(), (size_t)cuts.maxCandidates);
          sel.assign(passed.begin(), passed.begin() + k);
        }
      }
      const uint32_t matFlag = s.hasMaterial ? CK_FLAG_HAS_MATERIAL : 0u;
      if (!sel.empty()) {
        // new states (the selected candidates in ascending chi2)
        const int first = (int)states.size();
        if (first + (int)sel.size() > cuts.maxStates) return CK_TRACK_TOO_MANY_STATES;
        for (const Cand& c : sel) {
          CkfState x;
          x.surface = sid;
          x.prev = prevTip;
          x.meas = c.m;
          x.flags = CK_FLAG_HAS_PARAMETERS | CK_FLAG_HAS_MEASUREMENT | matFlag |
                    (isOutlier ? CK_FLAG_IS_OUTLIER : 0u);
          x.chi2 = c.chi2;
          x.pathLength = st.pathAccumulated;
          x.pred = bp;
          x.predCov = st.cov;
          x.jac = st.jacobian;
          states.push_back(x);
        }
        // processNewTrackStates: the new branches from the worst candidate to
        // the best (the best on top of the stack)
        const CkfBranch root = active.back();
        active.pop_back();
        int onSurface = 0;
        for (int i = (int)sel.size() - 1; i >= 0; --i) {
          CkfBranch b = root;
          b.tip = first + i;
          CkfState& x = states[b.tip];
          if (isOutlier) {
            x.filt = x.pred;
            x.filtCov = x.predCov;
            ++b.nOutliers;
          } else {
            S c2;
            const MeasRec<S> m = M.get(x.meas, sid);
            if (!gainMatrixUpdateSub(x.pred, x.predCov, m, o.josephs, x.filt, x.filtCov, c2))
              return CK_TRACK_UPDATE_FAILED;
            x.chi2 = c2;
            ++b.nMeas;
            b.ndf += (m.sub & 1) + ((m.sub >> 1) & 1);
            b.chi2 = b.chi2 + c2;
          }
          if ((int)active.size() >= cuts.maxBranches) return CK_TRACK_TOO_MANY_STATES;
          active.push_back(b);
          const int r = stopper(b);
          if (r == 0) {
            ++onSurface;
          } else {
            if (r == 1) {
              const int e = store();
              if (e != CK_TRACK_OK) return e;
            }
            active.pop_back();
          }
        }
        if (onSurface == 0) return reset();
      } else {
        // a hole (a sensitive surface without a selected measurement)
        if ((int)states.size() >= cuts.maxStates) return CK_TRACK_TOO_MANY_STATES;
        CkfState x;
        x.surface = sid;
        x.prev = prevTip;
        x.flags = CK_FLAG_HAS_PARAMETERS | CK_FLAG_IS_HOLE | matFlag;
        x.pathLength = st.pathAccumulated;
        x.pred = bp;
        x.predCov = st.cov;
        x.jac = st.jacobian;
        x.filt = bp;
        x.filtCov = st.cov;
        states.push_back(x);
        CkfBranch& b = active.back();
        b.tip = (int)states.size() - 1;
        ++b.nHoles;
        const int r = stopper(b);
        if (r != 0) {
          if (r == 1) {
            const int e = store();
            if (e != CK_TRACK_OK) return e;
          }
          active.pop_back();
          return reset();
        }
      }
      const CkfState& cur = states[active.back().tip];
      if ((cur.flags & CK_FLAG_HAS_MEASUREMENT) && !(cur.flags & CK_FLAG_IS_OUTLIER)) {
        // stepper.update with the filtered parameters (EigenStepper.ipp:128-138)
        st.pars = boundToFree(s, cur.filt);
        st.cov = cur.filtCov;
        st.jacToGlobal = s.boundToFreeJacobian(st.pos(), st.dir());
      }
      if (!material(sid, s, 2)) return CK_TRACK_NOT_ON_SURFACE;
      return CK_TRACK_OK;
    };
    auto act = [&]() -> int {
      if (!pathLimitSet) {
        pathLimit = loopLimit();
        pathLimitSet = true;
      }
      if (currentSurface >= 0) {
        const int r = filter(currentSurface);
        if (r != CK_TRACK_OK) return r;
        if (finished) return CK_TRACK_OK;
      }
      const bool pathReached = pathLimitCheck();
      bool targetReached = false;
      targetCheck(targetReached);
      if (pathReached || targetReached) {
        if (!pathReached) {
          Vec<S, 6> bp;
          if (!freeToBound(st.pars, sf[cuts.target], bp)) return CK_TRACK_NOT_ON_SURFACE;
          transportCovarianceToBound(st, sf[cuts.target]);
          active.back().hasParams = true;
          active.back().params = bp;
          active.back().cov = st.cov;
          st.stepSize.release(kNav);
        }
        const int e = store();
        if (e != CK_TRACK_OK) return e;
        active.pop_back();
        return reset();
      }
      return CK_TRACK_OK;
    };

    // the navigator's next target (Propagator.ipp:79-96, 166-181); with
    // endOfWorld a branch whose navigator has no surface of the sequence
    // left ends there, kept, as EndOfWorldReached ends it in Actor::act
    // (CombinatorialKalmanFilter.hpp:392-436), and the next branch restarts
    auto nextTarget = [&](bool release) -> int {
      while (true) {
        if (!haveTarget) {
          if (release) st.stepSize.release(kNav);
          int e;
          haveTarget = getNextTarget(e);
          if (e != CK_TRACK_OK) return e;
        }
        if (!(cuts.endOfWorld && navigationBreak)) return CK_TRACK_OK;
        int e = store();
        if (e != CK_TRACK_OK) return e;
        active.pop_back();
        e = reset();
        if (e != CK_TRACK_OK || finished) return e;
        release = true;
      }
    };

    // ---- Propagator::propagate (Propagator.ipp:25-210)
    err = act();
    if (err == CK_TRACK_OK && !finished) {
      err = nextTarget(false);
      bool terminated = finished;
      unsigned steps = 0;
      for (; err == CK_TRACK_OK && !terminated && steps < o.maxSteps; ++steps) {
        S h;
        int se = eigenStep(st, field, o, h, 1);
        if (se != kStepOk) {
          err = se == kStepField ? CK_TRACK_FIELD_OUT_OF_BOUNDS
                                 : (se == kStepStalled ? CK_TRACK_STEP_SIZE_STALLED
                                                       : CK_TRACK_STEP_ADJUST_FAILED);
          break;
        }
        st.stepSize.release(kNav);
        st.stepSize.release(kActor);
        if (haveTarget) {
          // a branch restart keeps the previous branch's target
          // (DirectNavigator::checkTargetValid is always true) while the
          // sequence index restarts; with the index before the sequence
          // start no current surface is set (the reference's navSurface()
          // would throw there)
          IStatus post = surfaceStatus(targetSurf, targetIdx);
          if (post == IStatus::onSurface && !navigationBreak && surfaceIndex >= 0 &&
              surfaceIndex < nSeq)
            currentSurface = seq[surfaceIndex];
          if (post != IStatus::reachable) haveTarget = false;
        }
        err = act();
        if (err != CK_TRACK_OK) break;
        if (finished) {
          terminated = true;
          break;
        }
        err = nextTarget(true);
        if (err != CK_TRACK_OK) break;
        if (finished) {
          terminated = true;
          break;
        }
      }
      if (err == CK_TRACK_OK && !terminated) err = CK_TRACK_STEP_COUNT_LIMIT;
    }
    if (err != CK_TRACK_OK) tracks.clear();
    return err;
  }

  // KalmanFitter::fit_impl (KalmanFitter.hpp:860-985): the forward filter,
  // then either the smoother or the reversed filter, then the extrapolation
  // to the reference surface.
  int fit(const Surface<S>& startSurface, const Vec<S, 6>& startPars, const Mat<S, 6, 6>& startCov,
          float mass, float absQ, int absPdg, const int* seq, int nSeq,
          const std::vector<MeasRec<S>>& meas, TrackOut& out) const {
    auto findMeas = [&](int sid) -> int {
      for (size_t i = 0; i < meas.size(); ++i)
        if (meas[i].surface == sid) return (int)i;
      return -1;
    };
    Pass fwd;
    int err = filterPass(startSurface, -2, startPars, startCov, mass, absQ, absPdg, seq, nSeq, meas,
                         1, -1, fwd);
    out.states.clear();
    if (err != CK_TRACK_OK) {
      out.status = err;
      return err;
    }
    if (fwd.measurementStates == 0) {
      out.status = CK_TRACK_NO_MEASUREMENT_FOUND;
      return out.status;
    }
    std::vector<IState>& states = fwd.states;
    // the track: states 0..lastMeasurementIndex (linear chain)
    int tip = fwd.lastMeasurementIndex;
    int lastMeas = -1;
    for (int k = tip; k >= 0; --k)
      if ((states[k].flags & CK_FLAG_HAS_MEASUREMENT) && !(states[k].flags & CK_FLAG_IS_OUTLIER)) {
        lastMeas = k;
        break;
      }
    // shareFrom(Filtered -> Smoothed) on the last measurement state
    // (KalmanFitter.hpp:889-891)
    states[lastMeas].smth = states[lastMeas].filt;
    states[lastMeas].smthCov = states[lastMeas].filtCov;
    states[lastMeas].smoothedSharesFiltered = true;
    int status = CK_TRACK_OK;
    bool haveTrackParams = false;
    // KalmanFitter.hpp:897-900 with SimpleReverseFilteringLogic
    // (Examples/Algorithms/TrackFitting/src/KalmanFitterFunction.cpp:50-58)
    const bool reverse =
        o.reverseFiltering ||
        std::abs(1.0 / (double)states[lastMeas].filt[4]) <= o.reverseMomThreshold;
    if (reverse) {
      // KalmanFitter.hpp:901-945: filter backwards from the last measurement
      // state (its parameters, covariance scaled), towards the reference
      // surface; the first measurement state's smoothed parameters are the
      // reversed pass's last filtered ones. No other state has smoothed
      // parameters (NaN here).
      int first = -1;
      for (int k = 0; k <= tip && first < 0; ++k)
        if ((states[k].flags & CK_FLAG_HAS_MEASUREMENT) && !(states[k].flags & CK_FLAG_IS_OUTLIER))
          first = k;
      const IState& ls = states[lastMeas];
      Mat<S, 6, 6> c = ls.filtCov;
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) c.a[i][j] = c.a[i][j] * S(o.reverseCovScaling);
      Pass rev;
      int e = filterPass((*surfaces)[ls.surface], ls.surface, ls.filt, c, mass, absQ, absPdg, seq,
                         nSeq, meas, -1, o.referenceSurface, rev);
      if (e == CK_TRACK_OK && rev.measurementStates == 0) e = CK_TRACK_NO_MEASUREMENT_FOUND;
      int revLast = -1;
      for (int k = rev.lastMeasurementIndex; e == CK_TRACK_OK && k >= 0 && revLast < 0; --k)
        if ((rev.states[k].flags & CK_FLAG_HAS_MEASUREMENT) &&
            !(rev.states[k].flags & CK_FLAG_IS_OUTLIER))
          revLast = k;
      if (e == CK_TRACK_OK && rev.states[revLast].surface != states[first].surface)
        e = CK_TRACK_INCONSISTENT_STATES;
      if (e != CK_TRACK_OK) {
        out.status = e;
        return e;
      }
      const S nan = S(std::numeric_limits<double>::quiet_NaN());
      for (int k = 0; k <= tip; ++k)
        if (k != lastMeas)
          for (int i = 0; i < 6; ++i) {
            states[k].smth[i] = nan;
            for (int j = 0; j < 6; ++j) states[k].smthCov.a[i][j] = nan;
          }
      states[first].smth = rev.states[revLast].filt;
      states[first].smthCov = rev.states[revLast].filtCov;
      if (rev.fitted) {
        put6(out.trackParams, rev.fittedPars);
        put36(out.trackCov, rev.fittedCov);
        out.hasTrackParams = true;
        haveTrackParams = true;
      }
    } else {
      // the smoother starts by sharing the tip's filtered parameters
      states[tip].smth = states[tip].filt;
      states[tip].smthCov = states[tip].filtCov;
    }
    if (!reverse && o.smoother == CK_SMOOTHER_MBF) {
      // MbfSmoother::operator() (MbfSmoother.hpp:48-90): backwards from the
      // tip with zero lambdas; the first state updates no lambdas
      Mat<S, 6, 6> L = Mat<S, 6, 6>::zero();
      Vec<S, 6> l;
      for (int i = 0; i < 6; ++i) l[i] = S(0.0);
      for (int k = tip; k >= 0; --k) {
        IState& ts = states[k];
        Vec<S, 6> sm;
        Mat<S, 6, 6> Ps;
        mbfSmoothed(ts.filt, ts.filtCov, L, l, ts.smoothedSharesFiltered, sm, Ps);
        ts.smth = sm;
        ts.smthCov = Ps;
        if (ts.smoothedSharesFiltered) {
          ts.filt = sm;
          ts.filtCov = Ps;
        }
        if (k == 0) break;
        if ((ts.flags & CK_FLAG_HAS_MEASUREMENT) && !(ts.flags & CK_FLAG_IS_OUTLIER)) {
          const MeasRec<S>& m = meas[findMeas(ts.surface)];
          mbfVisitMeasurementSub(ts.jac, ts.pred, ts.predCov, m, L, l);
        } else {
          mbfVisitNonMeasurement(ts.jac, L, l);
        }
      }
    }
    // GainMatrixSmoother::operator() (GainMatrixSmoother.hpp:43-99)
    for (int k = tip - 1; k >= 0 && o.smoother != CK_SMOOTHER_MBF && !reverse; --k) {
      IState& ts = states[k];
      const IState& pv = states[k + 1];
      if (!smoothStep(ts.filt, ts.filtCov, pv.pred, pv.predCov, pv.jac, pv.smth, pv.smthCov,
                      ts.smth, ts.smthCov)) {
        status = CK_TRACK_SMOOTH_FAILED;
        break;
      }
      if (ts.smoothedSharesFiltered) {
        // smoothed storage is shared with filtered: writing it overwrites
        // the filtered parameters as well
        ts.filt = ts.smth;
        ts.filtCov = ts.smthCov;
      }
    }
    out.status = status;
    if (status != CK_TRACK_OK) return status;
    // calculateTrackQuantities (TrackHelpers.hpp:421-448)
    out.nStates = tip + 1;
    out.states.resize(tip + 1);
    for (int k = 0; k <= tip; ++k) {
      const IState& ts = states[k];
      TrackOut::St& o2 = out.states[k];
      o2.surface = ts.surface;
      o2.flags = ts.flags;
      o2.pathLength = (double)ts.pathLength;
      o2.chi2 = (double)ts.chi2;
      put6(o2.pred, ts.pred);
      put36(o2.predCov, ts.predCov);
      put6(o2.filt, ts.filt);
      put36(o2.filtCov, ts.filtCov);
      put6(o2.smth, ts.smth);
      put36(o2.smthCov, ts.smthCov);
      put36(o2.jac, ts.jac);
      if (ts.flags & CK_FLAG_IS_HOLE) {
        ++out.nHoles;
      } else if (ts.flags & CK_FLAG_IS_OUTLIER) {
        ++out.nOutliers;
      } else if (ts.flags & CK_FLAG_HAS_MEASUREMENT) {
        ++out.nMeasurements;
        out.chi2 += (double)ts.chi2;
        out.ndf += ts.measDim;
      }
    }
    if (o.referenceSurface >= 0 && !haveTrackParams) {
      // KalmanFitter.hpp:959-972: the fit fails when the extrapolation does
      const int e = extrapolate(states, tip, mass, absQ, absPdg, out);
      if (e != CK_TRACK_OK) {
        out.status = e;
        out.states.clear();
        out.nStates = out.nMeasurements = out.nHoles = out.nOutliers = out.ndf = 0;
        out.chi2 = 0;
        return e;
      }
    }
    return CK_TRACK_OK;
  }
};

}  // namespace kfo
