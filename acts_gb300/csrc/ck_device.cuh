// ck_device.cuh — device building blocks of the CudaKalman fitter.
//
// One track is fitted by one thread. Everything here is a __device__
// function on small register-resident arrays; the propagation scalar P is
// double (plain FP64 form) or float (mixed form). The Kalman update, the 2x2
// and 6x6 inverses and chi2 are always double.
//
// The algorithms restate the reference (paths relative to the acts repo):
//   EigenStepper RKN4 + transport   Core/include/Acts/Propagator/EigenStepper.ipp:168-388,
//                                   EigenStepperDefaultExtension.hpp:40-228
//   surfaces                        Core/src/Surfaces/{Plane,Cylinder}Surface.cpp, Surface.cpp:249-306
//   covariance transport            Core/src/Propagator/detail/CovarianceEngine.cpp:102-165,
//                                   JacobianEngine.cpp:19-45,122-141
//   material                        Core/src/Material/Interactions.cpp, PointwiseMaterialInteraction.*
//   GainMatrixUpdater               Core/include/Acts/TrackFitting/detail/GainMatrixUpdaterImpl.hpp:21-91
//   GainMatrixSmoother              Core/src/TrackFitting/GainMatrixSmoother.cpp:18-97
// GB300-specific reformulations (same mathematics, different evaluation):
//  * the 8x8 free transport Jacobian is never formed: the kernel transports
//    T = jacTransport * jacToGlobal (8x6), of which only the 21 entries in
//    rows 0-6 of the phi/theta/(q/p) columns change during a step;
//  * covariances are kept as packed symmetric 6x6 (21 entries);
//  * the bound-to-bound Jacobian is assembled from T with the sparsity of
//    the free-to-bound Jacobian and the path-derivative correction.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "ck_internal.h"

namespace ck {

#define CK_D __device__ __forceinline__

constexpr double kPi = 3.14159265358979323846;
constexpr double kOnSurfaceTolerance = 1e-4;
constexpr double kNotSet = 1.7976931348623157e308;  // DBL_MAX

// packed symmetric index (upper triangle, row-major)
CK_D constexpr int sidx(int i, int j) {
  return (i <= j) ? (i * 6 - (i * (i - 1)) / 2 + (j - i)) : (j * 6 - (j * (j - 1)) / 2 + (i - j));
}

// -------------------------------------------------------- periodic helpers
// Core/include/Acts/Utilities/detail/periodic.hpp:19-93
template <typename S>
CK_D S wrap_periodic(S value, S start, S range) {
  S diff = value - start;
  return ((S(0) <= diff) && (diff < range)) ? value : (value - range * floor(diff / range));
}
CK_D double radian_pos(double x) { return wrap_periodic<double>(x, 0.0, 2 * kPi); }
CK_D double radian_sym(double x) { return wrap_periodic<double>(x, -kPi, 2 * kPi); }
CK_D void normalizePhiTheta(double& phi, double& theta) {
  theta = radian_pos(theta);
  if (kPi < theta) {
    phi = phi + kPi;
    theta = 2 * kPi - theta;
  }
  phi = radian_sym(phi);
}

// ------------------------------------------------------------------ float
// Correctly rounded float logarithm shared with the CPU oracle.
CK_D float ck_logf(float x) { return (float)log((double)x); }
// The material physics' logarithm: correctly rounded (plain form, equal to
// the oracle's) or the FP32 logf (mixed form, within 2 ulp).
template <bool EXACT>
CK_D float mlogf(float x) {
  if constexpr (EXACT)
    return ck_logf(x);
  else
    return logf(x);
}
// Un-contracted float arithmetic: the reference evaluates its material
// physics in float without FMA; these intrinsics keep the device identical.
CK_D float fm(float a, float b) { return __fmul_rn(a, b); }
CK_D float fa(float a, float b) { return __fadd_rn(a, b); }
CK_D float fs(float a, float b) { return __fsub_rn(a, b); }
CK_D float fd(float a, float b) { return __fdiv_rn(a, b); }
CK_D float fsq(float a) { return __fsqrt_rn(a); }
CK_D double dm(double a, double b) { return __dmul_rn(a, b); }
CK_D double da(double a, double b) { return __dadd_rn(a, b); }

// ---------------------------------------------------------------- surface
template <typename P>
struct Surf {
  P R[9];
  P c[3];
  P radius;
  int type;
  CK_D void load(const DevSurface* __restrict__ s) {
    if constexpr (sizeof(P) == sizeof(float)) {
#pragma unroll
      for (int i = 0; i < 9; ++i) R[i] = __ldg(&s->Rf[i]);
#pragma unroll
      for (int i = 0; i < 3; ++i) c[i] = __ldg(&s->cf[i]);
      radius = __ldg(&s->radiusf);
    } else {
#pragma unroll
      for (int i = 0; i < 9; ++i) R[i] = (P)__ldg(&s->R[i]);
#pragma unroll
      for (int i = 0; i < 3; ++i) c[i] = (P)__ldg(&s->c[i]);
      radius = (P)__ldg(&s->radius);
    }
    type = __ldg(&s->type);
  }
  CK_D void loadPlane(const double* __restrict__ f12) {
#pragma unroll
    for (int i = 0; i < 9; ++i) R[i] = (P)f12[i];
#pragma unroll
    for (int i = 0; i < 3; ++i) c[i] = (P)f12[9 + i];
    radius = P(0);
    type = CK_SURFACE_PLANE;
  }
  // R^T (p - c)
  CK_D void toLocal3(const P p[3], P l[3]) const {
    P d0 = p[0] - c[0], d1 = p[1] - c[1], d2 = p[2] - c[2];
#pragma unroll
    for (int j = 0; j < 3; ++j) l[j] = R[0 * 3 + j] * d0 + R[1 * 3 + j] * d1 + R[2 * 3 + j] * d2;
  }
  CK_D void toGlobal3(const P l[3], P g[3]) const {
#pragma unroll
    for (int i = 0; i < 3; ++i) g[i] = (R[i * 3 + 0] * l[0] + R[i * 3 + 1] * l[1] + R[i * 3 + 2] * l[2]) + c[i];
  }
};

// ------------------------------------ FP64 <-> FP32 on the integer pipes
// On GB300 a conversion between double and float issues to the FP64 unit
// (one warp instruction holds it ~16 clocks, like an FP64 FMA), and the
// mixed form converts a few thousand values per track between its FP64 free
// state and its FP32 stages. d2f / f2d do the conversions with integer
// instructions on the bit patterns: they give cvt.rn.f32.f64 /
// cvt.f64.f32 results bit for bit for normal values and signed zero; other
// inputs (subnormal results, overflow to inf, inf, nan) take the hardware
// conversion.
CK_D float d2f(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u > 253u) {  // float exponent e - 896 outside [1, 254]
    if (e == 0u && ((hi & 0xfffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    return __double2float_rn(x);
  }
  const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // 23 mantissa bits
  const unsigned r = lo & 0x1fffffffu;                      // 29 bits rounded off
  unsigned f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
  // to nearest, ties to even; a carry out of the mantissa is the correct
  // next binade (or inf above the largest float)
  f += (r > 0x10000000u || (r == 0x10000000u && (m & 1u))) ? 1u : 0u;
  return __uint_as_float(f);
}
CK_D double f2d(float y) {
  const unsigned u = __float_as_uint(y);
  const unsigned e = (u >> 23) & 0xffu;
  if (e - 1u > 253u) {  // zero, subnormal, inf or nan
    if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
    return (double)y;
  }
  const unsigned hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hi, (int)(u << 29));
}
// double -> P (the form's stage type) and P -> double. toP / toD are the
// hardware conversions: in the forward filter the integer sequences (with
// their branch for the rare operands) cost more than they save (measured:
// the uneven workload's mixed filter 19.4 -> 23.6 ms), because they split the
// straight-line code the scheduler interleaves. The smoother, whose
// conversions sit between long FP64 sequences, uses the integer ones
// (toPi / toDi; its kernel 4.17 -> 3.75 ms on 500k barrel tracks).
template <typename P>
CK_D P toP(double x) {
  return (P)x;
}
CK_D double toD(float y) { return (double)y; }
CK_D double toD(double y) { return y; }
template <typename P>
CK_D P toPi(double x) {
  if constexpr (sizeof(P) == sizeof(float))
    return d2f(x);
  else
    return x;
}
CK_D double toDi(float y) { return f2d(y); }
CK_D double toDi(double y) { return y; }

// ------------------------------------------- FP64 functions of the mixed form
// 1/sqrt(v): FP32 estimate refined by one FP64 Newton step (~1e-14 relative).
CK_D double rsqrtRefined(double v) {
  const double y = toD(rsqrtf(d2f(v)));
  return y * (1.5 - 0.5 * v * y * y);
}

// atan2 in FP64 by table-driven argument reduction: an FP32 atan2 picks the
// nearest reference angle a_k = k pi/64; the vector (x, y) is rotated by -a_k
// with the tabulated (cos a_k, sin a_k), so the residual angle d satisfies
// |d| < pi/128 + 1e-6; d = atan(t), t = y'/x' (FP32 reciprocal refined by
// FP64 Newton and residual steps), from the odd Taylor series of atan to
// t^11 (truncation below 1e-19 relative); result a_k + d, wrapped to [-pi, pi].
// Agrees with a correctly rounded atan2 to a few ulp.
CK_D double atan2Table(double y, double x, const double2* __restrict__ tab) {
  const float f = atan2f(d2f(y), d2f(x));
  int k = __float2int_rn(f * (float)(1.0 / kTrigStep));
  k = k < -64 ? -64 : (k > 64 ? 64 : k);
  const double2 cs = __ldg(&tab[k + 64]);
  const double xr = x * cs.x + y * cs.y;
  const double yr = y * cs.x - x * cs.y;
  if (!(xr > 0.0)) return (double)f;  // only for (x, y) = (0, 0)
  double r = toD(1.0f / d2f(xr));
  r = r * (2.0 - xr * r);
  double t = yr * r;
  t = t + r * (yr - xr * t);
  const double t2 = t * t;
  const double d =
      t * (1.0 + t2 * (-1.0 / 3 + t2 * (1.0 / 5 + t2 * (-1.0 / 7 + t2 * (1.0 / 9 + t2 * (-1.0 / 11))))));
  double a = (double)k * kTrigStep + d;
  if (a > kPi) a -= 2 * kPi;
  if (a < -kPi) a += 2 * kPi;
  return a;
}

// intersection status: 0 unreachable, 1 reachable, 2 on surface
template <typename P>
CK_D int statusOf(P path, P tol) {
  return (fabs(path) < fabs(tol)) ? 2 : 1;
}

// Surface::intersect with BoundaryTolerance::Infinite. Returns the number of
// entries (1 for planes, 2 for cylinders), ordered by path length.
template <typename P>
CK_D int intersect(const Surf<P>& s, const P pos[3], const P dir[3], P tol, P path[2], int st[2]) {
  if (s.type == CK_SURFACE_PLANE) {
    // PlanarHelper.hpp:56-77
    P n0 = s.R[2], n1 = s.R[5], n2 = s.R[8];
    P denom = dir[0] * n0 + dir[1] * n1 + dir[2] * n2;
    if (denom == P(0)) {
      path[0] = P(0);
      st[0] = 0;
      return 1;
    }
    P pl = (n0 * (s.c[0] - pos[0]) + n1 * (s.c[1] - pos[1]) + n2 * (s.c[2] - pos[2])) / denom;
    path[0] = pl;
    st[0] = statusOf(pl, tol);
    return 1;
  }
  // CylinderSurface::intersectionSolver + RealQuadraticEquation
  P a0 = s.R[2], a1 = s.R[5], a2 = s.R[8];  // symmetry axis
  P pc0 = pos[0] - s.c[0], pc1 = pos[1] - s.c[1], pc2 = pos[2] - s.c[2];
  P px0 = pc1 * a2 - pc2 * a1, px1 = pc2 * a0 - pc0 * a2, px2 = pc0 * a1 - pc1 * a0;
  P lx0 = dir[1] * a2 - dir[2] * a1, lx1 = dir[2] * a0 - dir[0] * a2, lx2 = dir[0] * a1 - dir[1] * a0;
  P a = lx0 * lx0 + lx1 * lx1 + lx2 * lx2;
  P b = P(2) * (lx0 * px0 + lx1 * px1 + lx2 * px2);
  P cc = (px0 * px0 + px1 * px1 + px2 * px2) - s.radius * s.radius;
  P disc = b * b - P(4) * a * cc;
  if (!(disc >= P(0))) {
    st[0] = st[1] = 0;
    path[0] = path[1] = P(0);
    return 2;
  }
  P sq = sqrt(disc);
  P q = P(-0.5) * (b + (b > P(0) ? sq : -sq));
  P first = q / a;
  if (disc == P(0)) {
    path[0] = path[1] = first;
    st[0] = st[1] = statusOf(first, tol);
    return 2;
  }
  P second = cc / q;
  if (first <= second) {
    path[0] = first;
    path[1] = second;
  } else {
    path[0] = second;
    path[1] = first;
  }
  st[0] = statusOf(path[0], tol);
  st[1] = statusOf(path[1], tol);
  return 2;
}

// Surface::intersect for the mixed form: position and direction in FP64.
// The plane distance n.(c - x) and the cylinder's |x_perp|^2 - R^2 (the
// quantities that cancel near the surface) are formed in FP64; the quadratic
// is solved in FP32 (root nearest to zero as c/q) and each root is refined
// by one Newton step on the FP64 quadratic, so the path to the surface is
// FP64-accurate (the final step lands on the surface as in the plain form).
// `coarse`: a root beyond this path length (of a quadratic with well
// separated roots) keeps its FP32 value, unrefined. The navigator passes
// twice its accuracy step size plus 1 mm: such a root is neither on the
// surface nor the binding step-size constraint, refined or not, so the
// propagation is the same.
CK_D int intersectMixed(const Surf<double>& s, const double pos[3], const double dir[3],
                        double tol, double path[2], int st[2], double coarse = kNotSet) {
  // (finite roots only; the default refines every root)
  const bool useCoarse = coarse < 1e30;
  const float farf = useCoarse ? d2f(coarse) : 0.0f;
  auto isFar = [&](float t) { return useCoarse && t > farf && t <= 3.4e38f; };
  // (every multiply-add is an explicit fma and every product feeding an add an
  // explicit __dmul_rn, so that the roundings do not depend on the kernel
  // instance the code is inlined into)
  if (s.type == CK_SURFACE_PLANE) {
    const double denom = fma(dir[2], s.R[8], fma(dir[1], s.R[5], __dmul_rn(dir[0], s.R[2])));
    if (denom == 0.0) {
      path[0] = 0.0;
      st[0] = 0;
      return 1;
    }
    const double num = fma(s.R[8], s.c[2] - pos[2],
                           fma(s.R[5], s.c[1] - pos[1], __dmul_rn(s.R[2], s.c[0] - pos[0])));
    // FP32 quotient refined by one FP64 residual step
    const float denomf = d2f(denom);
    const float p0f = d2f(num) / denomf;
    const double p0 = toD(p0f);
    const double pl = isFar(p0f) ? p0 : p0 + toD(d2f(fma(-p0, denom, num)) / denomf);
    path[0] = pl;
    st[0] = statusOf(pl, tol);
    return 1;
  }
  double ad, bd, ccd;
  const double r2 = __dmul_rn(s.radius, s.radius);
  if (s.R[2] == 0.0 && s.R[5] == 0.0 && s.R[8] == 1.0) {
    // axis along global z: the cross products with the axis are
    // (pc1, -pc0, 0) and (dir1, -dir0, 0); the same roundings as the general
    // expressions below give for this axis
    const double pc0 = pos[0] - s.c[0], pc1 = pos[1] - s.c[1];
    ad = fma(dir[0], dir[0], __dmul_rn(dir[1], dir[1]));
    bd = 2.0 * fma(dir[0], pc0, __dmul_rn(dir[1], pc1));
    ccd = fma(pc0, pc0, __dmul_rn(pc1, pc1)) - r2;
  } else {
    const double a0 = s.R[2], a1 = s.R[5], a2 = s.R[8];
    const double pc0 = pos[0] - s.c[0], pc1 = pos[1] - s.c[1], pc2 = pos[2] - s.c[2];
    const double px0 = fma(pc1, a2, -__dmul_rn(pc2, a1)), px1 = fma(pc2, a0, -__dmul_rn(pc0, a2)),
                 px2 = fma(pc0, a1, -__dmul_rn(pc1, a0));
    const double lx0 = fma(dir[1], a2, -__dmul_rn(dir[2], a1)),
                 lx1 = fma(dir[2], a0, -__dmul_rn(dir[0], a2)),
                 lx2 = fma(dir[0], a1, -__dmul_rn(dir[1], a0));
    ad = fma(lx2, lx2, fma(lx1, lx1, __dmul_rn(lx0, lx0)));
    bd = 2.0 * fma(lx2, px2, fma(lx1, px1, __dmul_rn(lx0, px0)));
    ccd = fma(px2, px2, fma(px1, px1, __dmul_rn(px0, px0))) - r2;
  }
  const float a = d2f(ad), b = d2f(bd), cc = d2f(ccd);
  const float disc = fmaf(b, b, -__fmul_rn(4.0f * a, cc));
  if (!(disc >= 0.0f)) {
    st[0] = st[1] = 0;
    path[0] = path[1] = 0.0;
    return 2;
  }
  const float sq = sqrtf(disc);
  const float q = -0.5f * (b + (b > 0.0f ? sq : -sq));
  // roots apart by more than 1 % of |b| / a: each FP32 root within ~1e-5 of its
  // value, far from the other
  const bool separated = disc > 1e-4f * (b * b);
  auto refine = [&](float t0f) -> double {
    if (separated && isFar(t0f)) return toD(t0f);
    const double t0 = toD(t0f);
    const double f = fma(fma(ad, t0, bd), t0, ccd);
    const double df = fma(2.0 * ad, t0, bd);
    return df != 0.0 ? t0 - toD(d2f(f) / d2f(df)) : t0;
  };
  const double first = refine(q / a);
  if (disc == 0.0f) {
    path[0] = path[1] = first;
    st[0] = st[1] = statusOf(first, tol);
    return 2;
  }
  const double second = refine(cc / q);
  if (first <= second) {
    path[0] = first;
    path[1] = second;
  } else {
    path[0] = second;
    path[1] = first;
  }
  st[0] = statusOf(path[0], tol);
  st[1] = statusOf(path[1], tol);
  return 2;
}

// Surface::globalToLocal (PlaneSurface.cpp:77-86, CylinderSurface.cpp:125-145)
template <typename P>
CK_D bool globalToLocal(const Surf<P>& s, const P pos[3], double tol, P loc[2]) {
  P l[3];
  s.toLocal3(pos, l);
  if (s.type == CK_SURFACE_PLANE) {
    if (fabs((double)l[2]) > fabs(tol)) return false;
    loc[0] = l[0];
    loc[1] = l[1];
    return true;
  }
  double inttol = tol;
  if (tol == kOnSurfaceTolerance) inttol = (double)s.radius * 0.0001;
  if (inttol < 0.01) inttol = 0.01;
  P r = sqrt(l[0] * l[0] + l[1] * l[1]);
  if (fabs((double)(r - s.radius)) > inttol) return false;
  loc[0] = s.radius * atan2(l[1], l[0]);
  loc[1] = l[2];
  return true;
}

// Surface::localToGlobal (PlaneSurface.cpp:72-75, CylinderSurface.cpp:116-123)
template <typename P>
CK_D void localToGlobal(const Surf<P>& s, const P loc[2], P g[3]) {
  P l[3];
  if (s.type == CK_SURFACE_PLANE) {
    l[0] = loc[0];
    l[1] = loc[1];
    l[2] = P(0);
  } else {
    P phi = loc[0] / s.radius;
    P sp, cp;
    sincos(phi, &sp, &cp);
    l[0] = s.radius * cp;
    l[1] = s.radius * sp;
    l[2] = loc[1];
  }
  s.toGlobal3(l, g);
}

// Reference frame columns x and y (the measurement frame), and z.
// PlaneSurface: the rotation; CylinderSurface: (axis x normal, axis, normal).
template <typename P>
CK_D void referenceFrame(const Surf<P>& s, const P pos[3], P ex[3], P ey[3], P ez[3]) {
  if (s.type == CK_SURFACE_PLANE) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      ex[i] = s.R[i * 3 + 0];
      ey[i] = s.R[i * 3 + 1];
      ez[i] = s.R[i * 3 + 2];
    }
    return;
  }
  P l[3];
  s.toLocal3(pos, l);
  P n2 = l[0] * l[0] + l[1] * l[1];
  P nl0 = l[0], nl1 = l[1];
  if (n2 > P(0)) {
    P inv = sqrt(n2);
    nl0 = l[0] / inv;
    nl1 = l[1] / inv;
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    ez[i] = s.R[i * 3 + 0] * nl0 + s.R[i * 3 + 1] * nl1;
    ey[i] = s.R[i * 3 + 2];
  }
  P x0 = ey[1] * ez[2] - ey[2] * ez[1];
  P x1 = ey[2] * ez[0] - ey[0] * ez[2];
  P x2 = ey[0] * ez[1] - ey[1] * ez[0];
  P xn = x0 * x0 + x1 * x1 + x2 * x2;
  if (xn > P(0)) {
    P nn = sqrt(xn);
    x0 = x0 / nn;
    x1 = x1 / nn;
    x2 = x2 / nn;
  }
  ex[0] = x0;
  ex[1] = x1;
  ex[2] = x2;
}

// Surface::pathCorrection (PlaneSurface.cpp:155-160, CylinderSurface.cpp:165-171)
template <typename P>
CK_D P pathCorrection(const Surf<P>& s, const P pos[3], const P dir[3]) {
  P ex[3], ey[3], ez[3];
  if (s.type == CK_SURFACE_PLANE) {
    P d = s.R[2] * dir[0] + s.R[5] * dir[1] + s.R[8] * dir[2];
    return P(1) / fabs(d);
  }
  referenceFrame(s, pos, ex, ey, ez);
  P cosAlpha = ez[0] * dir[0] + ez[1] * dir[1] + ez[2] * dir[2];
  return fabs(P(1) / cosAlpha);
}

// VectorHelpers::evaluateTrigonomics (VectorHelpers.hpp:165-178)
template <typename P>
struct Trig {
  P cosPhi, sinPhi, cosTheta, sinTheta, invSinTheta;
};
template <typename P>
CK_D Trig<P> trig(const P d[3]) {
  Trig<P> t;
  t.cosTheta = d[2];
  P az = fabs(d[2]);
  t.sinTheta = sqrt((P(1) - az) * (P(1) + az));
  t.invSinTheta = P(1) / t.sinTheta;
  t.cosPhi = d[0] * t.invSinTheta;
  t.sinPhi = d[1] * t.invSinTheta;
  return t;
}

// ------------------------------------------------------ bound <-> free
// TransformationHelpers.cpp:17-63
template <typename P>
CK_D void boundToFree(const Surf<P>& s, const double b[6], P f[8]) {
  double sp, cp, st, ct;
  sincos(b[2], &sp, &cp);
  sincos(b[3], &st, &ct);
  P dir[3] = {(P)(cp * st), (P)(sp * st), (P)ct};
  P loc[2] = {(P)b[0], (P)b[1]};
  P pos[3];
  localToGlobal(s, loc, pos);
  f[0] = pos[0];
  f[1] = pos[1];
  f[2] = pos[2];
  f[3] = (P)b[5];
  f[4] = dir[0];
  f[5] = dir[1];
  f[6] = dir[2];
  f[7] = (P)b[4];
}

template <typename P>
CK_D bool freeToBound(const P f[8], const Surf<P>& s, double b[6]) {
  P pos[3] = {f[0], f[1], f[2]};
  P loc[2];
  if (!globalToLocal(s, pos, kOnSurfaceTolerance, loc)) return false;
  b[0] = (double)loc[0];
  b[1] = (double)loc[1];
  b[5] = (double)f[3];
  b[2] = (double)atan2(f[5], f[4]);
  b[3] = (double)atan2(sqrt(f[4] * f[4] + f[5] * f[5]), f[6]);
  b[4] = (double)f[7];
  return true;
}

// Surface::boundToFreeJacobian in the reduced transport form:
// T columns loc0/loc1 hold the frame (rows 0-2); the dynamic block holds
// rows 0..6 of the phi, theta, q/p columns (Surface.cpp:249-268,
// JacobianHelpers.hpp:26-43).
template <typename P>
struct Transport {
  P loc[3][2];  // rows 0-2 of columns loc0, loc1 (constant during a segment)
  P dyn[7][3];  // rows 0-6 of columns phi, theta, q/p
};

template <typename P>
CK_D void initTransport(const Surf<P>& s, const P f[8], Transport<P>& T) {
  P pos[3] = {f[0], f[1], f[2]};
  P dir[3] = {f[4], f[5], f[6]};
  P ex[3], ey[3], ez[3];
  referenceFrame(s, pos, ex, ey, ez);
  Trig<P> t = trig(dir);
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    T.loc[i][0] = ex[i];
    T.loc[i][1] = ey[i];
  }
#pragma unroll
  for (int i = 0; i < 7; ++i)
#pragma unroll
    for (int c = 0; c < 3; ++c) T.dyn[i][c] = P(0);
  T.dyn[4][0] = -dir[1];
  T.dyn[5][0] = dir[0];
  T.dyn[6][0] = P(0);
  T.dyn[4][1] = t.cosTheta * t.cosPhi;
  T.dyn[5][1] = t.cosTheta * t.sinPhi;
  T.dyn[6][1] = -t.sinTheta;
}

// ------------------------------------------------------------------ field
template <typename P>
CK_D bool getGridField(const DevField& F, const P p[3], P B[3]);

template <typename P>
CK_D bool getField(const DevField& F, const P p[3], P B[3]) {
  if (F.kind == CK_FIELD_CONSTANT) {
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if constexpr (sizeof(P) == sizeof(float))
        B[i] = F.bf[i];
      else
        B[i] = F.b[i];
    }
    return true;
  }
  return getGridField(F, p, B);
}

// the grid constants of the form's type (float copies for the FP32 form)
template <typename P>
CK_D void gridConstants(const DevField& F, int i, P& mn, P& width, P& upper) {
  if constexpr (sizeof(P) == sizeof(float)) {
    mn = F.mnf[i];
    width = F.widthf[i];
    upper = F.upperf[i];
  } else {
    mn = F.mn[i];
    width = F.width[i];
    upper = F.upper[i];
  }
}

// The cell of a point (0-based lower node per axis) and its fractional
// position in it, with the axis arithmetic of the reference's equidistant
// Axis; false outside the map's [min, max) range. Every multiply-add is an
// explicit fma, so that the roundings do not depend on the inlining context.
template <typename P>
CK_D bool gridCell(const DevField& F, const P p[3], int bin[3], P f[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    P mn, width, upper;
    gridConstants(F, i, mn, width, upper);
    if (p[i] < mn || p[i] >= upper) return false;
    P u = (p[i] - mn) / width;
    int bb = (int)floor(u);  // 0-based lower node
    bb = max(0, min(bb, F.n[i] - 2));
    bin[i] = bb;
    P ll = fma((P)bb, width, mn);
    P ur = fma((P)(bb + 1), width, mn);
    f[i] = (p[i] - ll) / (ur - ll);
  }
  return true;
}

// (1 - t) a + t b as one rounded product and one fma
template <typename P>
CK_D P lerpF(P t, P a, P b) {
  return fma(t, b, (P(1) - t) * a);
}

// Interpolation (Interpolation.hpp:96-120): the eight nodes reduced along z,
// then y, then x; the result converted from Tesla to the internal unit
template <typename P>
CK_D void trilinear(const float4 v[8], const P f[3], P B[3]) {
  P r[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    r[i][0] = lerpF(f[2], (P)v[2 * i].x, (P)v[2 * i + 1].x);
    r[i][1] = lerpF(f[2], (P)v[2 * i].y, (P)v[2 * i + 1].y);
    r[i][2] = lerpF(f[2], (P)v[2 * i].z, (P)v[2 * i + 1].z);
  }
  const P unit = (P)0.000299792458;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const P s0 = lerpF(f[1], r[0][c], r[1][c]);
    const P s1 = lerpF(f[1], r[2][c], r[3][c]);
    B[c] = lerpF(f[0], s0, s1) * unit;
  }
}

template <typename P>
CK_D bool getGridField(const DevField& F, const P p[3], P B[3]) {
  // InterpolatedBFieldMap::getField with the equidistant axes of
  // fieldMapXYZ and the trilinear interpolate (z, then y, then x)
  int bin[3];
  P f[3];
  if (!gridCell(F, p, bin, f)) return false;
  const size_t nz = F.n[2], nyz = (size_t)F.n[1] * F.n[2];
  const size_t base = bin[0] * nyz + bin[1] * nz + bin[2];
  float4 v[8];
#pragma unroll
  for (int cx = 0; cx < 2; ++cx)
#pragma unroll
    for (int cy = 0; cy < 2; ++cy)
#pragma unroll
      for (int cz = 0; cz < 2; ++cz)
        v[cx * 4 + cy * 2 + cz] = __ldg(&F.nodes[base + cx * nyz + cy * nz + cz]);
  trilinear(v, f, B);
  return true;
}

// --------------------------------------------------------------- material
// Interactions.cpp (float physics) with un-contracted float arithmetic.
struct RelQ {
  float q2OverBeta2, beta2, betaGamma, gamma;
  CK_D RelQ(float mass, float qOverP, float absQ) {
    q2OverBeta2 = fa(fm(absQ, absQ), fm(fm(mass, qOverP), fm(mass, qOverP)));
    const float mOverP = fm(mass, fabsf(fd(qOverP, absQ)));
    const float pOverM = fd(1.0f, mOverP);
    beta2 = fd(1.0f, fa(1.0f, fm(mOverP, mOverP)));
    betaGamma = pOverM;
    gamma = fsq(fa(fm(1.0f, 1.0f), fm(pOverM, pOverM)));
  }
};

CK_D float computeEpsilon(const MatConst& C, float Ne, float thickness, const RelQ& rq) {
  return fm(fm(fm(fm(0.5f, C.K), Ne), thickness), rq.q2OverBeta2);
}
template <bool EXACT>
CK_D float computeDeltaHalf(const MatConst& C, float I, float Ne, const RelQ& rq) {
  if (rq.betaGamma < 10.0f) return 0.0f;
  const float plasmaEnergy = fm(C.plasmaScale, fsq(fd(Ne, C.invCm3)));
  return fs(fa(mlogf<EXACT>(rq.betaGamma), mlogf<EXACT>(fd(plasmaEnergy, I))), 0.5f);
}

template <bool EXACT = true>
CK_D float energyLossBethe(const MatConst& C, float I, float Ne, float thickness, float m,
                           float qOverP, float absQ) {
  const RelQ rq(m, qOverP, absQ);
  const float eps = computeEpsilon(C, Ne, thickness, rq);
  const float dhalf = computeDeltaHalf<EXACT>(C, I, Ne, rq);
  const float u = fm(fm(fm(2.0f, C.Me), rq.betaGamma), rq.betaGamma);
  const float mfrac = fd(C.Me, m);
  const float nominator = fm(fm(fm(2.0f, C.Me), rq.betaGamma), rq.betaGamma);
  const float denom = fa(fa(1.0f, fm(fm(2.0f, rq.gamma), mfrac)), fm(mfrac, mfrac));
  const float wmax = fd(nominator, denom);
  const float running =
      fs(fs(fa(mlogf<EXACT>(fd(u, I)), mlogf<EXACT>(fd(wmax, I))), fm(2.0f, rq.beta2)),
         fm(2.0f, dhalf));
  return fm(eps, running);
}

CK_D float landauSigmaQOverP(const MatConst& C, float Ne, float thickness, float m, float qOverP,
                             float absQ) {
  const RelQ rq(m, qOverP, absQ);
  const float fwhm = fm(4.0f, computeEpsilon(C, Ne, thickness, rq));
  const float sigmaE = fm(fwhm, 0.42466090014400953f);
  const float pInv = fd(qOverP, absQ);
  const float qOverBeta = fsq(rq.q2OverBeta2);
  return fm(fm(fm(qOverBeta, pInv), pInv), sigmaE);
}

template <bool EXACT = true>
CK_D float theta0(const MatConst& C, float tX0, int absPdg, float m, float qOverP, float absQ) {
  const float momentumInv = fabsf(fd(qOverP, absQ));
  const float q2OverBeta2 = RelQ(m, qOverP, absQ).q2OverBeta2;
  const float t = fsq(fm(tX0, q2OverBeta2));
  if (absPdg == 11) {
    // Rossi-Greisen (Interactions.cpp:490-495), log10 = log / log(10)
    const float lg = fd(mlogf<EXACT>(fm(10.0f, tX0)), C.log10f);
    return (float)dm(dm(dm(C.rossi, (double)momentumInv), (double)t),
                     (double)fa(1.0f, fm(0.125f, lg)));
  }
  // Highland (Interactions.cpp:484-489): double product of the float terms
  return (float)dm(dm(dm(C.highland, (double)momentumInv), (double)t),
                   (double)fa(1.0f, fm(fm(0.038f, 2.0f), mlogf<EXACT>(t))));
}

struct MatEffects {
  double eLoss, varPhi, varTheta, varQoP;
};

// computeMaterialEffects (PointwiseMaterialInteraction.cpp:49-90) for a
// slab scaled by `scale` (float, as MaterialSlab::scaleThickness receives).
template <typename P>
CK_D MatEffects materialEffects(const MatConst& C, const DevSurface* __restrict__ s, float f1,
                                float f2, int absPdg, float mass, float absQ, const P dir[3],
                                float qOverP, bool ms, bool el, bool& vacuum) {
  MatEffects e{0.0, 0.0, 0.0, 0.0};
  float thick = __ldg(&s->thickness);
  float tX0 = __ldg(&s->tX0);
  // MaterialSlab::scaleThickness twice: split/mode factor, then path correction
  thick = fm(thick, f1);
  tX0 = fm(tX0, f1);
  thick = fm(thick, f2);
  tX0 = fm(tX0, f2);
  vacuum = (__ldg(&s->vacuum) != 0) || thick <= 0.0f;
  if (vacuum) return e;
  const float I = __ldg(&s->matI), Ne = __ldg(&s->matNe);
  // the plain form reproduces the reference's float physics bit for bit; the
  // mixed form evaluates the same formulas in FP32 throughout
  constexpr bool EXACT = sizeof(P) == sizeof(double);
  if (el) e.eLoss = (double)energyLossBethe<EXACT>(C, I, Ne, thick, mass, qOverP, absQ);
  if (ms) {
    const float th0f = theta0<EXACT>(C, tX0, absPdg, mass, qOverP, absQ);
    if constexpr (EXACT) {
      const double th0 = (double)th0f;
      const double d0 = (double)dir[0], d1 = (double)dir[1], d2 = (double)dir[2];
      const double nrm = sqrt(da(da(dm(d0, d0), dm(d1, d1)), dm(d2, d2)));
      const double prp = sqrt(da(dm(d0, d0), dm(d1, d1)));
      const double sigmaPhi = dm(th0, nrm / prp);
      e.varPhi = dm(sigmaPhi, sigmaPhi);
      e.varTheta = dm(th0, th0);
    } else {
      const float d0 = (float)dir[0], d1 = (float)dir[1], d2 = (float)dir[2];
      const float sigmaPhi = th0f * sqrtf((d0 * d0 + d1 * d1 + d2 * d2) / (d0 * d0 + d1 * d1));
      e.varPhi = (double)(sigmaPhi * sigmaPhi);
      e.varTheta = (double)(th0f * th0f);
    }
  }
  if (el) {
    const double sq = (double)landauSigmaQOverP(C, Ne, thick, mass, qOverP, absQ);
    e.varQoP = dm(sq, sq);
  }
  return e;
}

// ----------------------------------------------------------- 2x2 / 6x6 math
struct Inv2 {
  double a00, a01, a10, a11;
};
// 1/d in FP64 from an FP32 reciprocal and two FP64 Newton steps (correct to
// about an ulp; no FP64 divide). Falls back to the divide where d is outside
// the FP32 range.
CK_D double rcpRefined(double d) {
  const float f = d2f(d);
  if (!(fabsf(f) > 1e-30f && fabsf(f) < 1e30f)) return 1.0 / d;
  double y = toD(1.0f / f);
  y = fma(y, fma(-d, y, 1.0), y);
  y = fma(y, fma(-d, y, 1.0), y);
  return y;
}

// Eigen's fixed 2x2 inverse (adjugate / determinant); FASTRCP takes the
// reciprocal of the determinant with rcpRefined (mixed form)
template <bool FASTRCP = false>
CK_D Inv2 inverse2(double m00, double m01, double m10, double m11) {
  double det = m00 * m11 - m01 * m10;
  double invdet = FASTRCP ? rcpRefined(det) : 1.0 / det;
  Inv2 r;
  r.a00 = m11 * invdet;
  r.a10 = -m10 * invdet;
  r.a01 = -m01 * invdet;
  r.a11 = m00 * invdet;
  return r;
}

// 6x6 inverse of a symmetric matrix given packed, by LU with partial
// pivoting (the algorithm of Eigen's fixed-size inverse for N > 4). The
// divisions by the pivots are multiplications by one reciprocal per pivot.
template <typename T, bool FASTRCP = false>
CK_D void inverse6(const T* __restrict__ Cp, double inv[36]) {
  double lu[36];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) lu[i * 6 + j] = toDi(Cp[sidx(i, j)]);
  int perm[6] = {0, 1, 2, 3, 4, 5};
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    int p = k;
    double best = fabs(lu[k * 6 + k]);
#pragma unroll
    for (int i = k + 1; i < 6; ++i) {
      double v = fabs(lu[i * 6 + k]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    if (p != k) {
      // swap rows k and p (register-resident: select per row)
#pragma unroll
      for (int i = k + 1; i < 6; ++i) {
        if (i == p) {
#pragma unroll
          for (int j = 0; j < 6; ++j) {
            double t = lu[k * 6 + j];
            lu[k * 6 + j] = lu[i * 6 + j];
            lu[i * 6 + j] = t;
          }
          int tp = perm[k];
          perm[k] = perm[i];
          perm[i] = tp;
        }
      }
    }
    const double rpiv = FASTRCP ? rcpRefined(lu[k * 6 + k]) : 1.0 / lu[k * 6 + k];
#pragma unroll
    for (int i = k + 1; i < 6; ++i) {
      double l = lu[i * 6 + k] * rpiv;
      lu[i * 6 + k] = l;
#pragma unroll
      for (int j = k + 1; j < 6; ++j) lu[i * 6 + j] = lu[i * 6 + j] - l * lu[k * 6 + j];
    }
  }
  double rdiag[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) rdiag[i] = FASTRCP ? rcpRefined(lu[i * 6 + i]) : 1.0 / lu[i * 6 + i];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    double y[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      double s = (perm[i] == c) ? 1.0 : 0.0;
#pragma unroll
      for (int j = 0; j < i; ++j) s = s - lu[i * 6 + j] * y[j];
      y[i] = s;
    }
#pragma unroll
    for (int i = 5; i >= 0; --i) {
      double s = y[i];
#pragma unroll
      for (int j = i + 1; j < 6; ++j) s = s - lu[i * 6 + j] * inv[j * 6 + c];
      inv[i * 6 + c] = s * rdiag[i];
    }
  }
}

// 6x6 inverse of a symmetric positive-definite matrix given packed, in FP64
// (the mixed form's smoother gain): the LDL^T factorisation without pivoting
// (Golub and Van Loan, Matrix Computations, 4th ed., section 4.1), A = L D L^T
// with L unit lower triangular, then A^-1 = W^T D^-1 W with W = L^-1. One
// reciprocal per pivot (rcpRefined); about half the FP64 operations of the
// pivoted LU inverse, no pivot search. Writes the upper triangle, packed.
template <typename T>
CK_D void inverseSym6(const T* __restrict__ Cp, double X[21]) {
  double L[6][6], d[6], rd[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    double v[6];
#pragma unroll
    for (int k = 0; k < j; ++k) v[k] = L[j][k] * d[k];
    double s = toDi(Cp[sidx(j, j)]);
#pragma unroll
    for (int k = 0; k < j; ++k) s = fma(-L[j][k], v[k], s);
    d[j] = s;
    rd[j] = rcpRefined(s);
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double t = toDi(Cp[sidx(i, j)]);
#pragma unroll
      for (int k = 0; k < j; ++k) t = fma(-L[i][k], v[k], t);
      L[i][j] = t * rd[j];
    }
  }
  // W = L^-1, unit lower triangular: column by column, W[i][j] for i > j
  double W[6][6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
#pragma unroll
    for (int i = j + 1; i < 6; ++i) {
      double t = -L[i][j];
#pragma unroll
      for (int k = j + 1; k < i; ++k) t = fma(-L[i][k], W[k][j], t);
      W[i][j] = t;
    }
  }
  // X = W^T D^-1 W: X[i][j] = sum over k >= max(i, j) of W[k][i] rd[k] W[k][j]
  double U[6][6];
#pragma unroll
  for (int k = 0; k < 6; ++k)
#pragma unroll
    for (int i = 0; i < k; ++i) U[k][i] = W[k][i] * rd[k];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      // k = j term: W[j][j] = 1
      double s = (i == j) ? rd[j] : U[j][i];
#pragma unroll
      for (int k = j + 1; k < 6; ++k) s = fma(U[k][i], W[k][j], s);
      X[sidx(i, j)] = s;
    }
}

// ------------------------------------------------------ Kalman update (N=2)
// GainMatrixUpdater::visitMeasurementImpl<2>. pred/P packed symmetric;
// writes filt and F (packed). Returns false on NaN gain (UpdateFailed).
template <bool FASTRCP = false>
CK_D bool kalmanUpdate(const double pred[6], const double Pp[21], double m0, double m1,
                       const double V[4], bool joseph, double filt[6], double F[21],
                       double& chi2) {
  // S = H P H^T + V ; K = P H^T S^-1
  Inv2 Si = inverse2<FASTRCP>(Pp[sidx(0, 0)] + V[0], Pp[sidx(0, 1)] + V[1], Pp[sidx(1, 0)] + V[2],
                     Pp[sidx(1, 1)] + V[3]);
  double K[6][2];
  bool nan = false;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double p0 = Pp[sidx(i, 0)], p1 = Pp[sidx(i, 1)];
    K[i][0] = p0 * Si.a00 + p1 * Si.a10;
    K[i][1] = p0 * Si.a01 + p1 * Si.a11;
    nan |= isnan(K[i][0]) || isnan(K[i][1]);
  }
  if (nan) return false;
  const double r0 = m0 - pred[0], r1 = m1 - pred[1];
#pragma unroll
  for (int i = 0; i < 6; ++i) filt[i] = pred[i] + (K[i][0] * r0 + K[i][1] * r1);
  normalizePhiTheta(filt[2], filt[3]);
  // A P with A = I - K H : (AP)_ij = P_ij - K_i0 P_0j - K_i1 P_1j
  if (!joseph) {
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j)
        F[sidx(i, j)] = Pp[sidx(i, j)] - (K[i][0] * Pp[sidx(0, j)] + K[i][1] * Pp[sidx(1, j)]);
  } else {
    double AP[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j)
        AP[i][j] = Pp[sidx(i, j)] - (K[i][0] * Pp[sidx(0, j)] + K[i][1] * Pp[sidx(1, j)]);
    // (AP) A^T + K V K^T
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      double kv0 = K[i][0] * V[0] + K[i][1] * V[2];
      double kv1 = K[i][0] * V[1] + K[i][1] * V[3];
#pragma unroll
      for (int j = i; j < 6; ++j) {
        double apat = AP[i][j] - (AP[i][0] * K[j][0] + AP[i][1] * K[j][1]);
        F[sidx(i, j)] = apat + (kv0 * K[j][0] + kv1 * K[j][1]);
      }
    }
  }
  // chi2 = r^T [(I - H K) V]^-1 r with r = m - H filt
  const double s0 = m0 - filt[0], s1 = m1 - filt[1];
  const double b00 = 1.0 - K[0][0], b01 = -K[0][1], b10 = -K[1][0], b11 = 1.0 - K[1][1];
  Inv2 Mi = inverse2<FASTRCP>(b00 * V[0] + b01 * V[2], b00 * V[1] + b01 * V[3], b10 * V[0] + b11 * V[2],
                     b10 * V[1] + b11 * V[3]);
  const double t0 = s0 * Mi.a00 + s1 * Mi.a10;
  const double t1 = s0 * Mi.a01 + s1 * Mi.a11;
  chi2 = t0 * s0 + t1 * s1;
  return true;
}

// calculatePredictedChi2 (TrackHelpers.hpp:563-694)
template <bool FASTRCP = false>
CK_D double predictedChi2(const double pred[6], const double Pp[21], double m0, double m1,
                          const double V[4]) {
  const double r0 = m0 - pred[0], r1 = m1 - pred[1];
  Inv2 Ri = inverse2<FASTRCP>(V[0] + Pp[sidx(0, 0)], V[1] + Pp[sidx(0, 1)], V[2] + Pp[sidx(1, 0)],
                     V[3] + Pp[sidx(1, 1)]);
  const double t0 = r0 * Ri.a00 + r1 * Ri.a10;
  const double t1 = r0 * Ri.a01 + r1 * Ri.a11;
  return t0 * r0 + t1 * r1;
}

// visitMeasurementImpl<N> for N = 2 (sub = CK_MEAS_LOC01: values m0, m1,
// covariance V) and N = 1 (sub = CK_MEAS_LOC0 / LOC1: value m0, variance
// V[0] of bound parameter a = sub >> 1) in one code path: the 1D case runs
// the 2x2 algebra with its second row switched off (S = diag(S_aa, 1), the
// second gain column and residual zero), which reduces exactly to the scalar
// formulas, so strip and pixel measurements share the kernel's registers.
// The 2D case evaluates the same expressions as kalmanUpdate.
template <bool FASTRCP = false>
CK_D bool kalmanUpdateSub(const double pred[6], const double Pp[21], int sub, double m0, double m1,
                          const double Vin[4], bool joseph, double filt[6], double F[21],
                          double& chi2) {
  const bool two = sub == CK_MEAS_LOC01;
  const bool a1 = sub == CK_MEAS_LOC1;  // the (first) measured parameter is loc1
  const double V0 = Vin[0], V1 = two ? Vin[1] : 0.0, V2 = two ? Vin[2] : 0.0,
               V3 = two ? Vin[3] : 0.0;
  double ra[6], r1[6];  // row a and row 1 of Pp
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    r1[j] = Pp[sidx(1, j)];
    ra[j] = a1 ? r1[j] : Pp[sidx(0, j)];
  }
  const double saa = (a1 ? ra[1] : ra[0]) + V0;
  Inv2 Si = inverse2<FASTRCP>(saa, two ? ra[1] + V1 : 0.0, two ? r1[0] + V2 : 0.0,
                              two ? r1[1] + V3 : 1.0);
  double K[6][2];
  bool nan = false;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const double pa = a1 ? Pp[sidx(i, 1)] : Pp[sidx(i, 0)], p1 = Pp[sidx(i, 1)];
    K[i][0] = pa * Si.a00 + p1 * Si.a10;
    K[i][1] = two ? pa * Si.a01 + p1 * Si.a11 : 0.0;
    nan |= isnan(K[i][0]) || isnan(K[i][1]);
  }
  if (nan) return false;
  const double r0 = m0 - (a1 ? pred[1] : pred[0]);
  const double rr1 = two ? m1 - pred[1] : 0.0;
#pragma unroll
  for (int i = 0; i < 6; ++i) filt[i] = pred[i] + (K[i][0] * r0 + K[i][1] * rr1);
  normalizePhiTheta(filt[2], filt[3]);
  // A P with A = I - K H : (AP)_ij = P_ij - K_i0 P_aj - K_i1 P_1j
  if (!joseph) {
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j)
        F[sidx(i, j)] = Pp[sidx(i, j)] - (K[i][0] * ra[j] + K[i][1] * r1[j]);
  } else {
    double AP[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j)
        AP[i][j] = Pp[sidx(i, j)] - (K[i][0] * ra[j] + K[i][1] * r1[j]);
    // (AP) A^T + K V K^T
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const double kv0 = K[i][0] * V0 + K[i][1] * V2;
      const double kv1 = K[i][0] * V1 + K[i][1] * V3;
      const double apa = a1 ? AP[i][1] : AP[i][0];
#pragma unroll
      for (int j = i; j < 6; ++j) {
        const double apat = AP[i][j] - (apa * K[j][0] + AP[i][1] * K[j][1]);
        F[sidx(i, j)] = apat + (kv0 * K[j][0] + kv1 * K[j][1]);
      }
    }
  }
  // chi2 = r^T [(I - H K) V]^-1 r with r = m - H filt
  const double s0 = m0 - (a1 ? filt[1] : filt[0]);
  const double s1 = two ? m1 - filt[1] : 0.0;
  const double ka0 = a1 ? K[1][0] : K[0][0], ka1 = a1 ? K[1][1] : K[0][1];
  const double b00 = 1.0 - ka0, b01 = -ka1, b10 = -K[1][0], b11 = 1.0 - K[1][1];
  Inv2 Mi = inverse2<FASTRCP>(b00 * V0 + b01 * V2, two ? b00 * V1 + b01 * V3 : 0.0,
                              two ? b10 * V0 + b11 * V2 : 0.0, two ? b10 * V1 + b11 * V3 : 1.0);
  const double t0 = s0 * Mi.a00 + s1 * Mi.a10;
  const double t1 = s0 * Mi.a01 + s1 * Mi.a11;
  chi2 = t0 * s0 + t1 * s1;
  return true;
}

// kalmanUpdateSub in FP32 (the mixed form): the same algebra on the float
// covariance the mixed form stores, with the residuals formed in FP64 and
// the parameter correction K r added to the FP64 parameters; the gain, the
// covariance update and the chi2 run on the FP32 pipe.
CK_D bool kalmanUpdateSubF(const double pred[6], const float P[21], int sub, double m0, double m1,
                           const double Vin[4], bool joseph, double filt[6], float F[21],
                           double& chi2) {
  const bool two = sub == CK_MEAS_LOC01;
  const bool a1 = sub == CK_MEAS_LOC1;
  const float V0 = d2f(Vin[0]), V1 = two ? d2f(Vin[1]) : 0.0f, V2 = two ? d2f(Vin[2]) : 0.0f,
              V3 = two ? d2f(Vin[3]) : 0.0f;
  float ra[6], r1[6];
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    r1[j] = P[sidx(1, j)];
    ra[j] = a1 ? r1[j] : P[sidx(0, j)];
  }
  const float s00 = (a1 ? ra[1] : ra[0]) + V0, s01 = two ? ra[1] + V1 : 0.0f,
              s10 = two ? r1[0] + V2 : 0.0f, s11 = two ? r1[1] + V3 : 1.0f;
  const float idet = 1.0f / (s00 * s11 - s01 * s10);
  const float i00 = s11 * idet, i01 = -s01 * idet, i10 = -s10 * idet, i11 = s00 * idet;
  float K[6][2];
  bool nan = false;
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    const float pa = a1 ? P[sidx(i, 1)] : P[sidx(i, 0)], p1 = P[sidx(i, 1)];
    K[i][0] = pa * i00 + p1 * i10;
    K[i][1] = two ? pa * i01 + p1 * i11 : 0.0f;
    nan |= isnan(K[i][0]) || isnan(K[i][1]);
  }
  if (nan) return false;
  const float r0 = d2f(m0 - (a1 ? pred[1] : pred[0]));
  const float rr1 = two ? d2f(m1 - pred[1]) : 0.0f;
#pragma unroll
  for (int i = 0; i < 6; ++i) filt[i] = pred[i] + (double)(K[i][0] * r0 + K[i][1] * rr1);
  normalizePhiTheta(filt[2], filt[3]);
  if (!joseph) {
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = i; j < 6; ++j)
        F[sidx(i, j)] = P[sidx(i, j)] - (K[i][0] * ra[j] + K[i][1] * r1[j]);
  } else {
    float AP[6][6];
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j)
        AP[i][j] = P[sidx(i, j)] - (K[i][0] * ra[j] + K[i][1] * r1[j]);
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      const float kv0 = K[i][0] * V0 + K[i][1] * V2;
      const float kv1 = K[i][0] * V1 + K[i][1] * V3;
      const float apa = a1 ? AP[i][1] : AP[i][0];
#pragma unroll
      for (int j = i; j < 6; ++j) {
        const float apat = AP[i][j] - (apa * K[j][0] + AP[i][1] * K[j][1]);
        F[sidx(i, j)] = apat + (kv0 * K[j][0] + kv1 * K[j][1]);
      }
    }
  }
  const float s0 = d2f(m0 - (a1 ? filt[1] : filt[0]));
  const float s1 = two ? d2f(m1 - filt[1]) : 0.0f;
  const float ka0 = a1 ? K[1][0] : K[0][0], ka1 = a1 ? K[1][1] : K[0][1];
  const float b00 = 1.0f - ka0, b01 = -ka1, b10 = -K[1][0], b11 = 1.0f - K[1][1];
  const float c00 = b00 * V0 + b01 * V2, c01 = two ? b00 * V1 + b01 * V3 : 0.0f,
              c10 = two ? b10 * V0 + b11 * V2 : 0.0f, c11 = two ? b10 * V1 + b11 * V3 : 1.0f;
  const float jdet = 1.0f / (c00 * c11 - c01 * c10);
  const float t0 = s0 * (c11 * jdet) + s1 * (-c10 * jdet);
  const float t1 = s0 * (-c01 * jdet) + s1 * (c00 * jdet);
  chi2 = (double)(t0 * s0 + t1 * s1);
  return true;
}

// predictedChi2Sub in FP32 on the mixed form's float covariance (residuals
// formed in FP64)
CK_D double predictedChi2SubF(const double pred[6], const float P[21], int sub, double m0,
                              double m1, const double Vin[4]) {
  const bool two = sub == CK_MEAS_LOC01;
  const bool a1 = sub == CK_MEAS_LOC1;
  const float r0 = d2f(m0 - (a1 ? pred[1] : pred[0]));
  const float r1 = two ? d2f(m1 - pred[1]) : 0.0f;
  const float s00 = d2f(Vin[0]) + (a1 ? P[sidx(1, 1)] : P[sidx(0, 0)]);
  const float s01 = two ? d2f(Vin[1]) + P[sidx(0, 1)] : 0.0f;
  const float s10 = two ? d2f(Vin[2]) + P[sidx(1, 0)] : 0.0f;
  const float s11 = two ? d2f(Vin[3]) + P[sidx(1, 1)] : 1.0f;
  const float idet = 1.0f / (s00 * s11 - s01 * s10);
  const float t0 = r0 * (s11 * idet) + r1 * (-s10 * idet);
  const float t1 = r0 * (-s01 * idet) + r1 * (s00 * idet);
  return (double)(t0 * r0 + t1 * r1);
}

// calculatePredictedChi2 for either subspace (as kalmanUpdateSub)
template <bool FASTRCP = false>
CK_D double predictedChi2Sub(const double pred[6], const double Pp[21], int sub, double m0,
                             double m1, const double Vin[4]) {
  const bool two = sub == CK_MEAS_LOC01;
  const bool a1 = sub == CK_MEAS_LOC1;
  const double r0 = m0 - (a1 ? pred[1] : pred[0]);
  const double r1 = two ? m1 - pred[1] : 0.0;
  Inv2 Ri = inverse2<FASTRCP>(Vin[0] + (a1 ? Pp[sidx(1, 1)] : Pp[sidx(0, 0)]),
                              two ? Vin[1] + Pp[sidx(0, 1)] : 0.0,
                              two ? Vin[2] + Pp[sidx(1, 0)] : 0.0,
                              two ? Vin[3] + Pp[sidx(1, 1)] : 1.0);
  const double t0 = r0 * Ri.a00 + r1 * Ri.a10;
  const double t1 = r0 * Ri.a01 + r1 * Ri.a11;
  return t0 * r0 + t1 * r1;
}

// ------------------------------------------------ free-to-bound correction
// Eigen decomposition of a symmetric 8x8 matrix (row-major A) by cyclic
// Jacobi rotations: A ends with the eigenvalues on its diagonal, V holds the
// eigenvectors in its columns. For the positive semi-definite free
// covariance this is the SVD U S U^T the reference takes (JacobiSVD).
static __device__ __noinline__ void jacobiEigen8(double* A, double* V) {
  for (int i = 0; i < 64; ++i) V[i] = (i % 9 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int p = 0; p < 8; ++p) {
      diag += A[p * 9] * A[p * 9];
      for (int q = p + 1; q < 8; ++q) off += A[p * 8 + q] * A[p * 8 + q];
    }
    if (!(off > 1e-60 * diag)) break;
    for (int p = 0; p < 7; ++p)
      for (int q = p + 1; q < 8; ++q) {
        const double apq = A[p * 8 + q];
        if (apq == 0.0) continue;
        const double theta = (A[q * 9] - A[p * 9]) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 8; ++k) {
          const double akp = A[k * 8 + p], akq = A[k * 8 + q];
          A[k * 8 + p] = c * akp - sn * akq;
          A[k * 8 + q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 8; ++k) {
          const double apk = A[p * 8 + k], aqk = A[q * 8 + k];
          A[p * 8 + k] = c * apk - sn * aqk;
          A[q * 8 + k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 8; ++k) {
          const double vkp = V[k * 8 + p], vkq = V[k * 8 + q];
          V[k * 8 + p] = c * vkp - sn * vkq;
          V[k * 8 + q] = sn * vkp + c * vkq;
        }
      }
  }
}

// detail::CorrectedFreeToBoundTransformer::operator()
// (Core/src/EventData/CorrectedTransformationFreeToBound.cpp:51-183) with the
// FreeToBoundCorrection defaults (alpha 0.1, beta 2, incidence window
// [1e-5, 0.99500417]): the unscented transform of the free covariance C
// (row-major 8x8, destroyed) through free-to-bound, each shifted sigma point
// re-intersected with the surface along its direction. False when no
// correction applies. FP64 in both forms; out of line (it runs only with the
// option on, and is heavy).
static __device__ __noinline__ bool correctedFreeToBound(const Surf<double>& s, const double* f,
                                                         double* C, double* mean, double* cov) {
  const double alpha = 0.1, beta = 2.0;
  const double pos[3] = {f[0], f[1], f[2]}, dir[3] = {f[4], f[5], f[6]};
  double ex[3], ey[3], ez[3];
  referenceFrame(s, pos, ex, ey, ez);
  const double absCos = fabs(dir[0] * ez[0] + dir[1] * ez[1] + dir[2] * ez[2]);
  if (absCos < 1e-5 || absCos > 0.99500417) return false;
  double U[64];
  jacobiEigen8(C, U);
  const double kappa = alpha * alpha * 8.0, lambda = kappa - 8.0, gamma = sqrt(kappa);
  double b0[6];
  if (!freeToBound(f, s, b0)) return false;
  double b[17][6];
  for (int r = 0; r < 6; ++r) b[0][r] = b0[r];
  for (int i = 0; i < 8; ++i) {
    const double sq = C[i * 9] > 0.0 ? sqrt(C[i * 9]) : 0.0;  // covSqrt = U sqrt(S)
    for (int sg = 0; sg < 2; ++sg) {
      double p[8];
      for (int r = 0; r < 8; ++r) {
        const double dlt = (U[r * 8 + i] * sq) * gamma;
        p[r] = sg == 0 ? f[r] + dlt : f[r] - dlt;
      }
      const double pp[3] = {p[0], p[1], p[2]}, pd[3] = {p[4], p[5], p[6]};
      double path[2];
      int st[2];
      const int n = intersect(s, pp, pd, kOnSurfaceTolerance, path, st);
      int best = -1;
      for (int j = 0; j < n; ++j) {
        if (st[j] == 0) continue;
        if (best < 0 || fabs(path[j]) < fabs(path[best])) best = j;
      }
      if (best < 0) return false;
      for (int r = 0; r < 3; ++r) p[r] = pp[r] + path[best] * pd[r];
      if (!freeToBound(p, s, b[1 + 2 * i + sg])) return false;
    }
  }
  const double wm0 = lambda / kappa, wc0 = lambda / kappa + (1.0 - alpha * alpha + beta);
  const double w = 0.5 / kappa;
  for (int r = 0; r < 6; ++r) {
    double m = 0.0;
    for (int k = 0; k < 17; ++k) m += (k == 0 ? wm0 : w) * b[k][r];
    mean[r] = m;
  }
  for (int r = 0; r < 6; ++r)
    for (int c = r; c < 6; ++c) {
      double v = 0.0;
      for (int k = 0; k < 17; ++k) v += (k == 0 ? wc0 : w) * (b[k][r] - mean[r]) * (b[k][c] - mean[c]);
      cov[sidx(r, c)] = v;
    }
  return true;
}

// CovarianceEngine.cpp:120-144: the free covariance T C T^T (T = transport
// x bound-to-free Jacobian, here its reduced form: tloc = T.loc (3x2),
// tdyn = T.dyn (7x3); C = the bound covariance at the previous surface,
// packed) through correctedFreeToBound at the free state fr. Out of line,
// with its operands copied, so that the fit kernels' registers are not
// sized for it.
template <typename P, typename CV>
__device__ __noinline__ bool correctedTransport(const Surf<double>& sfd, const P* tloc,
                                                const P* tdyn, const CV* cov, const double* fr,
                                                double* mean, double* bc) {
  double T8[8][6];
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 6; ++c) T8[r][c] = 0.0;
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 2; ++c) T8[r][c] = (double)tloc[r * 2 + c];
  for (int r = 0; r < 7; ++r)
    for (int c = 0; c < 3; ++c) T8[r][2 + c] = (double)tdyn[r * 3 + c];
  T8[7][4] = 1.0;
  T8[3][5] = 1.0;
  double TC[8][6];
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 6; ++c) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += T8[r][k] * (double)cov[sidx(k, c)];
      TC[r][c] = s;
    }
  double C[64];
  for (int r = 0; r < 8; ++r)
    for (int c = 0; c < 8; ++c) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += TC[r][k] * T8[c][k];
      C[r * 8 + c] = s;
    }
  return correctedFreeToBound(sfd, fr, C, mean, bc);
}

// ---------------------------------------------------------------- smoother
// GainMatrixSmoother::calculate. Inputs: filtered state k (filt, Pf packed),
// state k+1 predicted (pp, Ppp packed), its Jacobian J (row-major 36) and its
// smoothed state (ps, Psp packed). Outputs smoothed state k. False on NaN G.
// The inverse of Ppp is taken in FP64; the gain and covariance products run
// in GP (double in the plain form, float in the mixed form); parameters are
// accumulated in FP64.
template <typename GP>
CK_D bool smoothStep(const double filt[6], const GP Pf[21], const double pp[6], const GP Ppp[21],
                     const GP* J, const double ps[6], const GP Psp[21], double sm[6],
                     GP Ps[21]) {
  // the inverse of Ppp in FP64, as GP: the pivoted LU inverse of the
  // reference (plain form), the symmetric LDL^T inverse (mixed form)
  GP invg[36];
  if constexpr (sizeof(GP) == sizeof(float)) {
    double X[21];
    inverseSym6<GP>(Ppp, X);
    GP xg[21];
#pragma unroll
    for (int i = 0; i < 21; ++i) xg[i] = toPi<GP>(X[i]);
#pragma unroll
    for (int i = 0; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < 6; ++j) invg[i * 6 + j] = xg[sidx(i, j)];
  } else {
    double inv[36];
    inverse6<GP>(Ppp, inv);
#pragma unroll
    for (int i = 0; i < 36; ++i) invg[i] = toPi<GP>(inv[i]);
  }
  // G = (Pf J^T) Pinv
  GP PJ[36];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += Pf[sidx(i, k)] * J[j * 6 + k];
      PJ[i * 6 + j] = s;
    }
  GP G[36];
  bool nan = false;
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += PJ[i * 6 + k] * invg[k * 6 + j];
      G[i * 6 + j] = s;
      nan |= isnan(s);
    }
  if (nan) return false;
  double d[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) d[i] = ps[i] - pp[i];
  d[2] = radian_sym(d[2]);
  d[3] = radian_sym(d[3]);
  GP dg[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) dg[k] = toPi<GP>(d[k]);
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    GP s = GP(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) s += G[i * 6 + k] * dg[k];
    sm[i] = filt[i] + toDi(s);
  }
  normalizePhiTheta(sm[2], sm[3]);
  // Ps = Pf + G (Psp - Ppp) G^T
  GP GD[36];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += G[i * 6 + k] * (Psp[sidx(k, j)] - Ppp[sidx(k, j)]);
      GD[i * 6 + j] = s;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += GD[i * 6 + k] * G[j * 6 + k];
      Ps[sidx(i, j)] = Pf[sidx(i, j)] + s;
    }
  return true;
}

// ------------------------------------------------- MbfSmoother (mBF form)
template <typename GP>
CK_D void mbfMeasurement1(const double pred[6], const GP Pp[21], int h, double m, double v,
                          GP L[21], GP l[6]);
// Modified Bryson-Frazier smoother (MbfSmoother.hpp:48-90,
// MbfSmoother.cpp:17-48, MbfSmootherImpl.hpp:17-58): a backward pass that
// carries Lambda (6x6 symmetric, packed) and lambda (6) from state to state;
// no 6x6 inverse. Products run in GP (double in the plain form, float in the
// mixed form); the residual covariance inverse, the gain, the residual and
// the parameter update are FP64.

// calculateSmoothed: Ps = Pf - Pf Lambda Pf, sm = filt - Pf lambda
// (normalised). `shared`: the state's smoothed storage is its filtered
// storage, so the parameter update reads the smoothed covariance.
template <typename GP>
CK_D void mbfSmoothed(const double filt[6], const GP Pf[21], const GP L[21], const GP l[6],
                      bool shared, double sm[6], GP Ps[21]) {
  GP B[36];  // Lambda Pf
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += L[sidx(i, k)] * Pf[sidx(k, j)];
      B[i * 6 + j] = s;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += Pf[sidx(i, k)] * B[k * 6 + j];
      Ps[sidx(i, j)] = Pf[sidx(i, j)] - s;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 6; ++k) s += toDi((shared ? Ps : Pf)[sidx(i, k)] * l[k]);
    sm[i] = filt[i] - s;
  }
  normalizePhiTheta(sm[2], sm[3]);
}

// visitNonMeasurement / the last line of visitMeasurementImpl:
// Lambda <- F^T Lambda F, lambda <- F^T lambda (F row-major)
template <typename GP>
CK_D void mbfTransport(const GP* F, GP L[21], GP l[6]) {
  GP A[36];  // Lambda F
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += L[sidx(i, k)] * F[k * 6 + j];
      A[i * 6 + j] = s;
    }
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      GP s = GP(0);
#pragma unroll
      for (int k = 0; k < 6; ++k) s += F[k * 6 + i] * A[k * 6 + j];
      L[sidx(i, j)] = s;
    }
  GP ln[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    GP s = GP(0);
#pragma unroll
    for (int k = 0; k < 6; ++k) s += F[k * 6 + i] * l[k];
    ln[i] = s;
  }
#pragma unroll
  for (int i = 0; i < 6; ++i) l[i] = ln[i];
}

// visitMeasurementImpl<2> with the (loc0, loc1) projector H, before the
// transport: S = H Pp H^T + V, K = Pp H^T S^-1, C = I - K H,
// Lambda~ = H^T S^-1 H + C^T Lambda C, lambda~ = -H^T S^-1 y + C^T lambda,
// y = m - H pred. C differs from I in its first two columns only, so
// Lambda C and C^T (Lambda C) change only those columns / rows.
template <typename GP>
CK_D void mbfMeasurement(const double pred[6], const GP Pp[21], double m0, double m1,
                         const double V[4], GP L[21], GP l[6]) {
  constexpr bool kFast = sizeof(GP) == sizeof(float);
  const Inv2 si = inverse2<kFast>(toDi(Pp[sidx(0, 0)]) + V[0], toDi(Pp[sidx(0, 1)]) + V[1],
                                  toDi(Pp[sidx(1, 0)]) + V[2], toDi(Pp[sidx(1, 1)]) + V[3]);
  GP K[6][2];
#pragma unroll
  for (int r = 0; r < 6; ++r) {
    const double p0 = toDi(Pp[sidx(r, 0)]), p1 = toDi(Pp[sidx(r, 1)]);
    K[r][0] = toPi<GP>(p0 * si.a00 + p1 * si.a10);
    K[r][1] = toPi<GP>(p0 * si.a01 + p1 * si.a11);
  }
  // A = Lambda C: columns 0 and 1 are Lambda[:,c] - Lambda K[:,c]
  GP A[6][6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) A[i][j] = L[sidx(i, j)];
#pragma unroll
  for (int c = 0; c < 2; ++c)
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      GP s = GP(0);
#pragma unroll
      for (int r = 0; r < 6; ++r) s += L[sidx(i, r)] * K[r][c];
      A[i][c] -= s;
    }
  // Lambda~ = C^T A (+ S^-1 on the loc block): rows 0 and 1 are
  // A[c,:] - K[:,c]^T A
  GP Lt[21];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      GP v = A[i][j];
      if (i < 2) {
        GP s = GP(0);
#pragma unroll
        for (int r = 0; r < 6; ++r) s += K[r][i] * A[r][j];
        v -= s;
      }
      Lt[sidx(i, j)] = v;
    }
  Lt[sidx(0, 0)] += toPi<GP>(si.a00);
  Lt[sidx(0, 1)] += toPi<GP>(0.5 * (si.a01 + si.a10));
  Lt[sidx(1, 1)] += toPi<GP>(si.a11);
  // lambda~ = C^T lambda - H^T S^-1 y
  const double y0 = m0 - pred[0], y1 = m1 - pred[1];
  GP lt[6];
#pragma unroll
  for (int i = 0; i < 6; ++i) lt[i] = l[i];
#pragma unroll
  for (int c = 0; c < 2; ++c) {
    GP s = GP(0);
#pragma unroll
    for (int r = 0; r < 6; ++r) s += K[r][c] * l[r];
    lt[c] -= s;
  }
  lt[0] -= toPi<GP>(si.a00 * y0 + si.a01 * y1);
  lt[1] -= toPi<GP>(si.a10 * y0 + si.a11 * y1);
#pragma unroll
  for (int i = 0; i < 21; ++i) L[i] = Lt[i];
#pragma unroll
  for (int i = 0; i < 6; ++i) l[i] = lt[i];
}

// visitMeasurementImpl<1> before the transport: projector row e_h,
// S = P_hh + v, K = P[:,h] / S, C = I - K e_h^T differs from I in column h.
template <typename GP>
CK_D void mbfMeasurement1(const double pred[6], const GP Pp[21], int h, double m, double v,
                          GP L[21], GP l[6]) {
  constexpr bool kFast = sizeof(GP) == sizeof(float);
  const double S = toDi(h ? Pp[sidx(1, 1)] : Pp[sidx(0, 0)]) + v;
  const double iS = kFast ? rcpRefined(S) : 1.0 / S;
  GP K[6];
#pragma unroll
  for (int r = 0; r < 6; ++r) K[r] = toPi<GP>(toDi(h ? Pp[sidx(r, 1)] : Pp[sidx(r, 0)]) * iS);
  // A = Lambda C: column h is Lambda[:,h] - Lambda K
  GP A[6][6];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < 6; ++j) A[i][j] = L[sidx(i, j)];
#pragma unroll
  for (int i = 0; i < 6; ++i) {
    GP s = GP(0);
#pragma unroll
    for (int r = 0; r < 6; ++r) s += L[sidx(i, r)] * K[r];
    if (h)
      A[i][1] -= s;
    else
      A[i][0] -= s;
  }
  // Lambda~ = C^T A (+ 1/S at (h, h)): row h is A[h,:] - K^T A
  GP Lt[21];
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      GP val = A[i][j];
      if (i == h) {
        GP s = GP(0);
#pragma unroll
        for (int r = 0; r < 6; ++r) s += K[r] * A[r][j];
        val -= s;
      }
      Lt[sidx(i, j)] = val;
    }
  if (h)
    Lt[sidx(1, 1)] += toPi<GP>(iS);
  else
    Lt[sidx(0, 0)] += toPi<GP>(iS);
  // lambda~ = C^T lambda - e_h (y / S), y = m - pred_h
  const double y = m - (h ? pred[1] : pred[0]);
  GP s = GP(0);
#pragma unroll
  for (int r = 0; r < 6; ++r) s += K[r] * l[r];
  const GP upd = s + toPi<GP>(iS * y);
  if (h)
    l[1] -= upd;
  else
    l[0] -= upd;
#pragma unroll
  for (int i = 0; i < 21; ++i) L[i] = Lt[i];
}

}  // namespace ck
