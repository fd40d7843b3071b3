// oracle_math.hpp -- scalar/vector arithmetic for the CPU oracle, templated on the
// real type. TEST INFRASTRUCTURE: only tests, the smoke check and the benchmark's
// CPU-baseline leg use anything under oracle/.
//
// Real = float  : every operation is one IEEE-754 single operation in a pinned order,
//                 and the transcendental built-ins are the ym:: routines, so the float
//                 oracle reproduces the kernel source's arithmetic bit for bit.
// Real = double : the same algorithm in double with libm; this is the FP64 accuracy
//                 oracle used for converged-image RMSE.
#pragma once

#include <cmath>
#include <cstdint>

#include "../yune_gb300/csrc/ym_math.h"

namespace orc {

template <class R> struct Ops;

template <> struct Ops<float> {
  static float add(float a, float b) { return ym::add(a, b); }
  static float sub(float a, float b) { return ym::sub(a, b); }
  static float mul(float a, float b) { return ym::mul(a, b); }
  static float div(float a, float b) { return ym::div(a, b); }
  static float sqrt(float a) { return ym::sqrt(a); }
  static float pow(float a, float b) { return ym::pow(a, b); }
  static float sin(float a) { return ym::sin(a); }
  static float cos(float a) { return ym::cos(a); }
  static float fabs(float a) { return ym::fabs(a); }
  static float fmax(float a, float b) { return ym::fmax(a, b); }
  static float fmin(float a, float b) { return ym::fmin(a, b); }
  static float max(float a, float b) { return ym::max(a, b); }
  static float min(float a, float b) { return ym::min(a, b); }
  static bool isnan(float a) { return a != a; }
  // seed / (float)UINT_MAX (the cast rounds UINT_MAX to 2^32)
  static float u01(uint32_t s) { return ym::u01(s); }
};

template <> struct Ops<double> {
  static double add(double a, double b) { return a + b; }
  static double sub(double a, double b) { return a - b; }
  static double mul(double a, double b) { return a * b; }
  static double div(double a, double b) { return a / b; }
  static double sqrt(double a) { return std::sqrt(a); }
  static double pow(double a, double b) { return std::pow(a, b); }
  static double sin(double a) { return std::sin(a); }
  static double cos(double a) { return std::cos(a); }
  static double fabs(double a) { return std::fabs(a); }
  static double fmax(double x, double y) { if (x != x) return y; if (y != y) return x; return (x < y) ? y : x; }
  static double fmin(double x, double y) { if (x != x) return y; if (y != y) return x; return (y < x) ? y : x; }
  static double max(double x, double y) { return (x < y) ? y : x; }
  static double min(double x, double y) { return (y < x) ? y : x; }
  static bool isnan(double a) { return a != a; }
  static double u01(uint32_t s) { return (double)s / 4294967296.0; }
};

template <class R> struct V4 { R x, y, z, w; };

template <class R> inline V4<R> v4(R x, R y, R z, R w) { return V4<R>{x, y, z, w}; }
template <class R> inline V4<R> operator+(V4<R> a, V4<R> b) { using O = Ops<R>; return {O::add(a.x, b.x), O::add(a.y, b.y), O::add(a.z, b.z), O::add(a.w, b.w)}; }
template <class R> inline V4<R> operator-(V4<R> a, V4<R> b) { using O = Ops<R>; return {O::sub(a.x, b.x), O::sub(a.y, b.y), O::sub(a.z, b.z), O::sub(a.w, b.w)}; }
template <class R> inline V4<R> operator*(V4<R> a, V4<R> b) { using O = Ops<R>; return {O::mul(a.x, b.x), O::mul(a.y, b.y), O::mul(a.z, b.z), O::mul(a.w, b.w)}; }
template <class R> inline V4<R> operator*(V4<R> a, R s) { using O = Ops<R>; return {O::mul(a.x, s), O::mul(a.y, s), O::mul(a.z, s), O::mul(a.w, s)}; }
template <class R> inline V4<R> operator*(R s, V4<R> a) { using O = Ops<R>; return {O::mul(s, a.x), O::mul(s, a.y), O::mul(s, a.z), O::mul(s, a.w)}; }
template <class R> inline V4<R> operator/(V4<R> a, R s) { using O = Ops<R>; return {O::div(a.x, s), O::div(a.y, s), O::div(a.z, s), O::div(a.w, s)}; }
template <class R> inline V4<R> operator-(V4<R> a) { return {-a.x, -a.y, -a.z, -a.w}; }

// OpenCL dot over four lanes, summed ((x + y) + z) + w
template <class R> inline R dot(V4<R> a, V4<R> b) {
  using O = Ops<R>;
  R s = O::mul(a.x, b.x);
  s = O::add(s, O::mul(a.y, b.y));
  s = O::add(s, O::mul(a.z, b.z));
  return O::add(s, O::mul(a.w, b.w));
}
template <class R> inline R length(V4<R> a) { return Ops<R>::sqrt(dot(a, a)); }
template <class R> inline R length3(V4<R> a) {
  using O = Ops<R>;
  R s = O::mul(a.x, a.x);
  s = O::add(s, O::mul(a.y, a.y));
  return O::sqrt(O::add(s, O::mul(a.z, a.z)));
}
template <class R> inline V4<R> normalize(V4<R> a) {
  using O = Ops<R>;
  const R l2 = dot(a, a);
  if (l2 == R(0)) return a;
  const R inv = O::div(R(1), O::sqrt(l2));
  return a * inv;
}
template <class R> inline V4<R> cross(V4<R> a, V4<R> b) {
  using O = Ops<R>;
  return {O::sub(O::mul(a.y, b.z), O::mul(a.z, b.y)), O::sub(O::mul(a.z, b.x), O::mul(a.x, b.z)),
          O::sub(O::mul(a.x, b.y), O::mul(a.y, b.x)), R(0)};
}
template <class R> inline bool any_nan(V4<R> a) {
  using O = Ops<R>;
  return O::isnan(a.x) || O::isnan(a.y) || O::isnan(a.z) || O::isnan(a.w);
}

}  // namespace orc
