// ym_math.h -- portable FP32 built-ins with one fixed operation sequence.
//
// The path tracer calls OpenCL C built-ins (dot, cross, normalize, length, pow, sin,
// cos, sqrt, fmax, min, max, clamp, pown). The OpenCL spec leaves their exact
// rounding to the implementation. This header pins every one of them to a fixed
// sequence of IEEE-754 single operations (+, -, *, /, sqrt, fma, compares), so the
// same source compiled by g++ for the CPU (with -ffp-contract=off) and by nvcc for
// sm_103a (with -fmad=false) returns identical bits on both sides. Nothing here
// calls a vendor math routine: sin/cos/pow/log2/exp2 are written from their
// Taylor/atanh series with Cody-Waite argument reduction (W. J. Cody and
// W. Waite, "Software Manual for the Elementary Functions", 1980).
//
// Accuracy (checked against double-precision libm in tests/test_ym_math.py):
//   sin/cos : <= 2 ulp for |x| <= 65536, double-precision reduction above that
//   log2    : relative error < 3e-7 ; exp2 : <= 2 ulp ;
//   pow     : relative error <= 3e-7 * (1 + |y * log2(x)|) (the FP32 log2 error scaled
//             by the exponent), exactly x for y == 1 and 1 for y == 0.
#pragma once

#include <stdint.h>
#include <math.h>
#include <string.h>

#if defined(__CUDACC__)
#define YM_HD __host__ __device__ __forceinline__
#else
#define YM_HD inline
#endif

namespace ym {

// ---- bit casts -----------------------------------------------------------------
YM_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
YM_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f; memcpy(&f, &u, 4); return f;
#endif
}

// ---- correctly rounded basic operations (never contracted) ---------------------
YM_HD float add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
YM_HD float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
YM_HD float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
YM_HD float div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}
YM_HD float rcp(float a) {
#if defined(__CUDA_ARCH__)
  return __frcp_rn(a);
#else
  return 1.0f / a;
#endif
}
YM_HD float sqrt(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return ::sqrtf(a);
#endif
}
YM_HD float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return ::fmaf(a, b, c);
#endif
}

YM_HD bool isnan(float x) { return x != x; }
YM_HD bool isinf(float x) { return (f2u(x) & 0x7fffffffu) == 0x7f800000u; }
YM_HD float fabs(float x) { return u2f(f2u(x) & 0x7fffffffu); }

// OpenCL C 1.2 s6.12.2: fmax/fmin ignore a NaN operand; ties return x.
YM_HD float fmax(float x, float y) {
  if (isnan(x)) return y;
  if (isnan(y)) return x;
  return (x < y) ? y : x;
}
YM_HD float fmin(float x, float y) {
  if (isnan(x)) return y;
  if (isnan(y)) return x;
  return (y < x) ? y : x;
}
// OpenCL C 1.2 s6.12.4 common functions: max = "y if x < y, otherwise x";
// min = "y if y < x, otherwise x".
YM_HD float max(float x, float y) { return (x < y) ? y : x; }
YM_HD float min(float x, float y) { return (y < x) ? y : x; }
YM_HD float clamp(float x, float lo, float hi) { return fmin(fmax(x, lo), hi); }

YM_HD float ceil(float x) {
#if defined(__CUDA_ARCH__)
  return ::ceilf(x);
#else
  return ::ceilf(x);
#endif
}
YM_HD float rint(float x) {
#if defined(__CUDA_ARCH__)
  return ::rintf(x);
#else
  return ::rintf(x);
#endif
}

// x * 2^n for an integer n, exact whenever the result is normal; two-step so a
// subnormal result is rounded once.
YM_HD float ldexp(float x, int n) {
  if (n > 127) { x = mul(x, u2f(0x7f000000u)); n -= 127; if (n > 127) n = 127; }
  if (n < -126) {
    x = mul(x, u2f(0x0c800000u));  // 2^-102
    n += 102;
    if (n < -126) { x = mul(x, u2f(0x0c800000u)); n += 102; if (n < -126) n = -126; }
  }
  return mul(x, u2f((uint32_t)(n + 127) << 23));
}

// ---- sin / cos -------------------------------------------------------------------
// Cody-Waite reduction by pi/2 in three float parts, Taylor polynomials on
// |r| <= pi/4 (truncation error below 3e-9 relative).
struct SinCosReduced { float r; int q; };

YM_HD SinCosReduced reduce_pio2(float x) {
  SinCosReduced s;
  const float ax = fabs(x);
  if (ax <= 65536.0f) {
    const float k = rint(mul(x, 0.636619746685028076171875f));   // x * 2/pi
    float r = fma(-k, 1.57079637050628662109375f, x);             // pi/2, part 1
    r = fma(-k, -4.37113882867379300296306610107421875e-08f, r);  // part 2
    r = fma(-k, -1.71512451000588185767965542129220217e-15f, r);  // part 3
    s.r = r; s.q = (int)k;
  } else {
    // large arguments: reduce in double (not reached by the renderer)
    const double dk = ::rint((double)x * 0.63661977236758134308);
    double r = (double)x - dk * 1.5707963267948966192313216916398;
    s.r = (float)r;
    long long kk = (long long)dk;
    s.q = (int)(kk & 3);
  }
  return s;
}

YM_HD float sin_poly(float r) {   // sin(r), |r| <= pi/4
  const float z = mul(r, r);
  float p = 2.7557319223985893e-06f;             //  1/9!
  p = fma(p, z, -1.9841269841269841e-04f);       // -1/7!
  p = fma(p, z, 8.3333333333333332e-03f);        //  1/5!
  p = fma(p, z, -1.6666666666666666e-01f);       // -1/3!
  return fma(mul(p, z), r, r);
}
YM_HD float cos_poly(float r) {   // cos(r), |r| <= pi/4
  const float z = mul(r, r);
  float p = -2.7557319223985888e-07f;            // -1/10!
  p = fma(p, z, 2.4801587301587302e-05f);        //  1/8!
  p = fma(p, z, -1.3888888888888889e-03f);       // -1/6!
  p = fma(p, z, 4.1666666666666664e-02f);        //  1/4!
  p = fma(p, z, -0.5f);                          // -1/2!
  return fma(p, z, 1.0f);
}

YM_HD float sin(float x) {
  if (isnan(x) || isinf(x)) return u2f(0x7fc00000u);
  SinCosReduced s = reduce_pio2(x);
  switch (s.q & 3) {
    case 0: return sin_poly(s.r);
    case 1: return cos_poly(s.r);
    case 2: return -sin_poly(s.r);
    default: return -cos_poly(s.r);
  }
}
YM_HD float cos(float x) {
  if (isnan(x) || isinf(x)) return u2f(0x7fc00000u);
  SinCosReduced s = reduce_pio2(x);
  switch (s.q & 3) {
    case 0: return cos_poly(s.r);
    case 1: return -sin_poly(s.r);
    case 2: return -cos_poly(s.r);
    default: return sin_poly(s.r);
  }
}

// ---- log2 / exp2 / pow ------------------------------------------------------------
// log2(x) = e + 2*atanh(s)/ln2 with s = (m-1)/(m+1), m in [sqrt(1/2), sqrt(2)).
YM_HD float log2_pos(float x) {      // x finite, > 0
  int e = 0;
  uint32_t u = f2u(x);
  if (u < 0x00800000u) { x = mul(x, 16777216.0f); u = f2u(x); e = -24; }  // subnormal
  e += (int)((u >> 23) & 0xff) - 127;
  float m = u2f((u & 0x007fffffu) | 0x3f800000u);                        // [1, 2)
  if (m > 1.41421353816986083984375f) { m = mul(m, 0.5f); e += 1; }
  const float s = div(sub(m, 1.0f), add(m, 1.0f));
  const float z = mul(s, s);
  float p = 0.0909090909090909f;          // 1/11
  p = fma(p, z, 0.1111111111111111f);     // 1/9
  p = fma(p, z, 0.14285714285714285f);    // 1/7
  p = fma(p, z, 0.2f);                    // 1/5
  p = fma(p, z, 0.3333333333333333f);     // 1/3
  const float atanh_s = fma(mul(p, z), s, s);
  // 2/ln2 = 2.8853900817779268
  return fma(atanh_s, 2.88539008177792681f, (float)e);
}

YM_HD float exp2(float t) {
  if (isnan(t)) return t;
  if (t >= 128.0f) return u2f(0x7f800000u);
  if (t < -150.0f) return 0.0f;
  const float n = rint(t);
  const float f = sub(t, n);                       // [-0.5, 0.5], exact
  const float g = mul(f, 0.693147182464599609375f);  // f * ln2
  float p = 1.9841269841269841e-04f;   // 1/7!
  p = fma(p, g, 1.3888888888888889e-03f);   // 1/6!
  p = fma(p, g, 8.3333333333333332e-03f);   // 1/5!
  p = fma(p, g, 4.1666666666666664e-02f);   // 1/4!
  p = fma(p, g, 1.6666666666666666e-01f);   // 1/3!
  p = fma(p, g, 0.5f);                      // 1/2!
  p = fma(p, g, 1.0f);
  p = fma(p, g, 1.0f);
  return ldexp(p, (int)n);
}

YM_HD bool is_int(float y) { return rint(y) == y; }
YM_HD bool is_odd_int(float y) {
  if (!is_int(y) || fabs(y) >= 16777216.0f) return false;
  const int k = (int)y;
  return (k & 1) != 0;
}

// pow with the C99/OpenCL special cases; the finite positive core is
// exp2(y * log2(x)).
YM_HD float pow(float x, float y) {
  const float inf = u2f(0x7f800000u);
  if (y == 0.0f) return 1.0f;
  if (y == 1.0f) return x;
  if (x == 1.0f) return 1.0f;
  if (isnan(x) || isnan(y)) return u2f(0x7fc00000u);
  if (isinf(y)) {
    const float ax = fabs(x);
    if (ax == 1.0f) return 1.0f;
    if ((ax < 1.0f) == (y > 0.0f)) return 0.0f;
    return inf;
  }
  if (x == 0.0f) {
    const bool odd = is_odd_int(y);
    if (y > 0.0f) return odd ? x : 0.0f;
    return odd ? (f2u(x) >> 31 ? -inf : inf) : inf;
  }
  float sign = 1.0f;
  if (x < 0.0f) {
    if (!is_int(y)) return u2f(0x7fc00000u);
    if (is_odd_int(y)) sign = -1.0f;
    x = -x;
  }
  if (isinf(x)) return (y > 0.0f) ? mul(sign, inf) : mul(sign, 0.0f);
  return mul(sign, exp2(mul(y, log2_pos(x))));
}

// OpenCL pown(x, n): repeated multiplication, left to right.
YM_HD float pown(float x, int n) {
  if (n == 0) return 1.0f;
  const bool neg = n < 0;
  if (neg) n = -n;
  float r = x;
  for (int i = 1; i < n; ++i) r = mul(r, x);
  return neg ? div(1.0f, r) : r;
}

// ---- 4-wide vector type with the OpenCL float4 operator semantics -------------------
struct alignas(16) f4 {
  float x, y, z, w;
};
YM_HD f4 mk(float x, float y, float z, float w) { f4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
YM_HD f4 splat(float s) { return mk(s, s, s, s); }
YM_HD f4 operator+(f4 a, f4 b) { return mk(add(a.x, b.x), add(a.y, b.y), add(a.z, b.z), add(a.w, b.w)); }
YM_HD f4 operator-(f4 a, f4 b) { return mk(sub(a.x, b.x), sub(a.y, b.y), sub(a.z, b.z), sub(a.w, b.w)); }
YM_HD f4 operator*(f4 a, f4 b) { return mk(mul(a.x, b.x), mul(a.y, b.y), mul(a.z, b.z), mul(a.w, b.w)); }
YM_HD f4 operator/(f4 a, f4 b) { return mk(div(a.x, b.x), div(a.y, b.y), div(a.z, b.z), div(a.w, b.w)); }
YM_HD f4 operator*(f4 a, float s) { return mk(mul(a.x, s), mul(a.y, s), mul(a.z, s), mul(a.w, s)); }
YM_HD f4 operator*(float s, f4 a) { return mk(mul(s, a.x), mul(s, a.y), mul(s, a.z), mul(s, a.w)); }
YM_HD f4 operator/(f4 a, float s) { return mk(div(a.x, s), div(a.y, s), div(a.z, s), div(a.w, s)); }
YM_HD f4 operator-(f4 a) { return mk(-a.x, -a.y, -a.z, -a.w); }

// dot over all four lanes, summed left to right: ((x + y) + z) + w.
YM_HD float dot(f4 a, f4 b) {
  float s = mul(a.x, b.x);
  s = add(s, mul(a.y, b.y));
  s = add(s, mul(a.z, b.z));
  return add(s, mul(a.w, b.w));
}
YM_HD float dot3(f4 a, f4 b) {   // dot of the .xyz lanes
  float s = mul(a.x, b.x);
  s = add(s, mul(a.y, b.y));
  return add(s, mul(a.z, b.z));
}
YM_HD float length(f4 a) { return sqrt(dot(a, a)); }
YM_HD float length3(f4 a) { return sqrt(dot3(a, a)); }
// OpenCL normalize: a zero vector is returned unchanged.
YM_HD f4 normalize(f4 a) {
  const float l2 = dot(a, a);
  if (l2 == 0.0f) return a;
  const float inv = div(1.0f, sqrt(l2));
  return a * inv;
}
// OpenCL cross for float4: w of the result is 0.
YM_HD f4 cross(f4 a, f4 b) {
  return mk(sub(mul(a.y, b.z), mul(a.z, b.y)),
            sub(mul(a.z, b.x), mul(a.x, b.z)),
            sub(mul(a.x, b.y), mul(a.y, b.x)), 0.0f);
}
YM_HD bool any_nan(f4 a) { return isnan(a.x) || isnan(a.y) || isnan(a.z) || isnan(a.w); }

// u32 -> [0,1]: seed / (float)UINT_MAX, where (float)UINT_MAX rounds to 2^32.
YM_HD float u01(uint32_t s) {
#if defined(__CUDA_ARCH__)
  return mul(__uint2float_rn(s), 2.3283064365386963e-10f);
#else
  return mul((float)s, 2.3283064365386963e-10f);
#endif
}

// Per-pixel RNG of the reference kernels (Thomas Wang's 32-bit hash and
// Marsaglia's xorshift32 with shifts 13/17/5).
YM_HD uint32_t wang_hash(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
YM_HD uint32_t xor_shift(uint32_t s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

}  // namespace ym
