// cl_shim.hpp -- just enough of OpenCL C 1.2 to compile Yune's kernel files as C++.
//
// TEST INFRASTRUCTURE (the recipe that builds the reference into oracle/_ref/). The
// kernel text is included inside namespace yref, after this header, so unqualified
// calls resolve to these built-ins and never to <cmath>. The built-ins are the ym::
// routines, i.e. the same IEEE operation sequence the oracle and the CUDA core use;
// the OpenCL spec leaves their rounding to the implementation, and this is the
// implementation the reference is run with here. Built with YREF_LIBM, cos, sin and pow
// come from the host C library instead (oracle/_ref/libyune_ref_libm.so).
#pragma once

#include <climits>
#include <cmath>
#include <cstddef>
#include <cstdint>

#include "../../yune_gb300/csrc/ym_math.h"

namespace yref {

typedef unsigned int uint;

struct float3 { float x, y, z; };
struct int2 {
  int x, y;
  int2() = default;
  int2(long a, long b) : x((int)a), y((int)b) {}
};
struct int4 { int x, y, z, w; };

struct alignas(16) float4 {
  float x, y, z, w;
  float4() = default;
  float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  float4(float s) : x(s), y(s), z(s), w(s) {}
  float3 xyz() const { return float3{x, y, z}; }
  float4& operator+=(const float4& o) { x = ym::add(x, o.x); y = ym::add(y, o.y); z = ym::add(z, o.z); w = ym::add(w, o.w); return *this; }
  float4& operator-=(const float4& o) { x = ym::sub(x, o.x); y = ym::sub(y, o.y); z = ym::sub(z, o.z); w = ym::sub(w, o.w); return *this; }
  float4& operator*=(const float4& o) { x = ym::mul(x, o.x); y = ym::mul(y, o.y); z = ym::mul(z, o.z); w = ym::mul(w, o.w); return *this; }
  float4& operator/=(const float4& o) { x = ym::div(x, o.x); y = ym::div(y, o.y); z = ym::div(z, o.z); w = ym::div(w, o.w); return *this; }
};

inline float4 operator+(float4 a, float4 b) { return a += b; }
inline float4 operator-(float4 a, float4 b) { return a -= b; }
inline float4 operator*(float4 a, float4 b) { return a *= b; }
inline float4 operator/(float4 a, float4 b) { return a /= b; }
inline float4 operator*(float4 a, float s) { return a *= float4(s); }
inline float4 operator*(float s, float4 a) { return float4(s) *= a; }
inline float4 operator/(float4 a, float s) { return a /= float4(s); }
inline float4 operator*(float4 a, int s) { return a * (float)s; }
inline float4 operator*(int s, float4 a) { return (float)s * a; }
inline float4 operator/(float4 a, int s) { return a / (float)s; }
inline float4 operator*(float4 a, double s) { return a * (float)s; }
inline float4 operator-(float4 a) { return float4(-a.x, -a.y, -a.z, -a.w); }

inline float3 operator*(float3 a, float3 b) { return float3{ym::mul(a.x, b.x), ym::mul(a.y, b.y), ym::mul(a.z, b.z)}; }
inline float3 operator/(float s, float3 a) { return float3{ym::div(s, a.x), ym::div(s, a.y), ym::div(s, a.z)}; }
inline float3 operator/(int s, float3 a) { return (float)s / a; }

inline float dot(float4 a, float4 b) {
  return ym::dot(ym::mk(a.x, a.y, a.z, a.w), ym::mk(b.x, b.y, b.z, b.w));
}
inline float length(float4 a) { return ym::sqrt(dot(a, a)); }
inline float length(float3 a) { return ym::length3(ym::mk(a.x, a.y, a.z, 0.0f)); }
inline float4 normalize(float4 a) {
  ym::f4 r = ym::normalize(ym::mk(a.x, a.y, a.z, a.w));
  return float4(r.x, r.y, r.z, r.w);
}
inline float4 cross(float4 a, float4 b) {
  ym::f4 r = ym::cross(ym::mk(a.x, a.y, a.z, a.w), ym::mk(b.x, b.y, b.z, b.w));
  return float4(r.x, r.y, r.z, r.w);
}

inline float fabs(float x) { return ym::fabs(x); }
inline float fmax(float x, float y) { return ym::fmax(x, y); }
inline float fmin(float x, float y) { return ym::fmin(x, y); }
inline float max(float x, float y) { return ym::max(x, y); }
inline float min(float x, float y) { return ym::min(x, y); }
inline float clamp(float x, float lo, float hi) { return ym::clamp(x, lo, hi); }
inline float4 clamp(float4 x, float4 lo, float4 hi) {
  return float4(clamp(x.x, lo.x, hi.x), clamp(x.y, lo.y, hi.y), clamp(x.z, lo.z, hi.z), clamp(x.w, lo.w, hi.w));
}
inline float sqrt(float x) { return ym::sqrt(x); }
#if defined(YREF_LIBM)
// the host C library's single-precision routines instead (another implementation the
// OpenCL spec allows: the measure of how far the image moves with the built-ins)
inline float cos(float x) { return ::cosf(x); }
inline float sin(float x) { return ::sinf(x); }
inline float pow(float x, float y) { return ::powf(x, y); }
#else
inline float cos(float x) { return ym::cos(x); }
inline float sin(float x) { return ym::sin(x); }
inline float pow(float x, float y) { return ym::pow(x, y); }
#endif
inline float4 pow(float4 x, float4 y) { return float4(pow(x.x, y.x), pow(x.y, y.y), pow(x.z, y.z), pow(x.w, y.w)); }
inline float pown(float x, int n) { return ym::pown(x, n); }
inline float ceil(float x) { return ym::ceil(x); }
inline int isnan(float x) { return x != x; }
inline int4 isnan(float4 v) { return int4{v.x != v.x ? -1 : 0, v.y != v.y ? -1 : 0, v.z != v.z ? -1 : 0, v.w != v.w ? -1 : 0}; }
inline int any(int4 v) { return (v.x < 0) || (v.y < 0) || (v.z < 0) || (v.w < 0); }

// images: a W x H RGBA32F buffer
struct image2d_t { float4* data; int w, h; };
typedef int sampler_t;
constexpr int CLK_NORMALIZED_COORDS_FALSE = 0, CLK_ADDRESS_CLAMP_TO_EDGE = 0, CLK_FILTER_NEAREST = 0;
inline int get_image_width(const image2d_t& im) { return im.w; }
inline int get_image_height(const image2d_t& im) { return im.h; }
inline float4 read_imagef(const image2d_t& im, sampler_t, int2 p) { return im.data[(size_t)p.y * im.w + p.x]; }
inline void write_imagef(const image2d_t& im, int2 p, float4 c) { im.data[(size_t)p.y * im.w + p.x] = c; }

// work-item ids of the calling thread
inline thread_local size_t tl_gid[2];
inline size_t get_global_id(int d) { return tl_gid[d]; }

// run-time knobs the transformed kernels read through macros
inline int yref_rr_threshold = 6;
inline int yref_max_depth = 100000;

}  // namespace yref
