// yc_sah.h -- the arithmetic of the binned SAH split over reference leaves, shared by the
// host repack (repack.cpp) and the device repack (repack_dev.cu) so that both choose the
// same splits bit for bit.
//
// Order independence: a node's bounds and bins are minima, maxima and integer sums over
// its leaves, which a sequential loop, threads merging chunks and device atomics all reach
// in different orders. Integer sums are exact in any order; float min / max are too, once
// equal values of different sign (-0 and +0) are ordered: sah_min / sah_max take -0 below
// +0, the order the sign-bit forms of the device atomics (sah_atomic_min / _max) give.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

namespace yc {

#if defined(__CUDACC__)
#define YC_SAH_HD __host__ __device__ __forceinline__
#else
#define YC_SAH_HD inline
#endif

constexpr int SAH_NB = 256;   // SAH bins per axis, at most

// bins for a range of n leaves: 256 for large ranges, fewer (8 per leaf, at least 32) for
// small ones, where binning would otherwise cost more than the range's own leaves
YC_SAH_HD int sah_bins_for(int n) {
  int v = 8 * n;
  v = v < 32 ? 32 : v;
  return v > SAH_NB ? SAH_NB : v;
}

YC_SAH_HD unsigned sah_bits(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  unsigned u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}

// min / max with -0 below +0 (a total order on the non-NaN floats)
YC_SAH_HD float sah_min(float a, float b) {
  if (a < b) return a;
  if (b < a) return b;
  return (sah_bits(a) & 0x80000000u) ? a : b;
}
YC_SAH_HD float sah_max(float a, float b) {
  if (a > b) return a;
  if (b > a) return b;
  return (sah_bits(a) & 0x80000000u) ? b : a;
}

// surface area of the box (lo, hi): 2 (dx dy + dx dz + dy dz)
YC_SAH_HD float sah_area(float lx, float ly, float lz, float hx, float hy, float hz) {
  const float d0 = hx - lx, d1 = hy - ly, d2 = hz - lz;
  return 2.0f * (d0 * d1 + d0 * d2 + d1 * d2);
}

// the bin of centroid coordinate c in a range whose centroids start at clo, with
// scale = nb / extent: floor((c - clo) scale) clamped to [0, nb); a NaN or non-positive
// product is bin 0 and a product of nb or more (an infinite scale of a tiny extent) bin
// nb - 1, the same on every machine
YC_SAH_HD int sah_bin(float c, float clo, float scale, int nb) {
  const float f = (c - clo) * scale;
  if (!(f > 0.0f)) return 0;
  if (f >= (float)nb) return nb - 1;
  return (int)f;
}

// the centroid coordinate of a leaf box
YC_SAH_HD float sah_centroid(float lo, float hi) { return 0.5f * (lo + hi); }

#if defined(__CUDACC__)
// the same min / max order as sah_min / sah_max, as atomics on a float in memory: a value
// with its sign bit clear orders like its bits as a signed integer, one with the sign bit
// set in reverse of its bits as an unsigned integer
__device__ __forceinline__ void sah_atomic_min(float* a, float v) {
  if (!(__float_as_uint(v) & 0x80000000u)) atomicMin(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMax(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
__device__ __forceinline__ void sah_atomic_max(float* a, float v) {
  if (!(__float_as_uint(v) & 0x80000000u)) atomicMax(reinterpret_cast<int*>(a), __float_as_int(v));
  else atomicMin(reinterpret_cast<unsigned*>(a), __float_as_uint(v));
}
#endif

}  // namespace yc
