// trace.cu -- the extend (closest-hit) and occlusion (any-hit) kernels.
//
// Persistent kernels: one grid of (SM count x resident blocks) CTAs; each warp takes 32
// queue entries at a time from a device cursor and every lane walks its ray to the end
// (yc_traverse.cuh). Each thread keeps its traversal stack in a column of dynamic shared
// memory (stride = block size, so the 32 lanes of a warp hit 32 different banks); the
// column holds depth + 1 entries of (link, entry distance). A walk that would overflow
// the stack is counted in DevStats::stack_overflow instead of writing out of bounds.
#include <cuda_runtime.h>

#include "yc_internal.h"
#include "yc_shade.cuh"
#include "yc_traverse.cuh"

namespace yc {

constexpr int TRACE_TB = 128;

__device__ __forceinline__ int warp_fetch(int* work, int n) {
  int base = 0;
  if ((threadIdx.x & 31) == 0) base = atomicAdd(work, 32);
  return __shfl_sync(0xffffffffu, base, 0);
}

// warp-reduced traversal counters, one atomic per warp and counter
template <bool ANY>
__device__ __forceinline__ void flush_counts(DevStats* st, unsigned rays, const WalkCount& wc,
                                             unsigned long long overflow) {
  unsigned long long r = rays, nn = wc.nodes, tt = wc.tris;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    r += __shfl_xor_sync(0xffffffffu, r, off);
    nn += __shfl_xor_sync(0xffffffffu, nn, off);
    tt += __shfl_xor_sync(0xffffffffu, tt, off);
    overflow += __shfl_xor_sync(0xffffffffu, overflow, off);
  }
  if ((threadIdx.x & 31) == 0) {
    if (ANY) {
      if (r) atomicAdd(&st->any_rays, r);
      if (nn) atomicAdd(&st->any_nodes, nn);
      if (tt) atomicAdd(&st->any_tris, tt);
    } else {
      if (r) atomicAdd(&st->ext_rays, r);
      if (nn) atomicAdd(&st->ext_nodes, nn);
      if (tt) atomicAdd(&st->ext_tris, tt);
    }
    if (overflow) atomicAdd(&st->stack_overflow, overflow);
  }
}

template <bool ANY>
__global__ void __launch_bounds__(TRACE_TB) k_trace_paths(DevScene sc, const int* __restrict__ queue,
                                                          const int* __restrict__ count, int* work,
                                                          const float4* __restrict__ ro,
                                                          const float4* __restrict__ rd, float4* hit, int stack_cap,
                                                          DevStats* st) {
  extern __shared__ int smem[];
  int* stack = smem + threadIdx.x;
  const int n = *count;
  unsigned long long overflow = 0;
  WalkCount wc;
  unsigned rays = 0;
  for (;;) {
    const int base = warp_fetch(work, n);
    if (base >= n) break;
    const int e = base + (threadIdx.x & 31);
    if (e < n) {
      const int p = queue[e];
      const float4 o = ro[p];
      const float4 d = rd[p];
      RayIn r{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
      HitOut h;
      if (!traverse<ANY>(sc, r, stack, TRACE_TB, stack_cap, h, wc)) ++overflow;
      ++rays;
      if (ANY) hit[p] = make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
      else hit[p] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
    }
  }
  flush_counts<ANY>(st, rays, wc, overflow);
}

// traceRay (udpt.cl:240-286) on explicit rays of 9 floats: light loop, then the BVH.
template <bool ANY>
__global__ void __launch_bounds__(TRACE_TB) k_trace_rays(DevScene sc, const float* __restrict__ rays, int n,
                                                         int* work, int* tri_out, float* t_out, int stack_cap,
                                                         DevStats* st) {
  extern __shared__ int smem[];
  int* stack = smem + threadIdx.x;
  unsigned long long overflow = 0;
  WalkCount wc;
  unsigned nrays = 0;
  for (;;) {
    const int base = warp_fetch(work, n);
    if (base >= n) break;
    const int e = base + (threadIdx.x & 31);
    if (e < n) {
      ++nrays;
      const float* q = rays + 9 * (size_t)e;
      const f4 o = ym::mk(q[0], q[1], q[2], q[3]);
      const f4 d = ym::mk(q[4], q[5], q[6], q[7]);
      float len = q[8];
      int light = -1;
      light_test(sc, o, d, len, light);
      RayIn r{o.x, o.y, o.z, len, d.x, d.y, d.z};
      HitOut h;
      if (!traverse<ANY>(sc, r, stack, TRACE_TB, stack_cap, h, wc)) ++overflow;
      if (ANY) {
        tri_out[e] = (h.tri >= 0 || light >= 0) ? 1 : 0;
        if (t_out) t_out[e] = h.tri >= 0 ? h.t : len;
      } else {
        tri_out[e] = h.tri;
        if (t_out) t_out[e] = h.tri >= 0 ? h.t : len;
        // light index for a light hit is packed after the triangle array by the caller
        if (h.tri < 0 && light >= 0) tri_out[e] = -2 - light;
      }
    }
  }
  flush_counts<ANY>(st, nrays, wc, overflow);
}

static int stack_cap_for(int depth) { return depth + 2; }
static size_t smem_for(int cap) { return (size_t)TRACE_TB * 2 * cap * sizeof(int); }

static int g_sm_count = 0;

int trace_grid_blocks(bool any_hit, int depth) {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 1;
  }
  const int cap = stack_cap_for(depth);
  const size_t smem = smem_for(cap);
  int per_sm = 0;
  if (any_hit) {
    cudaFuncSetAttribute(k_trace_paths<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_paths<true>, TRACE_TB, smem);
  } else {
    cudaFuncSetAttribute(k_trace_paths<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace_paths<false>, TRACE_TB, smem);
  }
  if (per_sm <= 0) return -1;
  return g_sm_count * per_sm;
}

int launch_trace(const DevScene& sc, bool any_hit, const int* queue, const int* count, int* work, const float4* ro,
                 const float4* rd, float4* hit, DevStats* st, int grid_blocks, cudaStream_t s) {
  const int cap = stack_cap_for(sc.depth);
  const size_t smem = smem_for(cap);
  if (any_hit)
    k_trace_paths<true><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  else
    k_trace_paths<false><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_trace_rays(const DevScene& sc, bool any_hit, const float* rays9, int n, int* tri_out, float* t_out,
                      int* work, DevStats* st, cudaStream_t s) {
  const int cap = stack_cap_for(sc.depth);
  const size_t smem = smem_for(cap);
  const int grid = trace_grid_blocks(any_hit, sc.depth);
  if (grid <= 0) return -1;
  if (any_hit) {
    cudaFuncSetAttribute(k_trace_rays<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_trace_rays<true><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  } else {
    cudaFuncSetAttribute(k_trace_rays<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_trace_rays<false><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yc
