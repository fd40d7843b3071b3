// trace.cu -- the extend (closest-hit) and occlusion (any-hit) kernels.
//
// Persistent kernels: one grid of (SM count x resident blocks) CTAs. A warp takes rays
// from a device cursor for its idle lanes (one atomic per refill) whenever at least
// REFILL_AT lanes are idle, and advances every busy lane's walk by one leaf per step
// (yc_traverse.cuh), so lanes whose rays end early do not wait for the warp's longest
// ray. Each thread keeps its traversal stack in a column of dynamic shared
// memory (stride = block size, so the 32 lanes of a warp hit 32 different banks); the
// column holds depth + 1 entries of (link, entry distance). A walk that would overflow
// the stack is counted in DevStats::stack_overflow instead of writing out of bounds.
#include <cuda_runtime.h>

#include "yc_internal.h"
#include "yc_shade.cuh"
#include "yc_traverse.cuh"

namespace yc {

constexpr int TRACE_TB = 128;

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

// Lanes refill when at least this many of a warp's 32 lanes are idle.
constexpr int REFILL_AT = 8;

// The persistent loop shared by both kernels. Src supplies ray e of the work list
// (begin) and stores its result (end).
template <bool ANY, class Src>
__device__ __forceinline__ void trace_loop(const DevScene& sc, Src& src, int n, int* work, int stack_cap,
                                           DevStats* st) {
  extern __shared__ int smem[];
  int* stack = smem + threadIdx.x;
  const int lane = threadIdx.x & 31;
  unsigned long long overflow = 0;
  WalkCount wc;
  unsigned rays = 0;
  Walk w;
  int e_cur = -1;            // work-list entry of this lane's ray, -1 when idle
  bool more = true;          // the work list may still hold rays (warp-uniform)
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, e_cur < 0);
    if (more && (__popc(idle) >= REFILL_AT || idle == 0xffffffffu)) {
      int base = 0;
      if (lane == 0) base = atomicAdd(work, __popc(idle));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base + __popc(idle) >= n) more = false;
      if (e_cur < 0) {
        const int e = base + __popc(idle & ((1u << lane) - 1));
        if (e < n) {
          e_cur = e;
          RayIn r;
          src.begin(e, r);
          walk_begin(sc, r, w);
          ++rays;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, e_cur >= 0) == 0) {
      if (!more) break;
      continue;
    }
    if (e_cur >= 0) {
      bool of = false;
      bool done = (w.link == LINK_NONE) || walk_step<ANY>(sc, w, stack, TRACE_TB, stack_cap, wc, of);
      if (of) ++overflow;
      if (done) {
        HitOut h;
        h.t = w.best; h.u = w.bu; h.v = w.bv; h.tri = w.best_tri;
        src.end(e_cur, h);
        e_cur = -1;
      }
    }
  }
  flush_counts<ANY>(st, rays, wc, overflow);
}

// rays of the path state, addressed through the queue
template <bool ANY>
struct PathSrc {
  const int* __restrict__ queue;
  const float4* __restrict__ ro;
  const float4* __restrict__ rd;
  float4* hit;
  int p;
  __device__ __forceinline__ void begin(int e, RayIn& r) {
    const int q = queue[e];
    const float4 o = ro[q];
    const float4 d = rd[q];
    r = RayIn{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
  }
  __device__ __forceinline__ void end(int e, const HitOut& h) {
    const int q = queue[e];
    if (ANY) hit[q] = make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
    else hit[q] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
};

template <bool ANY>
__global__ void __launch_bounds__(TRACE_TB) k_trace_paths(DevScene sc, const int* __restrict__ queue,
                                                          const int* __restrict__ count, int* work,
                                                          const float4* __restrict__ ro,
                                                          const float4* __restrict__ rd, float4* hit, int stack_cap,
                                                          DevStats* st) {
  PathSrc<ANY> src{queue, ro, rd, hit, 0};
  trace_loop<ANY>(sc, src, *count, work, stack_cap, st);
}

// traceRay (udpt.cl:240-286) on explicit rays of 9 floats: light loop, then the BVH.
template <bool ANY>
struct RaySrc {
  const DevScene* sc;
  const float* __restrict__ rays;
  int* tri_out;
  float* t_out;
  int light;
  float len;
  __device__ __forceinline__ void begin(int e, RayIn& r) {
    const float* q = rays + 9 * (size_t)e;
    const f4 o = ym::mk(q[0], q[1], q[2], q[3]);
    const f4 d = ym::mk(q[4], q[5], q[6], q[7]);
    len = q[8];
    light = -1;
    light_test(*sc, o, d, len, light);
    r = RayIn{o.x, o.y, o.z, len, d.x, d.y, d.z};
  }
  __device__ __forceinline__ void end(int e, const HitOut& h) {
    if (ANY) {
      tri_out[e] = (h.tri >= 0 || light >= 0) ? 1 : 0;
      if (t_out) t_out[e] = h.tri >= 0 ? h.t : len;
    } else {
      tri_out[e] = h.tri;
      if (t_out) t_out[e] = h.tri >= 0 ? h.t : len;
      // a light hit is reported as -2 - light (unpacked by the host entry point)
      if (h.tri < 0 && light >= 0) tri_out[e] = -2 - light;
    }
  }
};

template <bool ANY>
__global__ void __launch_bounds__(TRACE_TB) k_trace_rays(DevScene sc, const float* __restrict__ rays, int n,
                                                         int* work, int* tri_out, float* t_out, int stack_cap,
                                                         DevStats* st) {
  RaySrc<ANY> src{&sc, rays, tri_out, t_out, -1, 0.0f};
  trace_loop<ANY>(sc, src, n, work, stack_cap, st);
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
