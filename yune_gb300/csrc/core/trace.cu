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
#include "yc_trace_loop.cuh"

namespace yc {

// rays of the path state, addressed through the queue
template <bool ANY>
struct PathSrc {
  const DevScene* sc;
  const int* __restrict__ queue;
  SF<float4> ro;
  SF<float4> rd;
  SF<float4> hit;
  __device__ __forceinline__ const DevScene& begin(int e, RayIn& r) {
    const int q = queue[e];
    const float4 o = __ldg(&ro[q]);
    const float4 d = __ldg(&rd[q]);
    r = RayIn{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
    return *sc;
  }
  __device__ __forceinline__ void end(int e, const HitOut& h) {
    const int q = queue[e];
    if (ANY) hit[q] = make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
    else hit[q] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
};

template <bool ANY, bool WIDE>
__global__ void __launch_bounds__(TRACE_TB) k_trace_paths(DevScene sc, const int* __restrict__ queue,
                                                          const int* __restrict__ count, int* work,
                                                          SF<float4> ro,
                                                          SF<float4> rd, SF<float4> hit, int stack_cap,
                                                          DevStats* st) {
  PathSrc<ANY> src{&sc, queue, ro, rd, hit};
  trace_loop<ANY, WIDE>(src, *count, work, stack_cap, st);
}

// both queues of a round in one launch: closest-hit entries first, then any-hit (or the
// sorted list, which keeps that split)
struct PathMixedSrc {
  const DevScene* sc;
  const int* __restrict__ q_closest;
  const int* __restrict__ q_any;
  const int* __restrict__ sorted;   // non-null: this round's sorted work list
  int nc;
  SF<float4> ro;
  SF<float4> rd;
  SF<float4> hit;
  __device__ __forceinline__ int slot(int e, bool any) const {
    return sorted ? sorted[e] : (any ? q_any[e - nc] : q_closest[e]);
  }
  __device__ __forceinline__ const DevScene& begin(int e, bool any, RayIn& r) {
    const int q = slot(e, any);
    const float4 o = __ldg(&ro[q]);
    const float4 d = __ldg(&rd[q]);
    r = RayIn{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
    return *sc;
  }
  __device__ __forceinline__ void end(int e, bool any, const HitOut& h) {
    const int q = slot(e, any);
    hit[q] = any ? make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f)
                 : make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
};

template <bool WIDE>
__global__ void __launch_bounds__(TRACE_TB) k_trace_paths_mixed(DevScene sc, const int* __restrict__ q_closest,
                                                                const int* __restrict__ q_any, RoundCounters* rc,
                                                                SF<float4> ro,
                                                                SF<float4> rd, SF<float4> hit,
                                                                int stack_cap, DevStats* st, const int* sorted,
                                                                const RaySortCtl* rs, int n_smem, int* spill) {
  const int nc = rc->n_closest;
  PathMixedSrc src{&sc, q_closest, q_any, (rs && rs->use) ? sorted : nullptr, nc, ro, rd, hit};
  trace_loop_mixed<WIDE>(src, nc, nc + rc->n_any, &rc->work_closest, stack_cap, st, n_smem, spill);
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
  __device__ __forceinline__ const DevScene& begin(int e, RayIn& r) {
    const float* q = rays + 9 * (size_t)e;
    const f4 o = ym::mk(q[0], q[1], q[2], q[3]);
    const f4 d = ym::mk(q[4], q[5], q[6], q[7]);
    len = q[8];
    light = -1;
    light_test(*sc, o, d, len, light);
    r = RayIn{o.x, o.y, o.z, len, d.x, d.y, d.z};
    return *sc;
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

template <bool ANY, bool WIDE>
__global__ void __launch_bounds__(TRACE_TB) k_trace_rays(DevScene sc, const float* __restrict__ rays, int n,
                                                         int* work, int* tri_out, float* t_out, int stack_cap,
                                                         DevStats* st) {
  RaySrc<ANY> src{&sc, rays, tri_out, t_out, -1, 0.0f};
  trace_loop<ANY, WIDE>(src, n, work, stack_cap, st);
}

static int stack_cap_for(int depth) { return depth + 2; }
static size_t smem_for(int cap) { return (size_t)TRACE_TB * 2 * cap * sizeof(int); }

static int g_sm_count = 0;

template <class K>
static int resident_grid(K kernel, size_t smem) {
  if (g_sm_count == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (g_sm_count <= 0) g_sm_count = 1;
  }
  int per_sm = 0;
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TRACE_TB, smem);
  if (per_sm <= 0) return -1;
  return g_sm_count * per_sm;
}

int trace_grid_blocks(bool any_hit, int depth, bool wide) {
  const size_t smem = smem_for(stack_cap_for(depth));
  if (wide) return any_hit ? resident_grid(k_trace_paths<true, true>, smem) : resident_grid(k_trace_paths<false, true>, smem);
  return any_hit ? resident_grid(k_trace_paths<true, false>, smem) : resident_grid(k_trace_paths<false, false>, smem);
}

int launch_trace(const DevScene& sc, bool any_hit, const int* queue, const int* count, int* work, SF<float4> ro,
                 SF<float4> rd, SF<float4> hit, DevStats* st, int grid_blocks, cudaStream_t s) {
  const int cap = stack_cap_for(sc.depth);
  const size_t smem = smem_for(cap);
  const bool wide = sc.wide != 0;
  if (any_hit && wide)
    k_trace_paths<true, true><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  else if (any_hit)
    k_trace_paths<true, false><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  else if (wide)
    k_trace_paths<false, true><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  else
    k_trace_paths<false, false><<<grid_blocks, TRACE_TB, smem, s>>>(sc, queue, count, work, ro, rd, hit, cap, st);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

static_assert(TRACE_TB == TRACE_TB_PASS, "the host sizes the per-pass spill area by TRACE_TB_PASS");
int trace_stack_cap(int depth) { return stack_cap_for(depth); }

int trace_mixed_grid_blocks(int depth, bool wide, int n_smem) {
  const int cap = stack_cap_for(depth);
  const size_t smem = smem_for(n_smem > 0 && n_smem < cap ? n_smem : cap);
  return wide ? resident_grid(k_trace_paths_mixed<true>, smem) : resident_grid(k_trace_paths_mixed<false>, smem);
}

int launch_trace_mixed(const DevScene& sc, const int* q_closest, const int* q_any, RoundCounters* rc,
                       SF<float4> ro, SF<float4> rd, SF<float4> hit, DevStats* st, int grid_blocks,
                       cudaStream_t s, const int* sorted, const RaySortCtl* rs, int n_smem, int* spill) {
  const int cap = stack_cap_for(sc.depth);
  if (!(n_smem > 0 && n_smem < cap && spill)) n_smem = cap;
  const size_t smem = smem_for(n_smem);
  if (sc.wide)
    k_trace_paths_mixed<true><<<grid_blocks, TRACE_TB, smem, s>>>(sc, q_closest, q_any, rc, ro, rd, hit, cap, st,
                                                                  sorted, rs, n_smem, spill);
  else
    k_trace_paths_mixed<false><<<grid_blocks, TRACE_TB, smem, s>>>(sc, q_closest, q_any, rc, ro, rd, hit, cap, st,
                                                                   sorted, rs, n_smem, spill);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_trace_rays(const DevScene& sc, bool any_hit, const float* rays9, int n, int* tri_out, float* t_out,
                      int* work, DevStats* st, cudaStream_t s) {
  const int cap = stack_cap_for(sc.depth);
  const size_t smem = smem_for(cap);
  const bool wide = sc.wide != 0;
  int grid;
  if (any_hit && wide) {
    grid = resident_grid(k_trace_rays<true, true>, smem);
    if (grid > 0) k_trace_rays<true, true><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  } else if (any_hit) {
    grid = resident_grid(k_trace_rays<true, false>, smem);
    if (grid > 0) k_trace_rays<true, false><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  } else if (wide) {
    grid = resident_grid(k_trace_rays<false, true>, smem);
    if (grid > 0) k_trace_rays<false, true><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  } else {
    grid = resident_grid(k_trace_rays<false, false>, smem);
    if (grid > 0) k_trace_rays<false, false><<<grid, TRACE_TB, smem, s>>>(sc, rays9, n, work, tri_out, t_out, cap, st);
  }
  if (grid <= 0) return -1;
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yc
