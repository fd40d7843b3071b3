// tail.cu -- the end of a pass, when few paths are left.
//
// A pass's last rounds carry few paths (long glass and mirror paths survive Russian
// roulette), and a round of the wavefront then lasts as long as its slowest ray: the GPU
// waits on one latency-bound walk per round while almost all of it idles. Once the paths
// left fit in one resident launch, k_tail gives each of them a thread that runs the same
// steps in turn -- walk the pending ray, store the hit, advance the state machine
// (logic_path) -- until the path writes its pixel. Every path computes exactly what the
// round-by-round wavefront computes (same state, same operations), so the pass's result
// is unchanged; paths no longer wait for each other between rays.
// The kernel is launched after every round's logic kernel on that round's output
// queues: above the threshold it returns at once; at or below it, it finishes the pass
// and its last block to exit empties the queues, so the remaining round launches find
// nothing to do.
#include <cuda_runtime.h>

#include "yc_internal.h"
#include "yc_traverse.cuh"
#include "yc_udpt.cuh"

namespace yc {

constexpr int TAIL_TB = 128;
// far more rays than any path can take (max_depth 100000, three rays per bounce); a
// path that reaches it is left unfinished and counted in DevStats::stack_overflow
constexpr int TAIL_MAX_RAYS = 1 << 22;

template <bool ANY, bool WIDE>
__device__ __forceinline__ HitOut walk_full(const DevScene& sc, const float4& o, const float4& d, int* stack,
                                            int stack_cap, WalkCount& wc, unsigned& overflow) {
  const RayIn r{o.x, o.y, o.z, o.w, d.x, d.y, d.z};
  Walk w;
  walk_begin(sc, r, w);
  bool of = false;
  bool done = w.link == LINK_NONE;
  const WalkStack ws{stack, nullptr, TAIL_TB, 0, stack_cap, stack_cap};
  while (!done) done = walk_step<ANY, WIDE>(w, ws, wc, of);
  if (of) ++overflow;
  HitOut h;
  h.t = w.best; h.u = w.bu; h.v = w.bv; h.tri = w.best_tri;
  return h;
}

// three blocks per SM: up to 170 registers a thread, which the kernel needs without spills
template <bool WIDE>
__global__ void __launch_bounds__(TAIL_TB, 3) k_tail(PassParams pp, PathState ps, const int* __restrict__ in_closest,
                                                  const int* __restrict__ in_any, RoundCounters* rc_in,
                                                  int threshold, int stack_cap, DevStats* st) {
  extern __shared__ int smem[];
  int* stack = smem + threadIdx.x;
  __shared__ unsigned long long s_cnt[13];
  __shared__ bool s_last;
  const int nc = rc_in->n_closest, n = nc + rc_in->n_any;
  if (n == 0 || n > threshold) return;   // uniform over the grid
  if (threadIdx.x < 13) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  LogicCounts lc;
  WalkCount wce, wca;
  unsigned rays_e = 0, rays_a = 0, overflow = 0;
  for (;;) {
    const int e = atomicAdd(&rc_in->work_logic, 1);
    if (e >= n) break;
    const int p = e < nc ? in_closest[e] : in_any[e - nc];
    bool any = e >= nc;
    for (int k = 0;; ++k) {
      if (k == TAIL_MAX_RAYS) { ++overflow; break; }
      const float4 o = ps.ro[p], d = ps.rd[p];
      if (any) {
        const HitOut h = walk_full<true, WIDE>(pp.sc, o, d, stack, stack_cap, wca, overflow);
        ps.hit[p] = make_float4(h.tri >= 0 ? 1.0f : 0.0f, 0.0f, 0.0f, 0.0f);
        ++rays_a;
      } else {
        const HitOut h = walk_full<false, WIDE>(pp.sc, o, d, stack, stack_cap, wce, overflow);
        ps.hit[p] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
        ++rays_e;
      }
      const int emit = logic_path(pp, pp.reset, ps, p, lc);
      if (emit == 0) break;
      any = emit == 2;
    }
  }
  const unsigned long long v[13] = {lc.rays, lc.ext, lc.shadow, lc.mis, lc.trav, lc.samples,
                                    rays_e, wce.nodes, wce.tris, rays_a, wca.nodes, wca.tris, overflow};
#pragma unroll
  for (int q = 0; q < 13; ++q)
    if (v[q]) atomicAdd(&s_cnt[q], v[q]);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long* dst[13] = {&st->rays, &st->extension, &st->shadow, &st->mis, &st->traversed, &st->samples,
                                   &st->ext_rays, &st->ext_boxes, &st->ext_tris, &st->any_rays, &st->any_boxes,
                                   &st->any_tris, &st->stack_overflow};
    for (int q = 0; q < 13; ++q)
      if (s_cnt[q]) atomicAdd(dst[q], s_cnt[q]);
    if (s_cnt[12]) atomicAdd(&st->call_overflow, s_cnt[12]);
    // the last block to finish empties the queues (every block has read the counts)
    __threadfence();
    s_last = atomicAdd(&rc_in->pad[0], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (threadIdx.x == 0 && s_last) {
    rc_in->n_closest = 0;
    rc_in->n_any = 0;
    rc_in->pad[0] = 0;
  }
}

static size_t tail_smem(int cap) { return (size_t)TAIL_TB * 2 * cap * sizeof(int); }

template <class K>
static int tail_grid_of(K kernel, size_t smem) {
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, TAIL_TB, smem);
  return per_sm > 0 ? per_sm * sms : -1;
}

int tail_capacity(const DevScene& sc, int* grid_out) {
  const size_t smem = tail_smem(sc.depth + 2);
  const int grid = sc.wide ? tail_grid_of(k_tail<true>, smem) : tail_grid_of(k_tail<false>, smem);
  if (grid_out) *grid_out = grid;
  return grid > 0 ? grid * TAIL_TB : 0;
}

int launch_tail(const PassParams& pp, const PathState& ps, const int* in_closest, const int* in_any,
                RoundCounters* rc_in, int threshold, DevStats* st, int grid, cudaStream_t s) {
  const int cap = pp.sc.depth + 2;
  const size_t smem = tail_smem(cap);
  if (pp.sc.wide)
    k_tail<true><<<grid, TAIL_TB, smem, s>>>(pp, ps, in_closest, in_any, rc_in, threshold, cap, st);
  else
    k_tail<false><<<grid, TAIL_TB, smem, s>>>(pp, ps, in_closest, in_any, rc_in, threshold, cap, st);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yc
