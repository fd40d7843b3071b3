// udpt.cu -- wavefront form of the unidirectional path tracer (kernels/legacy/udpt.cl).
//
// The reference runs one work-item per pixel through `shading` (udpt.cl:433-533),
// calling traceRay 2-3 times per bounce. Here every path is a small state machine in
// HBM (PathState) and a pass is a sequence of rounds:
//   raygen (a)   -> primary rays into the closest-hit queue
//   trace        -> extend kernel (b) on the closest-hit queue, occlusion kernel on the
//                   any-hit queue (NEE shadow rays and MIS BRDF rays, (d))
//   logic        -> advances each path that got a result until it needs its next ray
//                   (shading (c), light sampling and MIS (d), Russian roulette); the new
//                   rays are appended to the next round's queues with one warp ballot +
//                   popc prefix and one atomic per warp (e), so finished paths drop out
//                   and the queues stay dense.
// A path that finishes writes its colour into the running-mean accumulator
// (udpt.cl:193-210). The random numbers of a path are drawn in the reference order,
// from the same per-pixel xorshift stream.
#include <cuda_runtime.h>

#include "yc_internal.h"
#include "yc_udpt.cuh"

namespace yc {
__global__ void __launch_bounds__(256) k_raygen(PassParams pp, PathState ps, int* q_closest, RoundCounters* rc,
                                                DevStats* st) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = pp.tile_w * pp.tile_h;
  const bool valid_thread = gid < n;
  int px = 0, py = 0;
  bool active = false;
  if (valid_thread) {
    px = gid % pp.tile_w + pp.off_x;
    py = gid / pp.tile_w + pp.off_y;
    active = px < pp.width && py < pp.height;
  }
  const int W = pp.width, H = pp.height;
  const int pix = py * W + px;
  if (active) {
    uint32_t seed;
    f4 o, d;
    float len;
    int k;
    camera_ray(pp, px, py, pp.rand_seed, seed, o, d, len, k);
    ps.misc[pix] = make_int4((int)seed, pix, pack_misc(S_PRIMARY, 0, -1, k), 0);
    ps.ro[pix] = make_float4(o.x, o.y, o.z, len);
    ps.rd[pix] = make_float4(d.x, d.y, d.z, d.w);
  }
  // warp-aggregated append of the active pixels to the closest-hit queue
  const unsigned m = __ballot_sync(0xffffffffu, active);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(&rc->n_closest, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (active) q_closest[base + __popc(m & ((1u << lane) - 1))] = pix;
  if (lane == 0 && m) {
    atomicAdd(&st->primary, (unsigned long long)__popc(m));
    atomicAdd(&st->rays, (unsigned long long)__popc(m));
    atomicAdd(&st->traversed, (unsigned long long)__popc(m));
  }
}

void launch_raygen(const PassParams& pp, const PathState& ps, int* q_closest, RoundCounters* rc, DevStats* st,
                   cudaStream_t s) {
  const int n = pp.tile_w * pp.tile_h;
  k_raygen<<<(n + 255) / 256, 256, 0, s>>>(pp, ps, q_closest, rc, st);
}

// ---- logic: one step of every path in the input queues ----

__global__ void __launch_bounds__(LOGIC_TB) k_logic(PassParams pp, PathState ps, const int* __restrict__ in_closest,
                                                    const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                    int* out_closest, int* out_any, RoundCounters* rc_out,
                                                    DevStats* st, const int* __restrict__ sorted,
                                                    const SortCtl* sctl) {
  __shared__ unsigned long long s_cnt[8];   // rays, extension, shadow, mis, traversed, samples
  if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int nc = rc_in->n_closest, na = rc_in->n_any;
  const int n = nc + na;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const bool use_sorted = sctl && sctl->use;
  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int e = wbase + lane;
    int emit = 0;
    int p = -1;
    LogicCounts lc;
    if (e < n) {
      p = use_sorted ? sorted[e] : (e < nc ? in_closest[e] : in_any[e - nc]);
      emit = logic_path(pp, pp.reset, ps, p, lc);
    }
    // compaction: ballot + popc prefix per queue, one atomic per warp and queue
    const unsigned mc = __ballot_sync(0xffffffffu, emit == 1);
    const unsigned ma = __ballot_sync(0xffffffffu, emit == 2);
    int bc = 0, ba = 0;
    if (lane == 0) {
      if (mc) bc = atomicAdd(&rc_out->n_closest, __popc(mc));
      if (ma) ba = atomicAdd(&rc_out->n_any, __popc(ma));
    }
    bc = __shfl_sync(0xffffffffu, bc, 0);
    ba = __shfl_sync(0xffffffffu, ba, 0);
    const unsigned below = (1u << lane) - 1;
    if (emit == 1) out_closest[bc + __popc(mc & below)] = p;
    if (emit == 2) out_any[ba + __popc(ma & below)] = p;
    // counters
    unsigned v[6] = {lc.rays, lc.ext, lc.shadow, lc.mis, lc.trav, lc.samples};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      unsigned x = v[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
      if (lane == 0 && x) atomicAdd(&s_cnt[q], (unsigned long long)x);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_cnt[0]) atomicAdd(&st->rays, s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&st->extension, s_cnt[1]);
    if (s_cnt[2]) atomicAdd(&st->shadow, s_cnt[2]);
    if (s_cnt[3]) atomicAdd(&st->mis, s_cnt[3]);
    if (s_cnt[4]) atomicAdd(&st->traversed, s_cnt[4]);
    if (s_cnt[5]) atomicAdd(&st->samples, s_cnt[5]);
  }
}

void launch_logic(const PassParams& pp, const PathState& ps, const int* in_closest, const int* in_any,
                  const RoundCounters* rc_in, int* out_closest, int* out_any, RoundCounters* rc_out, DevStats* st,
                  int grid, cudaStream_t s, const int* sorted, const SortCtl* sctl) {
  k_logic<<<grid, LOGIC_TB, 0, s>>>(pp, ps, in_closest, in_any, rc_in, out_closest, out_any, rc_out, st, sorted,
                                    sctl);
}

// ---- tonemap (kernels/post-proc/tonemap.cl:14-47) ----
__global__ void k_tonemap(const float4* __restrict__ in, float4* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 c = in[i];
  float y = ym::mul(0.212671f, c.x);
  y = ym::add(y, ym::mul(0.715160f, c.y));
  y = ym::add(y, ym::mul(0.072169f, c.z));
  y = ym::add(y, 0.001f);
  const float ldv = ym::div(ym::mul(y, ym::add(1.0f, ym::div(y, ym::mul(1.0f, 1.0f)))), ym::add(1.0f, y));
  const float g = ym::div(1.0f, 2.2f);
  float r[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) r[q] = ym::pow(ym::mul(ldv, ym::pow(ym::div(r[q], y), 1.0f)), g);
  out[i] = make_float4(r[0], r[1], r[2], r[3]);
}

void launch_tonemap(const float4* in, float4* out, int n, cudaStream_t s) {
  k_tonemap<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
}

}  // namespace yc
