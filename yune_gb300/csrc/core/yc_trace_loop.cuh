// yc_trace_loop.cuh -- the replenishing persistent traversal loop, shared by the per-pass
// trace kernels (trace.cu) and the batch engine (engine.cu).
#pragma once

#include "yc_internal.h"
#include "yc_traverse.cuh"

namespace yc {

constexpr int TRACE_TB = 128;       // block of the per-pass trace kernels
constexpr int TRACE_TB_MAX = 256;   // largest block of the batch engine's trace kernels

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
      if (nn) atomicAdd(&st->any_boxes, nn);
      if (tt) atomicAdd(&st->any_tris, tt);
    } else {
      if (r) atomicAdd(&st->ext_rays, r);
      if (nn) atomicAdd(&st->ext_boxes, nn);
      if (tt) atomicAdd(&st->ext_tris, tt);
    }
    if (overflow) {
      atomicAdd(&st->stack_overflow, overflow);
      atomicAdd(&st->call_overflow, overflow);
    }
  }
}

// Lanes refill when at least this many of a warp's 32 lanes are idle.
constexpr int REFILL_AT = 16;

// The walk stack of this thread: its first n_smem entries in a column of the block's
// dynamic shared memory (stride: the block size), the rest of stack_cap in a column of
// `spill` (stride: the grid's threads; unused when n_smem == stack_cap)
__device__ __forceinline__ WalkStack thread_stack(int stack_cap, int n_smem, int* spill) {
  extern __shared__ int smem[];
  WalkStack ws;
  ws.s = smem + threadIdx.x;
  ws.stride = (int)blockDim.x;
  ws.gstride = (int)(gridDim.x * blockDim.x);
  ws.g = spill ? spill + (blockIdx.x * blockDim.x + threadIdx.x) : nullptr;
  ws.cap = stack_cap;
  ws.n_smem = n_smem < stack_cap ? n_smem : stack_cap;
  return ws;
}

// The persistent loop shared by the kernels. Src supplies ray e of the work list and the
// scene it walks (begin) and stores its result (end). Each thread's stack is thread_stack.
template <bool ANY, bool WIDE, class Src>
__device__ __forceinline__ void trace_loop(Src& src, int n, int* work, int stack_cap, DevStats* st,
                                           int n_smem = 1 << 30, int* spill = nullptr) {
  const WalkStack stack = thread_stack(stack_cap, n_smem, spill);
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
          const DevScene& sc = src.begin(e, r);
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
      bool done = (w.link == LINK_NONE) || walk_step<ANY, WIDE>(w, stack, wc, of);
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

// The same loop over both queues of a round in one launch: entries [0, nc) are the
// closest-hit rays, [nc, n) the any-hit rays (Src::begin and Src::end take the entry and
// its kind). One launch over all of a round's rays keeps its warps refilling for longer
// than two launches over half of them each: the lanes a warp leaves idle once the work
// list runs dry are a smaller share of the launch. Each lane counts its walk's work
// under its ray's kind.
// The per-kind totals (rays, child boxes and triangles of closest-hit and any-hit walks)
// are kept in shared memory, added once per finished ray, rather than in six registers
// of every thread for the whole launch.
template <bool WIDE, class Src>
__device__ __forceinline__ void trace_loop_mixed(Src& src, int nc, int n, int* work, int stack_cap, DevStats* st,
                                                 int n_smem = 1 << 30, int* spill = nullptr) {
  __shared__ unsigned s_tot[6];   // closest: rays, boxes, triangles; any-hit: the same
  if (threadIdx.x < 6) s_tot[threadIdx.x] = 0;
  __syncthreads();
  const WalkStack stack = thread_stack(stack_cap, n_smem, spill);
  const int lane = threadIdx.x & 31;
  unsigned overflow = 0;
  WalkCount wc;   // the current ray's walk
  Walk w;
  int e_cur = -1;
  bool any = false;
  bool more = true;
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
          any = e >= nc;
          RayIn r;
          const DevScene& sc = src.begin(e, any, r);
          walk_begin(sc, r, w);
        }
      }
    }
    if (__ballot_sync(0xffffffffu, e_cur >= 0) == 0) {
      if (!more) break;
      continue;
    }
    if (e_cur >= 0) {
      bool of = false;
      bool done = (w.link == LINK_NONE) || walk_step_k<WIDE>(w, any, stack, wc, of);
      if (of) ++overflow;
      if (done) {
        HitOut h;
        h.t = w.best; h.u = w.bu; h.v = w.bv; h.tri = w.best_tri;
        src.end(e_cur, any, h);
        unsigned* t = s_tot + (any ? 3 : 0);
        atomicAdd(t, 1u);
        atomicAdd(t + 1, wc.nodes);
        atomicAdd(t + 2, wc.tris);
        wc.nodes = 0; wc.tris = 0;
        e_cur = -1;
      }
    }
  }
  unsigned long long of = overflow;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) of += __shfl_xor_sync(0xffffffffu, of, off);
  if (lane == 0 && of) {
    atomicAdd(&st->stack_overflow, of);
    atomicAdd(&st->call_overflow, of);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long* dst[6] = {&st->ext_rays, &st->ext_boxes, &st->ext_tris, &st->any_rays, &st->any_boxes,
                                  &st->any_tris};
    for (int k = 0; k < 6; ++k)
      if (s_tot[k]) atomicAdd(dst[k], (unsigned long long)s_tot[k]);
  }
}

}  // namespace yc
