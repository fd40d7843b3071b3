// raysort.cu -- counting sort of a round's traversal work list by ray origin and direction.
//
// Rays traced in a coherent order walk the same nodes in neighbouring lanes: fewer
// divergent branches per warp and more L1 hits. Before the mixed trace launch the
// round's rays (closest-hit queue, then any-hit queue) are sorted by a key of
//   kind (1 bit, closest-hit first, so entries [0, n_closest) stay the closest-hit ones)
//   | in a batch, the low jb bits of the ray's job (rays of different scenes walk
//     different trees: keyed by job they stop sharing warps)
//   | Morton code of the origin's cell in the scene box (ob bits per axis)
//   | Morton code of the direction's cell in [-1, 1]^3 (db bits per axis)
// with a counting sort: key and histogram (one atomic per run of equal keys in a warp),
// an exclusive scan in tiles of 1024 bins (which also clears the histogram for the next
// round), and a scatter of the path indices. In the batch engine the kernels that queue
// the rays (logic, fill) form the keys and fill the histogram themselves, from the ray
// they just wrote (RsProduce, engine.cu), and only the scan and the scatter run here. The key and scatter kernels are bound by
// the latency of dependent loads and of the cursor atomics, so each warp keeps four runs
// of 32 entries in flight. The order is a heuristic only: every ray is traced with
// the same arithmetic whatever its position, so results do not change.
#include <cuda_runtime.h>

#include "yc_engine.h"
#include "yc_internal.h"

namespace yc {

constexpr int RS_TB = 256;
constexpr int RS_SCAN_TB = 1024;
constexpr int RS_MAX_TILES = 64;   // 2^16 bins at most
constexpr int RS_U = 4;            // runs of 32 work-list entries a warp handles per step

// the scene box and job of the ray in slot p: one scene per pass, or the job's scene in
// a batch
struct BoxOne {
  float4 lo, hi;
  __device__ __forceinline__ void of(int, float4& l, float4& h, unsigned& job) const {
    l = lo;
    h = hi;
    job = 0;
  }
};
struct BoxBatch {
  const BatchJob* jobs;
  SF<int4> job_pass;
  __device__ __forceinline__ void of(int p, float4& l, float4& h, unsigned& job) const {
    job = (unsigned)job_pass[p].x;
    const DevScene& sc = jobs[job].pp.sc;
    l = sc.root_lo;
    h = sc.root_hi;
  }
};

template <class Box>
__global__ void __launch_bounds__(RS_TB) k_rs_key(Box box, const int* __restrict__ q_closest,
                                                  const int* __restrict__ q_any, const RoundCounters* rc,
                                                  SF<float4> ro, SF<float4> rd,
                                                  unsigned* keys, unsigned* hist, int threshold, int ob, int db,
                                                  int jb) {
  const int nc = rc->n_closest, n = nc + rc->n_any;
  if (threshold <= 0 || n < threshold) return;   // uniform over the grid
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const unsigned kind_bit = 1u << (3 * (ob + db) + jb);
  const unsigned job_mask = (1u << jb) - 1u;
  // RS_U runs of 32 entries per warp and step: their queue, origin and direction loads
  // are all issued before the first key is formed
  for (int wbase = warp_global * 32 * RS_U; wbase < n; wbase += warps_total * 32 * RS_U) {
    int p[RS_U];
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int e = wbase + u * 32 + lane;
      p[u] = e < n ? (e < nc ? q_closest[e] : q_any[e - nc]) : -1;
    }
    float4 o[RS_U], d[RS_U];
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int pc = p[u] >= 0 ? p[u] : 0;   // idle lanes read slot 0 (n > 0 here) and discard it
      o[u] = __ldg(&ro[pc]);
      d[u] = __ldg(&rd[pc]);
    }
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int e = wbase + u * 32 + lane;
      unsigned key = 0xffffffffu - lane;   // idle lanes match nobody
      if (e < n) {
        float4 lo, hi;
        unsigned job;
        box.of(p[u], lo, hi, job);
        key = ray_key(o[u], d[u], lo, hi, ob, db) | ((job & job_mask) << (3 * (ob + db))) | (e >= nc ? kind_bit : 0u);
        keys[e] = key;
      }
      const unsigned peers = __match_any_sync(0xffffffffu, key);
      if (e < n && lane == __ffs(peers) - 1) atomicAdd(&hist[key], (unsigned)__popc(peers));
    }
  }
}

// block-wide exclusive prefix of one value per thread (RS_SCAN_TB threads); *total gets
// the block's sum
__device__ __forceinline__ unsigned block_exclusive(unsigned v, unsigned* s_warp, unsigned* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  unsigned incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const unsigned u = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) s_warp[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    unsigned w = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned u = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += u;
    }
    s_warp[lane] = w;   // inclusive over warps
  }
  __syncthreads();
  *total = s_warp[(blockDim.x >> 5) - 1];
  return incl - v + (warp > 0 ? s_warp[warp - 1] : 0u);
}

// Exclusive scan of the histogram in tiles of RS_SCAN_TB bins, one block per tile
// (coalesced): cursor = prefix within the tile, blk_sum = tile totals (the scatter adds
// the prefix of the tile totals). Clears the histogram for the next round.
__global__ void __launch_bounds__(RS_SCAN_TB) k_rs_scan(const RoundCounters* rc, unsigned* hist, unsigned* cursor,
                                                        unsigned* blk_sum, RaySortCtl* ctl, int threshold,
                                                        int nbins) {
  __shared__ unsigned s_warp[32];
  const int n = rc->n_closest + rc->n_any;
  const int use = (threshold > 0 && n >= threshold) ? 1 : 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) ctl->use = use;
  const int bin = blockIdx.x * RS_SCAN_TB + threadIdx.x;
  const unsigned c = bin < nbins ? hist[bin] : 0u;
  if (!use) {   // uniform over the grid; the keys' producers filled the histogram all the same
    if (c) hist[bin] = 0;
    return;
  }
  unsigned total;
  const unsigned ex = block_exclusive(c, s_warp, &total);
  if (bin < nbins) {
    cursor[bin] = ex;
    hist[bin] = 0;
  }
  if (threadIdx.x == 0) blk_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(RS_TB) k_rs_scatter(const int* __restrict__ q_closest,
                                                      const int* __restrict__ q_any, const RoundCounters* rc,
                                                      const unsigned* __restrict__ keys,
                                                      const unsigned* __restrict__ keys_any, unsigned* cursor,
                                                      const unsigned* __restrict__ blk_sum, int nblk, int* sorted,
                                                      const RaySortCtl* ctl) {
  __shared__ unsigned s_base[RS_MAX_TILES];
  if (!ctl->use) return;
  if (threadIdx.x < 32) {   // exclusive prefix of the tile totals (nblk <= 64)
    const int lane = threadIdx.x;
    unsigned a = lane < nblk ? blk_sum[lane] : 0u, b = lane + 32 < nblk ? blk_sum[lane + 32] : 0u;
    unsigned ia = a, ib = b;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const unsigned u = __shfl_up_sync(0xffffffffu, ia, off), w = __shfl_up_sync(0xffffffffu, ib, off);
      if (lane >= off) { ia += u; ib += w; }
    }
    const unsigned tot_a = __shfl_sync(0xffffffffu, ia, 31);
    s_base[lane] = ia - a;
    s_base[lane + 32] = tot_a + ib - b;
  }
  __syncthreads();
  const int nc = rc->n_closest, n = nc + rc->n_any;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  // RS_U runs of 32 entries per warp and step: the runs' cursor atomics are in flight
  // together instead of one after another
  for (int wbase = warp_global * 32 * RS_U; wbase < n; wbase += warps_total * 32 * RS_U) {
    unsigned key[RS_U], peers[RS_U], base[RS_U];
    int val[RS_U];
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int e = wbase + u * 32 + lane;
      const bool active = e < n;
      key[u] = active ? (keys_any && e >= nc ? keys_any[e - nc] : keys[e]) : 0xffffffffu - lane;
      val[u] = active ? (e < nc ? q_closest[e] : q_any[e - nc]) : 0;
    }
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int e = wbase + u * 32 + lane;
      peers[u] = __match_any_sync(0xffffffffu, key[u]);
      unsigned b = 0;
      if (e < n && lane == __ffs(peers[u]) - 1)
        b = s_base[key[u] / RS_SCAN_TB] + atomicAdd(&cursor[key[u]], (unsigned)__popc(peers[u]));
      base[u] = b;
    }
#pragma unroll
    for (int u = 0; u < RS_U; ++u) {
      const int e = wbase + u * 32 + lane;
      const unsigned b = __shfl_sync(0xffffffffu, base[u], __ffs(peers[u]) - 1);
      if (e < n) sorted[b + __popc(peers[u] & ((1u << lane) - 1))] = val[u];
    }
  }
}

int raysort_bins(int ob, int db, int jb) { return 1 << (3 * (ob + db) + jb + 1); }

template <class Box>
static int launch_rs(const Box& box, const int* q_closest, const int* q_any, const RoundCounters* rc,
                     SF<float4> ro, SF<float4> rd, const RaySortBufs& b, int grid, cudaStream_t s) {
  if (!b.keys_any)   // else the keys and the histogram were written as the rays were queued
    k_rs_key<Box><<<grid, RS_TB, 0, s>>>(box, q_closest, q_any, rc, ro, rd, b.keys, b.hist, b.threshold, b.ob, b.db,
                                          b.jb);
  const int nbins = raysort_bins(b.ob, b.db, b.jb);
  const int nblk = (nbins + RS_SCAN_TB - 1) / RS_SCAN_TB;
  if (nblk > RS_MAX_TILES) return -1;
  k_rs_scan<<<nblk, RS_SCAN_TB, 0, s>>>(rc, b.hist, b.cursor, b.blk_sum, b.ctl, b.threshold, nbins);
  k_rs_scatter<<<grid, RS_TB, 0, s>>>(q_closest, q_any, rc, b.keys, b.keys_any, b.cursor, b.blk_sum, nblk, b.sorted,
                                      b.ctl);
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

int launch_raysort(const DevScene& sc, const int* q_closest, const int* q_any, const RoundCounters* rc,
                   SF<float4> ro, SF<float4> rd, const RaySortBufs& b, int grid, cudaStream_t s) {
  return launch_rs(BoxOne{sc.root_lo, sc.root_hi}, q_closest, q_any, rc, ro, rd, b, grid, s);
}

int launch_raysort_batch(const BatchJob* jobs, SF<int4> job_pass, const int* q_closest, const int* q_any,
                         const RoundCounters* rc, SF<float4> ro, SF<float4> rd, const RaySortBufs& b, int grid,
                         cudaStream_t s) {
  return launch_rs(BoxBatch{jobs, job_pass}, q_closest, q_any, rc, ro, rd, b, grid, s);
}

}  // namespace yc
