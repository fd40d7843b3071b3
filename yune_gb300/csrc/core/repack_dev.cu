// repack_dev.cu -- the upload's repack on the device for the default tree mode (an SAH
// hierarchy over the reference leaves; yc_upload_scene with YC_OPT_REPACK 1).
//
// The reference uploads its BVHNodeGPU array as it is and walks it (traverseBVH,
// kernels/legacy/udpt.cl:298-321); the core repacks it into the layout of yc_scene.h
// (repack.cpp states what the layout keeps: each reference leaf's triangles, their order
// and tie-break ranks). This file writes that layout on the GPU, byte for byte what the
// host repack writes: the leaves' triangle stream, the shading records and the two-child
// nodes of the binned SAH split of yc_sah.h.
//
// The split, top down. A range of leaves is one block's task: its bounds (block
// reduction), its bins (shared-memory atomics), its split (one warp per axis scans the
// bins, the first minimum of the cost in (axis, bin) order wins, as the host's sequential
// sweep), then a stable partition through a second buffer. A node's index is known before
// its subtree is built (pre-order: the left child follows its parent, the right child
// comes after the left subtree's leaves - 1 nodes), so every task writes its own box and
// link into its parent's record and no pass orders anything afterwards. Ranges of more
// than SMALL_MAX leaves are split one level per launch, a block per range, with the
// leaves in global memory; a range of at most SMALL_MAX leaves is loaded into one
// block's shared memory and its whole subtree built there.
//
// Compiled with -fmad=false like the rest of the core: the areas and costs round as the
// host's (-ffp-contract=off) do.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include "yc_internal.h"
#include "yc_repack.h"
#include "yc_sah.h"

namespace yc {

namespace {

constexpr int LEVEL_TB = 512;    // threads of a block that splits one large range
constexpr int SMALL_TB = 128;    // threads of a block that builds one small subtree
constexpr int SMALL_MAX = 512;   // ranges of at most this many leaves are built in shared memory
constexpr int ITEM_TB = 256;

// a reference leaf: its box, its triangle count (lo.w, integer bits) and its link (hi.w)
struct __align__(16) SahItem {
  float4 lo, hi;
};

// leaves [b, e) under node `node` (pre-order index); up = parent * 2 + side, -1 for the root
struct SahTask {
  int b, e, node, up, depth;
};

struct SahCtl {
  int n_next;    // ranges queued for the next level
  int n_small;   // ranges queued for the shared-memory builds
  int depth;     // deepest task or leaf (the root is 0)
  int bad;       // a list or a partition would have left its bounds (nothing was written there)
};

// per axis and bin: leaves, triangles, the union of the leaf boxes
struct SahBins {
  int cnt[3][SAH_NB];
  int w[3][SAH_NB];
  float lo[3][3][SAH_NB];
  float hi[3][3][SAH_NB];
};

struct SahScratch {
  float red[32][12];   // per-warp partial bounds
  float box[12];       // the range's lo[3], hi[3], centroid lo[3], centroid hi[3]
  float cost[3];       // per axis: the first minimal cost, its bin and left leaves
  int split[3], nleft[3];
  int axis, at, mid;   // the chosen axis (-1: split in half), bin, first leaf of the right side
  int wcount[32];
};

constexpr float kInf = INFINITY;

// a partial union of bins: box, leaves, triangles
struct Acc {
  float lo[3], hi[3];
  int cnt, w;
};
__device__ __forceinline__ void acc_empty(Acc& a) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = kInf;
    a.hi[k] = -kInf;
  }
  a.cnt = 0;
  a.w = 0;
}
__device__ __forceinline__ void acc_join(Acc& a, const Acc& b) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = sah_min(a.lo[k], b.lo[k]);
    a.hi[k] = sah_max(a.hi[k], b.hi[k]);
  }
  a.cnt += b.cnt;
  a.w += b.w;
}
__device__ __forceinline__ void acc_bin(Acc& a, const SahBins& bn, int k, int q) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a.lo[c] = sah_min(a.lo[c], bn.lo[k][c][q]);
    a.hi[c] = sah_max(a.hi[c], bn.hi[k][c][q]);
  }
  a.cnt += bn.cnt[k][q];
  a.w += bn.w[k][q];
}
__device__ __forceinline__ Acc acc_shfl_up(const Acc& a, int d) {
  Acc r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = __shfl_up_sync(0xffffffffu, a.lo[k], d);
    r.hi[k] = __shfl_up_sync(0xffffffffu, a.hi[k], d);
  }
  r.cnt = __shfl_up_sync(0xffffffffu, a.cnt, d);
  r.w = __shfl_up_sync(0xffffffffu, a.w, d);
  return r;
}
__device__ __forceinline__ Acc acc_shfl_down(const Acc& a, int d) {
  Acc r;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    r.lo[k] = __shfl_down_sync(0xffffffffu, a.lo[k], d);
    r.hi[k] = __shfl_down_sync(0xffffffffu, a.hi[k], d);
  }
  r.cnt = __shfl_down_sync(0xffffffffu, a.cnt, d);
  r.w = __shfl_down_sync(0xffffffffu, a.w, d);
  return r;
}

__device__ __forceinline__ float comp(const float4& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// the parent's record of a child: its box at the child's side and its link
__device__ __forceinline__ void put_child(float4* nodes, int up, const float lo[3], const float hi[3], int link) {
  if (up < 0) return;
  float* o = reinterpret_cast<float*>(nodes + 4 * (size_t)(up >> 1));
  const int side = up & 1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    o[4 * k + side] = lo[k];
    o[4 * k + 2 + side] = hi[k];
  }
  o[12 + side] = __int_as_float(link);
}

// bounds of items [b, e) into sc.box (all threads)
__device__ void range_bounds(const SahItem* it, int b, int e, SahScratch& sc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float v[12];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v[k] = kInf;
    v[3 + k] = -kInf;
    v[6 + k] = kInf;
    v[9 + k] = -kInf;
  }
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
    const float4 lo = it[i].lo, hi = it[i].hi;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float l = comp(lo, k), h = comp(hi, k), c = sah_centroid(l, h);
      v[k] = sah_min(v[k], l);
      v[3 + k] = sah_max(v[3 + k], h);
      v[6 + k] = sah_min(v[6 + k], c);
      v[9 + k] = sah_max(v[9 + k], c);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int j = 0; j < 12; ++j) {
      const float o = __shfl_xor_sync(0xffffffffu, v[j], off);
      v[j] = ((j / 3) & 1) ? sah_max(v[j], o) : sah_min(v[j], o);
    }
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < 12; ++j) sc.red[warp][j] = v[j];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int j = 0; j < 12; ++j) v[j] = lane < nw ? sc.red[lane][j] : (((j / 3) & 1) ? -kInf : kInf);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
      for (int j = 0; j < 12; ++j) {
        const float o = __shfl_xor_sync(0xffffffffu, v[j], off);
        v[j] = ((j / 3) & 1) ? sah_max(v[j], o) : sah_min(v[j], o);
      }
    if (lane == 0)
#pragma unroll
      for (int j = 0; j < 12; ++j) sc.box[j] = v[j];
  }
  __syncthreads();
}

// the bins of items [b, e) on the axes with a positive centroid extent (all threads)
__device__ void range_bins(const SahItem* it, int b, int e, int nb, SahBins& bn, const SahScratch& sc) {
  for (int x = threadIdx.x; x < 3 * nb; x += blockDim.x) {
    const int k = x / nb, q = x - k * nb;
    bn.cnt[k][q] = 0;
    bn.w[k][q] = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      bn.lo[k][c][q] = kInf;
      bn.hi[k][c][q] = -kInf;
    }
  }
  float clo[3], scale[3];
  bool on[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    clo[k] = sc.box[6 + k];
    const float ext = sc.box[9 + k] - clo[k];
    on[k] = ext > 0.0f;
    scale[k] = on[k] ? (float)nb / ext : 0.0f;
  }
  __syncthreads();
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) {
    const float4 lo = it[i].lo, hi = it[i].hi;
    const int w = __float_as_int(lo.w);
    const float l[3] = {lo.x, lo.y, lo.z}, h[3] = {hi.x, hi.y, hi.z};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (!on[k]) continue;
      const int q = sah_bin(sah_centroid(l[k], h[k]), clo[k], scale[k], nb);
      atomicAdd(&bn.cnt[k][q], 1);
      atomicAdd(&bn.w[k][q], w);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        sah_atomic_min(&bn.lo[k][c][q], l[c]);
        sah_atomic_max(&bn.hi[k][c][q], h[c]);
      }
    }
  }
  __syncthreads();
}

// the split of the binned range [b, e): sc.axis, sc.at, sc.mid (all threads). Warp k
// sweeps axis k: lane j owns bins [j per, (j + 1) per); the unions of the lanes below and
// above come from warp scans, then each lane walks its bins for the left unions (upward)
// and the right unions and costs (downward), keeping the smallest bin of its minimal cost.
constexpr int kMaxPer = SAH_NB / 32;

__device__ void range_split(int b, int e, int nb, const SahBins& bn, SahScratch& sc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (warp < 3) {
    const int k = warp;
    const float ext = sc.box[9 + k] - sc.box[6 + k];
    float best = kInf;
    int bq = -1, bl = 0;
    if (ext > 0.0f) {
      const int per = (nb + 31) >> 5;
      const int s0 = min(nb, lane * per), s1 = min(nb, s0 + per);
      Acc agg;
      acc_empty(agg);
      for (int q = s0; q < s1; ++q) acc_bin(agg, bn, k, q);
      // inclusive scans of the lane unions, upward and downward
      Acc up = agg, down = agg;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const Acc u = acc_shfl_up(up, d);
        if (lane >= d) acc_join(up, u);
        const Acc v = acc_shfl_down(down, d);
        if (lane + d < 32) acc_join(down, v);
      }
      Acc below = acc_shfl_up(up, 1), above = acc_shfl_down(down, 1);
      if (lane == 0) acc_empty(below);
      if (lane == 31) acc_empty(above);
      // left unions at the lane's bins
      Acc L[kMaxPer];
      Acc run = below;
#pragma unroll
      for (int j = 0; j < kMaxPer; ++j) {
        if (s0 + j < s1) acc_bin(run, bn, k, s0 + j);
        L[j] = run;
      }
      Acc R = above;   // the union of the bins above the current one
#pragma unroll
      for (int j = kMaxPer - 1; j >= 0; --j) {
        const int q = s0 + j;
        if (q >= s1) continue;
        if (q <= nb - 2 && L[j].cnt > 0 && R.cnt > 0) {
          const float cost = sah_area(L[j].lo[0], L[j].lo[1], L[j].lo[2], L[j].hi[0], L[j].hi[1], L[j].hi[2]) *
                                 (float)L[j].w +
                             sah_area(R.lo[0], R.lo[1], R.lo[2], R.hi[0], R.hi[1], R.hi[2]) * (float)R.w;
          if (cost < kInf && cost <= best) {   // downward: on equal costs the smaller bin
            best = cost;
            bq = q;
            bl = L[j].cnt;
          }
        }
        acc_bin(R, bn, k, q);
      }
    }
    // the first minimum over the lanes: the smaller cost, then the smaller bin
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const float oc = __shfl_xor_sync(0xffffffffu, best, off);
      const int oq = __shfl_xor_sync(0xffffffffu, bq, off);
      const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
      if (oq >= 0 && (bq < 0 || oc < best || (oc == best && oq < bq))) {
        best = oc;
        bq = oq;
        bl = ol;
      }
    }
    if (lane == 0) {
      sc.cost[k] = best;
      sc.split[k] = bq;
      sc.nleft[k] = bl;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int axis = -1;
    float best = kInf;
    for (int k = 0; k < 3; ++k)
      if (sc.split[k] >= 0 && sc.cost[k] < best) {
        best = sc.cost[k];
        axis = k;
      }
    sc.axis = axis;
    sc.at = axis >= 0 ? sc.split[axis] : -1;
    sc.mid = axis >= 0 ? b + sc.nleft[axis] : (b + e) / 2;   // coincident centroids: split the list in half
  }
  __syncthreads();
}

// stable partition of items [b, e) by the chosen split, through tmp (all threads)
__device__ void range_partition(SahItem* it, SahItem* tmp, int b, int e, int nb, SahScratch& sc, int* bad) {
  const int k = sc.axis, split = sc.at, mid = sc.mid;
  const float clo = sc.box[6 + k];
  const float scale = (float)nb / (sc.box[9 + k] - clo);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int run_l = 0, run_r = 0;
  for (int base = b; base < e; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const bool in = i < e;
    SahItem x;
    bool left = false;
    if (in) {
      x = it[i];
      left = sah_bin(sah_centroid(comp(x.lo, k), comp(x.hi, k)), clo, scale, nb) <= split;
    }
    const unsigned m = __ballot_sync(0xffffffffu, left);
    const int rank = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) sc.wcount[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
      const int c = sc.wcount[w];
      before += w < warp ? c : 0;
      total += c;
    }
    if (in) {
      const int at = left ? b + run_l + before + rank : mid + run_r + (int)threadIdx.x - before - rank;
      if (left ? at < mid : (at >= mid && at < e)) tmp[at] = x;
      else *bad = 1;   // the bins and the partition disagree: the upload fails
    }
    run_l += total;
    run_r += min((int)blockDim.x, e - base) - total;
    __syncthreads();
  }
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) it[i] = tmp[i];
  __syncthreads();
}

// one task: its box and link into the parent's record, its depth, its split (all threads)
__device__ void split_task(SahItem* it, SahItem* tmp, int b, int e, const SahTask& t, SahBins& bn, SahScratch& sc,
                           float4* nodes, int* depth, int* bad) {
  range_bounds(it, b, e, sc);
  if (threadIdx.x == 0) {
    const float lo[3] = {sc.box[0], sc.box[1], sc.box[2]}, hi[3] = {sc.box[3], sc.box[4], sc.box[5]};
    put_child(nodes, t.up, lo, hi, t.node);
    float* o = reinterpret_cast<float*>(nodes + 4 * (size_t)t.node);
    o[14] = 0.0f;
    o[15] = 0.0f;
    atomicMax(depth, t.depth);
  }
  const int nb = sah_bins_for(e - b);
  range_bins(it, b, e, nb, bn, sc);
  range_split(b, e, nb, bn, sc);
  if (sc.axis >= 0) range_partition(it, tmp, b, e, nb, sc, bad);
}

// a child range of one leaf: the parent's record takes the leaf's box and link
__device__ __forceinline__ void put_leaf(float4* nodes, int up, const SahItem& x) {
  const float lo[3] = {x.lo.x, x.lo.y, x.lo.z}, hi[3] = {x.hi.x, x.hi.y, x.hi.z};
  put_child(nodes, up, lo, hi, __float_as_int(x.hi.w));
}

// one level of the large ranges, a block per range
__global__ void __launch_bounds__(LEVEL_TB) k_sah_level(SahItem* items, SahItem* tmp, const SahTask* tasks,
                                                        SahTask* next, int cap_next, SahTask* small, int cap_small,
                                                        SahCtl* ctl, float4* nodes) {
  __shared__ SahBins bn;
  __shared__ SahScratch sc;
  const SahTask t = tasks[blockIdx.x];
  split_task(items, tmp, t.b, t.e, t, bn, sc, nodes, &ctl->depth, &ctl->bad);
  if (threadIdx.x == 0) {
    const int mid = sc.mid;
    const SahTask kids[2] = {{t.b, mid, t.node + 1, 2 * t.node, t.depth + 1},
                             {mid, t.e, t.node + (mid - t.b), 2 * t.node + 1, t.depth + 1}};
    for (const SahTask& c : kids) {
      const int n = c.e - c.b;
      if (n == 1) {
        put_leaf(nodes, c.up, items[c.b]);
        atomicMax(&ctl->depth, c.depth);
      } else if (n > SMALL_MAX) {
        const int at = atomicAdd(&ctl->n_next, 1);
        if (at < cap_next) next[at] = c;
        else ctl->bad = 1;
      } else {
        const int at = atomicAdd(&ctl->n_small, 1);
        if (at < cap_small) small[at] = c;
        else ctl->bad = 1;
      }
    }
  }
}

// A range of at most 32 leaves, split by one warp with the leaves in its lanes. The split
// is the binned sweep's without the bins: per axis the lanes are ranked by bin (stable),
// the unions of the first r + 1 ranked leaves and of the rest come from warp scans, and a
// cost is evaluated between neighbours of different bins only. Every bin q between two
// occupied bins has the same two sides, hence the same cost, so the sweep's first minimum
// in bin order is the first minimum in rank order, at the lower neighbour's bin; bins
// before the first occupied one or from the last one on have an empty side.
constexpr int TINY_MAX = 32;

__device__ __forceinline__ float shfl_f(float v, int src) { return __shfl_sync(0xffffffffu, v, src); }

// the tiny range [t.b, t.e) of `it` and its whole subtree, by one warp; stack: 16 entries
__device__ void tiny_subtree(SahItem* it, const SahTask& root, SahTask* stack, float4* nodes, int* dmax, int* bad) {
  const int lane = threadIdx.x & 31;
  int top = 0;
  SahTask t = root;
  for (;;) {
    const int b = t.b, e = t.e, n = e - b;
    const bool on = lane < n;
    float lo[3], hi[3], c[3];
    int w = 0, link = 0;
    {
      const SahItem x = on ? it[b + lane] : SahItem{};
      lo[0] = x.lo.x; lo[1] = x.lo.y; lo[2] = x.lo.z;
      hi[0] = x.hi.x; hi[1] = x.hi.y; hi[2] = x.hi.z;
      w = __float_as_int(x.lo.w);
      link = __float_as_int(x.hi.w);
    }
    __syncwarp();
    // bounds of the range (lanes past n contribute nothing)
    float box[12];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      c[k] = sah_centroid(lo[k], hi[k]);
      box[k] = on ? lo[k] : kInf;
      box[3 + k] = on ? hi[k] : -kInf;
      box[6 + k] = on ? c[k] : kInf;
      box[9 + k] = on ? c[k] : -kInf;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
      for (int j = 0; j < 12; ++j) {
        const float o = __shfl_xor_sync(0xffffffffu, box[j], off);
        box[j] = ((j / 3) & 1) ? sah_max(box[j], o) : sah_min(box[j], o);
      }
    if (lane == 0) {
      const float blo[3] = {box[0], box[1], box[2]}, bhi[3] = {box[3], box[4], box[5]};
      put_child(nodes, t.up, blo, bhi, t.node);
      float* o = reinterpret_cast<float*>(nodes + 4 * (size_t)t.node);
      o[14] = 0.0f;
      o[15] = 0.0f;
      atomicMax(dmax, t.depth);
    }
    const int nb = sah_bins_for(n);
    float best = kInf;
    int axis = -1, at = -1, nleft = 0;
    int q_of[3] = {0, 0, 0};
    if (n == 2) {
      // two leaves: on every axis where their centroids differ the one split puts the lower
      // centroid's leaf (bin 0) left and the other (the last bin) right, at the same cost
      // area(A) wA + area(B) wB (a sum of two terms: the same bits in either order), so the
      // first such axis wins if that cost is finite
      const float ai = sah_area(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]) * (float)w;
      const float cost = __shfl_sync(0xffffffffu, ai, 0) + __shfl_sync(0xffffffffu, ai, 1);
      for (int k = 0; k < 3 && axis < 0; ++k)
        if (box[9 + k] - box[6 + k] > 0.0f && cost < kInf) axis = k;
      if (axis >= 0) {
        const float ck = axis == 0 ? c[0] : (axis == 1 ? c[1] : c[2]);
        const float clo = axis == 0 ? box[6] : (axis == 1 ? box[7] : box[8]);
        const int qv = ck == clo ? 0 : nb - 1;
        q_of[0] = axis == 0 ? qv : 0;
        q_of[1] = axis == 1 ? qv : 0;
        q_of[2] = axis == 2 ? qv : 0;
        at = 0;
        nleft = 1;
      }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float clo = box[6 + k], ext = box[9 + k] - clo;
      if (n == 2 || !(ext > 0.0f)) continue;   // uniform across the warp
      const float scale = (float)nb / ext;
      const int q = on ? sah_bin(c[k], clo, scale, nb) : 0x7fffffff;
      q_of[k] = q;
      // stable rank by bin, then the leaf of each rank
      int rank = 0;
      for (int jj = 0; jj < n; ++jj) {
        const int qj = __shfl_sync(0xffffffffu, q, jj);
        rank += (qj < q || (qj == q && jj < lane)) ? 1 : 0;
      }
      // the lane holding the leaf of rank `lane` (lanes < n hold distinct ranks 0..n-1)
      int src = lane;
      for (int r = 0; r < n; ++r) {
        const unsigned m = __ballot_sync(0xffffffffu, on && rank == r);
        if (lane == r) src = __ffs(m) - 1;
      }
      const int qs = __shfl_sync(0xffffffffu, q, src);
      float slo[3], shi[3];
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        slo[cc] = shfl_f(lo[cc], src);
        shi[cc] = shfl_f(hi[cc], src);
      }
      const int sw = __shfl_sync(0xffffffffu, w, src);
      Acc a;   // the leaf of rank `lane` (lanes past n: empty)
      acc_empty(a);
      if (on) {
#pragma unroll
        for (int cc = 0; cc < 3; ++cc) {
          a.lo[cc] = slo[cc];
          a.hi[cc] = shi[cc];
        }
        a.cnt = 1;
        a.w = sw;
      }
      Acc L = a, R = a;   // inclusive prefix and suffix unions in rank order
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const Acc u = acc_shfl_up(L, d);
        if (lane >= d) acc_join(L, u);
        const Acc v = acc_shfl_down(R, d);
        if (lane + d < 32) acc_join(R, v);
      }
      const Acc R1 = acc_shfl_down(R, 1);          // the leaves ranked after this one
      const int qn = __shfl_down_sync(0xffffffffu, qs, 1);
      float cost = kInf;
      if (lane < n - 1 && qs < qn)
        cost = sah_area(L.lo[0], L.lo[1], L.lo[2], L.hi[0], L.hi[1], L.hi[2]) * (float)L.w +
               sah_area(R1.lo[0], R1.lo[1], R1.lo[2], R1.hi[0], R1.hi[1], R1.hi[2]) * (float)R1.w;
      float bc = cost < kInf ? cost : kInf;
      int br = cost < kInf ? lane : 32;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const float oc = __shfl_xor_sync(0xffffffffu, bc, off);
        const int orr = __shfl_xor_sync(0xffffffffu, br, off);
        if (oc < bc || (oc == bc && orr < br)) {
          bc = oc;
          br = orr;
        }
      }
      const int q_at = __shfl_sync(0xffffffffu, qs, br & 31);
      if (br < 32 && bc < best) {   // the first axis with the smallest cost
        best = bc;
        axis = k;
        at = q_at;
        nleft = br + 1;
      }
    }
    int mid;
    if (axis >= 0) {
      mid = b + nleft;
      const int qa = axis == 0 ? q_of[0] : (axis == 1 ? q_of[1] : q_of[2]);
      const bool left = on && qa <= at;
      const unsigned m = __ballot_sync(0xffffffffu, left);
      if (__popc(m) != nleft && lane == 0) *bad = 1;
      const int before = __popc(m & ((1u << lane) - 1u));
      if (on) {
        const int to = left ? b + before : mid + (lane - before);
        if (to >= b && to < e) {
          it[to].lo = make_float4(lo[0], lo[1], lo[2], __int_as_float(w));
          it[to].hi = make_float4(hi[0], hi[1], hi[2], __int_as_float(link));
        }
      }
    } else {
      mid = (b + e) / 2;   // coincident centroids: split the list in half
    }
    __syncwarp();
    if (lane == 0) {
      const SahTask kids[2] = {{b, mid, t.node + 1, 2 * t.node, t.depth + 1},
                               {mid, e, t.node + (mid - b), 2 * t.node + 1, t.depth + 1}};
      for (const SahTask& kd : kids) {
        if (kd.e - kd.b == 1) {
          put_leaf(nodes, kd.up, it[kd.b]);
          atomicMax(dmax, kd.depth);
        } else if (top < TINY_MAX / 2) {
          stack[top++] = kd;
        } else {
          *bad = 1;
        }
      }
    }
    top = __shfl_sync(0xffffffffu, top, 0);
    __syncwarp();
    if (top == 0) break;
    --top;
    t = stack[top];
    __syncwarp();
  }
}

// shared memory of a small-range block: the leaves, the partition buffer, the bins, the
// pending ranges (a stack from the bottom, the ranges of at most TINY_MAX leaves from the
// top: disjoint, of two leaves or more, so at most SMALL_MAX / 2 together) and a 16-entry
// stack per warp for the tiny subtrees
constexpr int SMALL_WARPS = SMALL_TB / 32;
constexpr int PEND_MAX = SMALL_MAX / 2;
constexpr size_t kSmallSmem = 2 * SMALL_MAX * sizeof(SahItem) + sizeof(SahBins) + PEND_MAX * sizeof(SahTask) +
                              SMALL_WARPS * (TINY_MAX / 2) * sizeof(SahTask);

// the whole subtree of a range of at most SMALL_MAX leaves, a block per range: the ranges
// above TINY_MAX leaves split by the whole block, then the tiny ones by one warp each
__global__ void __launch_bounds__(SMALL_TB) k_sah_small(const SahItem* items, const SahTask* small, SahCtl* ctl,
                                                        float4* nodes) {
  extern __shared__ __align__(16) unsigned char smem[];
  SahItem* it = reinterpret_cast<SahItem*>(smem);
  SahItem* tmp = it + SMALL_MAX;
  SahBins& bn = *reinterpret_cast<SahBins*>(tmp + SMALL_MAX);
  SahTask* pend = reinterpret_cast<SahTask*>(&bn + 1);
  SahTask* wstack = pend + PEND_MAX;
  __shared__ SahScratch sc;
  __shared__ int top, ntiny, tiny_next, dmax;
  const SahTask r = small[blockIdx.x];
  const int n = r.e - r.b;
  for (int i = threadIdx.x; i < n; i += blockDim.x) it[i] = items[r.b + i];
  if (threadIdx.x == 0) {
    const SahTask t0{0, n, r.node, r.up, r.depth};
    top = 0;
    ntiny = 0;
    tiny_next = 0;
    dmax = 0;
    if (n <= TINY_MAX) pend[PEND_MAX - 1 - ntiny++] = t0;
    else pend[top++] = t0;
  }
  __syncthreads();
  while (top > 0) {
    const SahTask t = pend[top - 1];
    __syncthreads();
    if (threadIdx.x == 0) --top;
    split_task(it, tmp, t.b, t.e, t, bn, sc, nodes, &dmax, &ctl->bad);
    if (threadIdx.x == 0) {
      const int mid = sc.mid;
      const SahTask kids[2] = {{t.b, mid, t.node + 1, 2 * t.node, t.depth + 1},
                               {mid, t.e, t.node + (mid - t.b), 2 * t.node + 1, t.depth + 1}};
      for (const SahTask& c : kids) {
        if (c.e - c.b == 1) {
          put_leaf(nodes, c.up, it[c.b]);
          dmax = max(dmax, c.depth);
        } else if (top + ntiny >= PEND_MAX) {
          ctl->bad = 1;
        } else if (c.e - c.b <= TINY_MAX) {
          pend[PEND_MAX - 1 - ntiny++] = c;
        } else {
          pend[top++] = c;
        }
      }
    }
    __syncthreads();
  }
  // the tiny ranges, one warp each
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (;;) {
    int k = 0;
    if (lane == 0) k = atomicAdd(&tiny_next, 1);
    k = __shfl_sync(0xffffffffu, k, 0);
    if (k >= ntiny) break;
    tiny_subtree(it, pend[PEND_MAX - 1 - k], wstack + warp * (TINY_MAX / 2), nodes, &dmax, &ctl->bad);
  }
  __syncthreads();
  if (threadIdx.x == 0) atomicMax(&ctl->depth, dmax);
}

// the leaf items and the leaves' triangle stream (as repack.cpp's fill_leaf), a thread per leaf
__global__ void __launch_bounds__(ITEM_TB) k_leaf_items(const yc_bvh_node* __restrict__ nodes,
                                                        const int* __restrict__ leaf_node,
                                                        const int* __restrict__ leaf_first, int n_leaf,
                                                        const yc_triangle* __restrict__ tris, SahItem* items,
                                                        float4* stream) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n_leaf) return;
  const int i = leaf_node[j];
  const yc_bvh_node& n = nodes[i];
  const int first = leaf_first[j], count = n.vert_len;
  const int link = ~((first << 4) | count);
  items[j].lo = make_float4(n.aabb.p_min.x, n.aabb.p_min.y, n.aabb.p_min.z, __int_as_float(count));
  items[j].hi = make_float4(n.aabb.p_max.x, n.aabb.p_max.y, n.aabb.p_max.z, __int_as_float(link));
  for (int k = 0; k < count; ++k) {
    const int id = n.vert_list[k];
    const yc_triangle& t = tris[id];
    float4* r = stream + 3 * ((size_t)first + k);
    r[0] = make_float4(t.v1.x, t.v1.y, t.v1.z, __int_as_float(id));
    r[1] = make_float4(__fsub_rn(t.v2.x, t.v1.x), __fsub_rn(t.v2.y, t.v1.y), __fsub_rn(t.v2.z, t.v1.z),
                       __int_as_float(i * 16 + k));
    r[2] = make_float4(__fsub_rn(t.v3.x, t.v1.x), __fsub_rn(t.v3.y, t.v1.y), __fsub_rn(t.v3.z, t.v1.z), 0.0f);
  }
}

// ---- ranges of more than BIG_MIN leaves (the top of the tree): each pass over a range's
// leaves is spread over blocks of CHUNK leaves; the bounds and bins of the chunks are merged
// with the order-independent atomics of yc_sah.h, one block per range chooses the split
// from the merged bins, and the stable partition is a count per chunk, the chunks'
// offsets (an exclusive scan over the range's chunks in order, on the host) and a scatter
// per chunk ----
constexpr int BIG_MIN = 1 << 16;
constexpr int CHUNK = 8192;
constexpr int BIG_TB = 512;

struct BigChunk {
  int task, b, e;
};
struct BigSplit {
  int axis, at, mid, pad;
};
// a range's lo[3], hi[3], centroid lo[3], centroid hi[3], merged over its chunks
struct BigStat {
  float box[12];
};

__global__ void __launch_bounds__(256) k_big_init(BigStat* st, SahBins* gb) {
  const int t = blockIdx.x;
  if (threadIdx.x < 12) st[t].box[threadIdx.x] = ((threadIdx.x / 3) & 1) ? -kInf : kInf;
  SahBins& g = gb[t];
  for (int x = threadIdx.x; x < 3 * SAH_NB; x += blockDim.x) {
    const int k = x / SAH_NB, q = x - k * SAH_NB;
    g.cnt[k][q] = 0;
    g.w[k][q] = 0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      g.lo[k][c][q] = kInf;
      g.hi[k][c][q] = -kInf;
    }
  }
}

__global__ void __launch_bounds__(BIG_TB) k_big_bounds(const SahItem* items, const BigChunk* ch, BigStat* st) {
  __shared__ SahScratch sc;
  const BigChunk c = ch[blockIdx.x];
  range_bounds(items, c.b, c.e, sc);
  if (threadIdx.x < 12) {
    float* a = &st[c.task].box[threadIdx.x];
    if ((threadIdx.x / 3) & 1) sah_atomic_max(a, sc.box[threadIdx.x]);
    else sah_atomic_min(a, sc.box[threadIdx.x]);
  }
}

__global__ void __launch_bounds__(BIG_TB) k_big_bins(const SahItem* items, const BigChunk* ch, const SahTask* tasks,
                                                     const BigStat* st, SahBins* gb) {
  __shared__ SahBins bn;
  __shared__ SahScratch sc;
  const BigChunk c = ch[blockIdx.x];
  if (threadIdx.x < 12) sc.box[threadIdx.x] = st[c.task].box[threadIdx.x];
  __syncthreads();
  const SahTask t = tasks[c.task];
  const int nb = sah_bins_for(t.e - t.b);
  range_bins(items, c.b, c.e, nb, bn, sc);
  SahBins& g = gb[c.task];
  for (int x = threadIdx.x; x < 3 * nb; x += blockDim.x) {
    const int k = x / nb, q = x - k * nb;
    if (bn.cnt[k][q] == 0) continue;
    atomicAdd(&g.cnt[k][q], bn.cnt[k][q]);
    atomicAdd(&g.w[k][q], bn.w[k][q]);
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      sah_atomic_min(&g.lo[k][cc][q], bn.lo[k][cc][q]);
      sah_atomic_max(&g.hi[k][cc][q], bn.hi[k][cc][q]);
    }
  }
}

__global__ void __launch_bounds__(BIG_TB) k_big_split(const SahTask* tasks, const BigStat* st, const SahBins* gb,
                                                      BigSplit* out, float4* nodes, int* depth) {
  __shared__ SahBins bn;
  __shared__ SahScratch sc;
  const SahTask t = tasks[blockIdx.x];
  if (threadIdx.x < 12) sc.box[threadIdx.x] = st[blockIdx.x].box[threadIdx.x];
  const int nb = sah_bins_for(t.e - t.b);
  const SahBins& g = gb[blockIdx.x];
  for (int x = threadIdx.x; x < 3 * nb; x += blockDim.x) {
    const int k = x / nb, q = x - k * nb;
    bn.cnt[k][q] = g.cnt[k][q];
    bn.w[k][q] = g.w[k][q];
#pragma unroll
    for (int cc = 0; cc < 3; ++cc) {
      bn.lo[k][cc][q] = g.lo[k][cc][q];
      bn.hi[k][cc][q] = g.hi[k][cc][q];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const float lo[3] = {sc.box[0], sc.box[1], sc.box[2]}, hi[3] = {sc.box[3], sc.box[4], sc.box[5]};
    put_child(nodes, t.up, lo, hi, t.node);
    float* o = reinterpret_cast<float*>(nodes + 4 * (size_t)t.node);
    o[14] = 0.0f;
    o[15] = 0.0f;
    atomicMax(depth, t.depth);
  }
  range_split(t.b, t.e, nb, bn, sc);
  if (threadIdx.x == 0) out[blockIdx.x] = BigSplit{sc.axis, sc.at, sc.mid, 0};
}

// the chosen split's bin scale of range t on axis k, as range_bins and range_partition form it
__device__ __forceinline__ float big_scale(const BigStat& s, int k, int nb) {
  return (float)nb / (s.box[9 + k] - s.box[6 + k]);
}

__global__ void __launch_bounds__(BIG_TB) k_big_count(const SahItem* items, const BigChunk* ch, const SahTask* tasks,
                                                      const BigStat* st, const BigSplit* sp, int* left) {
  __shared__ int wsum[BIG_TB / 32];
  const BigChunk c = ch[blockIdx.x];
  const BigSplit s = sp[c.task];
  if (s.axis < 0) {
    if (threadIdx.x == 0) left[blockIdx.x] = 0;
    return;
  }
  const int k = s.axis;
  const SahTask t = tasks[c.task];
  const int nb = sah_bins_for(t.e - t.b);
  const float clo = st[c.task].box[6 + k], scale = big_scale(st[c.task], k, nb);
  int cnt = 0;
  for (int i = c.b + threadIdx.x; i < c.e; i += blockDim.x) {
    const SahItem x = items[i];
    cnt += sah_bin(sah_centroid(comp(x.lo, k), comp(x.hi, k)), clo, scale, nb) <= s.at ? 1 : 0;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    int total = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) total += wsum[w];
    left[blockIdx.x] = total;
  }
}

__global__ void __launch_bounds__(BIG_TB) k_big_scatter(const SahItem* items, SahItem* tmp, const BigChunk* ch,
                                                        const SahTask* tasks, const BigStat* st, const BigSplit* sp,
                                                        const int* loff, const int* roff, int* bad) {
  __shared__ int wcount[BIG_TB / 32];
  const BigChunk c = ch[blockIdx.x];
  const BigSplit s = sp[c.task];
  if (s.axis < 0) return;
  const int k = s.axis;
  const SahTask t = tasks[c.task];
  const int nb = sah_bins_for(t.e - t.b);
  const float clo = st[c.task].box[6 + k], scale = big_scale(st[c.task], k, nb);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  int run_l = t.b + loff[blockIdx.x], run_r = s.mid + roff[blockIdx.x];
  for (int base = c.b; base < c.e; base += blockDim.x) {
    const int i = base + threadIdx.x;
    const bool in = i < c.e;
    SahItem x;
    bool left = false;
    if (in) {
      x = items[i];
      left = sah_bin(sah_centroid(comp(x.lo, k), comp(x.hi, k)), clo, scale, nb) <= s.at;
    }
    const unsigned m = __ballot_sync(0xffffffffu, left);
    const int rank = __popc(m & ((1u << lane) - 1u));
    if (lane == 0) wcount[warp] = __popc(m);
    __syncthreads();
    int before = 0, total = 0;
    for (int w = 0; w < nw; ++w) {
      const int cw = wcount[w];
      before += w < warp ? cw : 0;
      total += cw;
    }
    if (in) {
      const int at = left ? run_l + before + rank : run_r + (int)threadIdx.x - before - rank;
      if (left ? (at >= t.b && at < s.mid) : (at >= s.mid && at < t.e)) tmp[at] = x;
      else *bad = 1;
    }
    run_l += total;
    run_r += min((int)blockDim.x, c.e - base) - total;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(BIG_TB) k_big_copy(SahItem* items, const SahItem* tmp, const BigChunk* ch,
                                                     const BigSplit* sp) {
  const BigChunk c = ch[blockIdx.x];
  if (sp[c.task].axis < 0) return;
  for (int i = c.b + threadIdx.x; i < c.e; i += blockDim.x) items[i] = tmp[i];
}

// leaf children of the big ranges: (parent * 2 + side, leaf item)
__global__ void __launch_bounds__(256) k_put_leaves(const SahItem* items, const int2* leaves, int n, float4* nodes) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) put_leaf(nodes, leaves[j].x, items[leaves[j].y]);
}

// a device temporary, freed on scope exit
template <class T>
struct Tmp {
  T* p = nullptr;
  ~Tmp() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)); }
};

}  // namespace

int repack_device(const yc_triangle* tris_host, int n_tri, const yc_bvh_node* nodes_host, int n_node,
                  const DevRepackPlan& plan, float4* nodes, float4* stream, float4* shade, int& depth, cudaStream_t s,
                  std::string& err) {
  const int n_leaf = (int)plan.leaf_node.size();
  if (n_leaf < 2 || n_tri <= 0 || n_node <= 0) {
    err = "device repack: the plan has fewer than two leaves";
    return -1;
  }
  auto cuda_fail = [&](cudaError_t e, const char* what) {
    err = std::string("device repack: ") + what + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? -2 : -1;
  };
#define YC_REPACK_CUDA(call, what)                  \
  do {                                              \
    const cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)
  const size_t cap_large = (size_t)n_leaf / (SMALL_MAX + 1) + 1;   // disjoint ranges of more than SMALL_MAX
  const size_t cap_small = (size_t)n_leaf / 2 + 1;                 // disjoint ranges of two leaves or more
  Tmp<yc_triangle> d_tris;
  Tmp<yc_bvh_node> d_nodes;
  Tmp<int> d_leaf, d_first;
  Tmp<SahItem> d_items, d_tmp;
  Tmp<SahTask> d_ta, d_tb, d_small;
  Tmp<SahCtl> d_ctl;
  YC_REPACK_CUDA(d_tris.alloc(n_tri), "allocation");
  YC_REPACK_CUDA(d_nodes.alloc(n_node), "allocation");
  YC_REPACK_CUDA(d_leaf.alloc(n_leaf), "allocation");
  YC_REPACK_CUDA(d_first.alloc(n_leaf), "allocation");
  YC_REPACK_CUDA(d_items.alloc(n_leaf), "allocation");
  YC_REPACK_CUDA(d_tmp.alloc(n_leaf), "allocation");
  YC_REPACK_CUDA(d_ta.alloc(cap_large), "allocation");
  YC_REPACK_CUDA(d_tb.alloc(cap_large), "allocation");
  YC_REPACK_CUDA(d_small.alloc(cap_small), "allocation");
  YC_REPACK_CUDA(d_ctl.alloc(1), "allocation");
  YC_REPACK_CUDA(cudaMemcpyAsync(d_tris.p, tris_host, (size_t)n_tri * sizeof(yc_triangle), cudaMemcpyHostToDevice, s),
                 "copy");
  YC_REPACK_CUDA(
      cudaMemcpyAsync(d_nodes.p, nodes_host, (size_t)n_node * sizeof(yc_bvh_node), cudaMemcpyHostToDevice, s), "copy");
  YC_REPACK_CUDA(cudaMemcpyAsync(d_leaf.p, plan.leaf_node.data(), (size_t)n_leaf * sizeof(int),
                                 cudaMemcpyHostToDevice, s),
                 "copy");
  YC_REPACK_CUDA(cudaMemcpyAsync(d_first.p, plan.leaf_first.data(), (size_t)n_leaf * sizeof(int),
                                 cudaMemcpyHostToDevice, s),
                 "copy");
  // shading records: the refit's kernel alone (no stream slots, no nodes)
  if (launch_refit(RefitPlan(), d_tris.p, n_tri, nullptr, nullptr, 0, shade, false, LINK_NONE, false, nullptr, s))
    return cuda_fail(cudaGetLastError(), "shading records");
  k_leaf_items<<<(n_leaf + ITEM_TB - 1) / ITEM_TB, ITEM_TB, 0, s>>>(d_nodes.p, d_leaf.p, d_first.p, n_leaf, d_tris.p,
                                                                   d_items.p, stream);
  YC_REPACK_CUDA(cudaPeekAtLastError(), "leaf items");
  const SahTask root{0, n_leaf, 0, -1, 0};
  SahCtl h_ctl{0, 0, 0, 0};
  YC_REPACK_CUDA(cudaMemcpyAsync(d_ctl.p, &h_ctl, sizeof(h_ctl), cudaMemcpyHostToDevice, s), "copy");
  // the ranges above BIG_MIN leaves, level by level, many blocks per range; their children
  // of more than SMALL_MAX leaves start the block-per-range levels, the smaller ones the
  // shared-memory subtrees, the single leaves a leaf record each
  std::vector<SahTask> big, lvl, sml;
  std::vector<int2> leaves;
  int host_depth = 0;
  if (n_leaf > BIG_MIN) big.push_back(root);
  else if (n_leaf > SMALL_MAX) lvl.push_back(root);
  else sml.push_back(root);
  if (!big.empty()) {
    const size_t cap_big = (size_t)n_leaf / (BIG_MIN + 1) + 1;
    const size_t cap_chunks = (size_t)n_leaf / CHUNK + 2 * cap_big + 1;
    Tmp<SahTask> d_big;
    Tmp<BigStat> d_stat;
    Tmp<SahBins> d_gbins;
    Tmp<BigSplit> d_split;
    Tmp<BigChunk> d_chunks;
    Tmp<int> d_left, d_loff, d_roff;
    YC_REPACK_CUDA(d_big.alloc(cap_big), "allocation");
    YC_REPACK_CUDA(d_stat.alloc(cap_big), "allocation");
    YC_REPACK_CUDA(d_gbins.alloc(cap_big), "allocation");
    YC_REPACK_CUDA(d_split.alloc(cap_big), "allocation");
    YC_REPACK_CUDA(d_chunks.alloc(cap_chunks), "allocation");
    YC_REPACK_CUDA(d_left.alloc(cap_chunks), "allocation");
    YC_REPACK_CUDA(d_loff.alloc(cap_chunks), "allocation");
    YC_REPACK_CUDA(d_roff.alloc(cap_chunks), "allocation");
    std::vector<BigChunk> chunks;
    std::vector<BigSplit> splits;
    std::vector<int> left, loff, roff;
    while (!big.empty()) {
      const int nt = (int)big.size();
      chunks.clear();
      for (int ti = 0; ti < nt; ++ti)
        for (int b = big[ti].b; b < big[ti].e; b += CHUNK) chunks.push_back(BigChunk{ti, b, std::min(b + CHUNK, big[ti].e)});
      const int nc = (int)chunks.size();
      if ((size_t)nt > cap_big || (size_t)nc > cap_chunks) {
        err = "device repack: too many top-level ranges";
        return -1;
      }
      YC_REPACK_CUDA(cudaMemcpyAsync(d_big.p, big.data(), nt * sizeof(SahTask), cudaMemcpyHostToDevice, s), "copy");
      YC_REPACK_CUDA(cudaMemcpyAsync(d_chunks.p, chunks.data(), nc * sizeof(BigChunk), cudaMemcpyHostToDevice, s),
                     "copy");
      k_big_init<<<nt, 256, 0, s>>>(d_stat.p, d_gbins.p);
      k_big_bounds<<<nc, BIG_TB, 0, s>>>(d_items.p, d_chunks.p, d_stat.p);
      k_big_bins<<<nc, BIG_TB, 0, s>>>(d_items.p, d_chunks.p, d_big.p, d_stat.p, d_gbins.p);
      k_big_split<<<nt, BIG_TB, 0, s>>>(d_big.p, d_stat.p, d_gbins.p, d_split.p, nodes, &d_ctl.p->depth);
      k_big_count<<<nc, BIG_TB, 0, s>>>(d_items.p, d_chunks.p, d_big.p, d_stat.p, d_split.p, d_left.p);
      YC_REPACK_CUDA(cudaPeekAtLastError(), "top-level split");
      splits.resize(nt);
      left.resize(nc);
      YC_REPACK_CUDA(cudaMemcpyAsync(splits.data(), d_split.p, nt * sizeof(BigSplit), cudaMemcpyDeviceToHost, s),
                     "copy");
      YC_REPACK_CUDA(cudaMemcpyAsync(left.data(), d_left.p, nc * sizeof(int), cudaMemcpyDeviceToHost, s), "copy");
      YC_REPACK_CUDA(cudaStreamSynchronize(s), "top-level split");
      // each chunk's place on its range's two sides: the chunks before it in order
      loff.resize(nc);
      roff.resize(nc);
      std::vector<int> run_l(nt, 0), run_r(nt, 0);
      for (int ci = 0; ci < nc; ++ci) {
        const int ti = chunks[ci].task;
        loff[ci] = run_l[ti];
        roff[ci] = run_r[ti];
        run_l[ti] += left[ci];
        run_r[ti] += (chunks[ci].e - chunks[ci].b) - left[ci];
      }
      for (int ti = 0; ti < nt; ++ti)
        if (splits[ti].axis >= 0 && big[ti].b + run_l[ti] != splits[ti].mid) {
          err = "device repack: the bins and the partition of a top-level range disagree";
          return -1;
        }
      YC_REPACK_CUDA(cudaMemcpyAsync(d_loff.p, loff.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
      YC_REPACK_CUDA(cudaMemcpyAsync(d_roff.p, roff.data(), nc * sizeof(int), cudaMemcpyHostToDevice, s), "copy");
      k_big_scatter<<<nc, BIG_TB, 0, s>>>(d_items.p, d_tmp.p, d_chunks.p, d_big.p, d_stat.p, d_split.p, d_loff.p,
                                          d_roff.p, &d_ctl.p->bad);
      k_big_copy<<<nc, BIG_TB, 0, s>>>(d_items.p, d_tmp.p, d_chunks.p, d_split.p);
      YC_REPACK_CUDA(cudaPeekAtLastError(), "top-level partition");
      std::vector<SahTask> next;
      for (int ti = 0; ti < nt; ++ti) {
        const SahTask& t = big[ti];
        const int mid = splits[ti].mid;
        const SahTask kids[2] = {{t.b, mid, t.node + 1, 2 * t.node, t.depth + 1},
                                 {mid, t.e, t.node + (mid - t.b), 2 * t.node + 1, t.depth + 1}};
        for (const SahTask& c : kids) {
          const int n = c.e - c.b;
          if (n == 1) {
            leaves.push_back(make_int2(c.up, c.b));
            host_depth = std::max(host_depth, c.depth);
          } else if (n > BIG_MIN) {
            next.push_back(c);
          } else if (n > SMALL_MAX) {
            lvl.push_back(c);
          } else {
            sml.push_back(c);
          }
        }
      }
      big.swap(next);
      YC_REPACK_CUDA(cudaStreamSynchronize(s), "top-level partition");   // the host vectors above are reused
    }
    if (!leaves.empty()) {
      Tmp<int2> d_leaves;
      YC_REPACK_CUDA(d_leaves.alloc(leaves.size()), "allocation");
      YC_REPACK_CUDA(cudaMemcpyAsync(d_leaves.p, leaves.data(), leaves.size() * sizeof(int2), cudaMemcpyHostToDevice,
                                     s),
                     "copy");
      k_put_leaves<<<((int)leaves.size() + 255) / 256, 256, 0, s>>>(d_items.p, d_leaves.p, (int)leaves.size(), nodes);
      YC_REPACK_CUDA(cudaPeekAtLastError(), "leaf records");
      YC_REPACK_CUDA(cudaStreamSynchronize(s), "leaf records");
    }
  }
  if (lvl.size() > cap_large || sml.size() > cap_small) {
    err = "device repack: a split left its bounds";
    return -1;
  }
  int n_large = (int)lvl.size();
  YC_REPACK_CUDA(cudaMemcpyAsync(&h_ctl, d_ctl.p, sizeof(h_ctl), cudaMemcpyDeviceToHost, s), "copy");
  YC_REPACK_CUDA(cudaStreamSynchronize(s), "upload");
  h_ctl.n_next = 0;
  h_ctl.n_small = (int)sml.size();
  h_ctl.depth = std::max(h_ctl.depth, host_depth);
  if (n_large)
    YC_REPACK_CUDA(cudaMemcpyAsync(d_ta.p, lvl.data(), lvl.size() * sizeof(SahTask), cudaMemcpyHostToDevice, s),
                   "copy");
  if (!sml.empty())
    YC_REPACK_CUDA(cudaMemcpyAsync(d_small.p, sml.data(), sml.size() * sizeof(SahTask), cudaMemcpyHostToDevice, s),
                   "copy");
  YC_REPACK_CUDA(cudaMemcpyAsync(d_ctl.p, &h_ctl, sizeof(h_ctl), cudaMemcpyHostToDevice, s), "copy");
  YC_REPACK_CUDA(cudaStreamSynchronize(s), "upload");   // h_ctl and the lists are read by the copies above
  while (n_large > 0) {
    k_sah_level<<<n_large, LEVEL_TB, 0, s>>>(d_items.p, d_tmp.p, d_ta.p, d_tb.p, (int)cap_large, d_small.p,
                                             (int)cap_small, d_ctl.p, nodes);
    YC_REPACK_CUDA(cudaPeekAtLastError(), "split level");
    YC_REPACK_CUDA(cudaMemcpyAsync(&h_ctl, d_ctl.p, sizeof(h_ctl), cudaMemcpyDeviceToHost, s), "copy");
    YC_REPACK_CUDA(cudaStreamSynchronize(s), "split level");
    n_large = h_ctl.n_next;
    if (h_ctl.bad || (size_t)n_large > cap_large || (size_t)h_ctl.n_small > cap_small) {
      err = "device repack: a split left its bounds";
      return -1;
    }
    YC_REPACK_CUDA(cudaMemsetAsync(&d_ctl.p->n_next, 0, sizeof(int), s), "reset");
    std::swap(d_ta.p, d_tb.p);
  }
  if (h_ctl.n_small > 0) {
    YC_REPACK_CUDA(cudaFuncSetAttribute(k_sah_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmallSmem),
                   "shared memory");
    k_sah_small<<<h_ctl.n_small, SMALL_TB, kSmallSmem, s>>>(d_items.p, d_small.p, d_ctl.p, nodes);
    YC_REPACK_CUDA(cudaPeekAtLastError(), "subtrees");
  }
  YC_REPACK_CUDA(cudaMemcpyAsync(&h_ctl, d_ctl.p, sizeof(h_ctl), cudaMemcpyDeviceToHost, s), "copy");
  YC_REPACK_CUDA(cudaStreamSynchronize(s), "subtrees");
#undef YC_REPACK_CUDA
  if (h_ctl.bad) {
    err = "device repack: a split left its bounds";
    return -1;
  }
  depth = h_ctl.depth + 1;
  return 0;
}

}  // namespace yc
