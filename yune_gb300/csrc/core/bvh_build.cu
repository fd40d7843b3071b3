// bvh_build.cu -- BVH::createBVH (src/BVH.cpp:56-173, :175-247) on the GPU, level by level.
//
// Produces the reference's node array: breadth-first order, the same split axis, bin
// planes, costs, membership and median fallback, evaluated with the same FP32 operations
// (this unit is compiled with -fmad=false), and the same bottom-up refit. The host
// restatement (csrc/host/yh_bvh.cpp) is the specification; the tests compare the two node
// arrays. One level of the tree is one round of kernels:
//   bounds   per node, the union of its primitives' padded boxes (atomic min/max on
//            order-preserving integer images of the floats)
//   hist     per primitive, its bin (the first plane not below its centroid, when the
//            centroid lies in the node box) into the node's histogram
//   decide   one thread per node: leaf, empty, binned SAH split or spatial median
//   scan     child slots for the splitting nodes, in node order (breadth-first numbering)
//   flags    per primitive, whether its centroid lies in the first child's box
//   scan     positions of a stable partition of every node's segment
//   scatter  primitives into their children's segments
// then a refit over the levels in reverse. The only liberty taken: a box bound that is
// zero is stored as +0 (atomics cannot keep "the first of -0 and +0 met", which the
// sequential builder does); the traversal's arithmetic is the same for either zero.
#include <climits>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "yc_internal.h"

namespace yc {

namespace {

constexpr int BB_TB = 256;
constexpr float FMAX = 3.402823466e+38f;
// trees deeper than this are refused: more than leaf_max triangles with one centroid are
// never separated, and the reference builder does not terminate on them
constexpr int kMaxLevels = 1024;

__device__ __forceinline__ int ord(float f) {   // monotone map float -> int (+0 for both zeros)
  const int i = __float_as_int(f + 0.0f);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float unord(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

__device__ __forceinline__ float get(const yc_float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void put(yc_float4& v, int a, float x) {
  if (a == 0) v.x = x; else if (a == 1) v.y = x; else v.z = x;
}
__device__ __forceinline__ float surface_area(const yc_aabb& b) {
  const float d0 = b.p_max.x - b.p_min.x, d1 = b.p_max.y - b.p_min.y, d2 = b.p_max.z - b.p_min.z;
  return 2 * (d0 * d1 + d0 * d2 + d1 * d2);
}

__device__ __forceinline__ void fresh(yc_bvh_node& g, const yc_aabb& box) {
  g.aabb = box;
  for (int k = 0; k < 10; ++k) g.vert_list[k] = -1;
  g.child_idx = -2;
  g.vert_len = -1;
}

// TriangleCPU::computeCentroid / computeAABB (src/TriangleCPU.cpp:41-71)
__global__ void k_tri_info(const yc_triangle* __restrict__ t, int n, float4* cen, float4* lo, float4* hi, int* root) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = i < n;
  int rl[3] = {INT_MAX, INT_MAX, INT_MAX}, rh[3] = {INT_MIN, INT_MIN, INT_MIN};
  if (act) {
    const yc_triangle tr = t[i];
    const float a[3] = {tr.v1.x, tr.v1.y, tr.v1.z}, b[3] = {tr.v2.x, tr.v2.y, tr.v2.z}, c[3] = {tr.v3.x, tr.v3.y, tr.v3.z};
    float ce[3], l[3], h[3];
    for (int k = 0; k < 3; ++k) {
      ce[k] = ((a[k] + b[k]) + c[k]) / 3.0f;
      l[k] = fminf(a[k], fminf(b[k], c[k]));
      h[k] = fmaxf(a[k], fmaxf(b[k], c[k]));
      if (h[k] - l[k] == 0.0f) h[k] += 0.2f;
      rl[k] = ord(l[k]);
      rh[k] = ord(h[k]);
    }
    cen[i] = make_float4(ce[0], ce[1], ce[2], 0.0f);
    lo[i] = make_float4(l[0], l[1], l[2], 0.0f);
    hi[i] = make_float4(h[0], h[1], h[2], 0.0f);
  }
  // the scene box: one update per warp (lanes past n carry the neutral values)
  for (int k = 0; k < 3; ++k) {
    rl[k] = __reduce_min_sync(0xffffffffu, rl[k]);
    rh[k] = __reduce_max_sync(0xffffffffu, rh[k]);
  }
  if ((threadIdx.x & 31) == 0 && rl[0] != INT_MAX) {
    for (int k = 0; k < 3; ++k) {
      atomicMin(&root[k], rl[k]);
      atomicMax(&root[3 + k], rh[k]);
    }
  }
}

__global__ void k_iota(int* a, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = i;
}

// per-node working state of the level being split
struct NodeWork {
  int s, e;          // segment of perm
  int box[6];        // union of the primitives' boxes, ord() images (min xyz, max xyz)
  int split;         // 1: the node splits into two children
  int n1;            // primitives of the first child
  int axis;
  int pad;
};

__global__ void k_root(yc_bvh_node* nodes, NodeWork* work, const int* root, int n) {
  yc_aabb box;
  box.p_min = yc_float4{unord(root[0]), unord(root[1]), unord(root[2]), 1.0f};
  box.p_max = yc_float4{unord(root[3]), unord(root[4]), unord(root[5]), 1.0f};
  fresh(nodes[0], box);
  work[0].s = 0;
  work[0].e = n;
}

__global__ void k_level_clear(NodeWork* work, int* hist, int a, int b, int bins) {
  const int i = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= b) return;
  NodeWork& w = work[i];
  for (int k = 0; k < 3; ++k) { w.box[k] = 0x7fffffff; w.box[3 + k] = (int)0x80000000; }
  w.split = 0;
  w.n1 = 0;
  for (int k = 0; k < bins; ++k) hist[(size_t)(i - a) * bins + k] = 0;
}

// primitives of the level's nodes that can split: their node's box union. A node's
// primitives are contiguous in perm, so the lanes of a warp mostly share one node: they
// combine their boxes first and one lane per run of equal nodes updates the node (six
// atomics per run instead of per primitive; min and max of the ord() images are exact
// in any order). Every lane reaches the match, lanes without work with a key of their own.
__global__ void k_bounds(const int* __restrict__ perm, const int* __restrict__ pnode, const float4* __restrict__ lo,
                         const float4* __restrict__ hi, NodeWork* work, int n, int a, int b, int leaf_max) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int nd = -1;
  bool act = false;
  if (i < n) {
    nd = pnode[i];
    act = nd >= a && nd < b && work[nd].e - work[nd].s > leaf_max;
  }
  const unsigned peers = __match_any_sync(0xffffffffu, act ? nd : -1 - lane);
  if (!act) return;
  const float4 l = lo[perm[i]], h = hi[perm[i]];
  const int x0 = __reduce_min_sync(peers, ord(l.x)), y0 = __reduce_min_sync(peers, ord(l.y));
  const int z0 = __reduce_min_sync(peers, ord(l.z));
  const int x1 = __reduce_max_sync(peers, ord(h.x)), y1 = __reduce_max_sync(peers, ord(h.y));
  const int z1 = __reduce_max_sync(peers, ord(h.z));
  if (lane == __ffs(peers) - 1) {
    NodeWork& w = work[nd];
    atomicMin(&w.box[0], x0); atomicMin(&w.box[1], y0); atomicMin(&w.box[2], z0);
    atomicMax(&w.box[3], x1); atomicMax(&w.box[4], y1); atomicMax(&w.box[5], z1);
  }
}

// split axis: the longest extent of the union (BVH.cpp:280-314)
__device__ __forceinline__ int split_axis(const NodeWork& w) {
  int axis = 0;
  float diff = -FMAX;
  for (int k = 0; k < 3; ++k) {
    const float d = unord(w.box[3 + k]) - unord(w.box[k]);
    if (d > diff) { diff = d; axis = k; }
  }
  return axis;
}

// the bin of primitive perm[i] of node nd (BVH.cpp:93-126): the first plane not below its
// centroid, by binary search
__device__ __forceinline__ int bin_of(const int* __restrict__ perm, const float4* __restrict__ cen,
                                      const yc_bvh_node* nodes, const NodeWork* work, int i, int nd, int bins) {
  const NodeWork& w = work[nd];
  const int axis = split_axis(w);
  const yc_aabb pbox = nodes[nd].aabb;
  const float4 c4 = cen[perm[i]];
  const float c[3] = {c4.x, c4.y, c4.z};
  const float bl[3] = {pbox.p_min.x, pbox.p_min.y, pbox.p_min.z}, bh[3] = {pbox.p_max.x, pbox.p_max.y, pbox.p_max.z};
  bool inside = true;
  for (int k = 0; k < 3; ++k) {
    if (k == axis) { if (c[k] < bl[k]) inside = false; }
    else if (c[k] < bl[k] || c[k] > bh[k]) inside = false;
  }
  const int nsplit = bins - 1;
  int first = nsplit;
  if (inside) {
    float inc = get(pbox.p_max, axis) - get(pbox.p_min, axis);
    inc /= (float)bins;
    const float base = get(pbox.p_min, axis);
    int lo_ = 0, hi_ = nsplit;   // lower_bound over plane[b] = base + (b + 1) * inc
    while (lo_ < hi_) {
      const int mid = (lo_ + hi_) >> 1;
      const float plane = base + (float)(mid + 1) * inc;
      if (plane < c[axis]) lo_ = mid + 1; else hi_ = mid;
    }
    first = lo_;
  }
  return first;
}

// bin counts of the level's nodes that split by SAH
__global__ void k_hist(const int* __restrict__ perm, const int* __restrict__ pnode, const float4* __restrict__ cen,
                       const yc_bvh_node* nodes, NodeWork* work, int* hist, int n, int a, int b, int bins,
                       int leaf_max) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int nd = -1;
  bool act = false;
  if (i < n) {
    nd = pnode[i];
    if (nd >= a && nd < b) {
      const int np = work[nd].e - work[nd].s;
      act = np > leaf_max && bins > 2 && np > 20;
    }
  }
  int key = -1 - lane;   // lanes without work: a key no other lane has
  if (act) key = (nd - a) * bins + bin_of(perm, cen, nodes, work, i, nd, bins);
  // lanes that fall in the same bin of the same node add once (counts are exact in any order)
  const unsigned peers = __match_any_sync(0xffffffffu, key);
  if (act && lane == __ffs(peers) - 1) atomicAdd(&hist[key], __popc(peers));
}

// one thread per node: leaf, empty, binned SAH split or spatial median (BVH.cpp:69-160)
__global__ void k_decide(const int* __restrict__ perm, yc_bvh_node* nodes, NodeWork* work, const int* hist,
                         yc_aabb* child_box, int a, int b, int bins, int leaf_max) {
  const int nd = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (nd >= b) return;
  NodeWork& w = work[nd];
  yc_bvh_node& g = nodes[nd];
  const int np = w.e - w.s;
  if (np == 0) return;
  if (np <= leaf_max) {
    g.vert_len = np;
    g.child_idx = -1;
    for (int j = 0; j < np; ++j) g.vert_list[j] = perm[w.s + j];
    return;
  }
  const int axis = split_axis(w);
  w.axis = axis;
  const yc_aabb pbox = g.aabb;
  bool median = false;
  yc_aabb best1 = pbox, best2 = pbox;
  if (bins > 2 && np > 20) {
    const float cost_isect = 1.0f, cost_trav = 1 / 8.0f;
    float cost = surface_area(pbox) * cost_isect * (float)np;
    const float initial_cost = cost;
    float inc = get(pbox.p_max, axis) - get(pbox.p_min, axis);
    inc /= (float)bins;
    const float sa_p = surface_area(pbox);
    const int* h = hist + (size_t)(nd - a) * bins;
    int below = 0;
    for (int k = 0; k < bins - 1; ++k) {
      below += h[k];
      const float plane = get(pbox.p_min, axis) + (float)(k + 1) * inc;
      yc_aabb c1 = pbox, c2 = pbox;
      put(c1.p_max, axis, plane);
      put(c2.p_min, axis, plane);
      int n1, n2;
      if (surface_area(c1) == 0.0f) { n1 = 0; n2 = np; }
      else if (surface_area(c2) == 0.0f) { n1 = np; n2 = 0; }
      else { n1 = below; n2 = np - below; }
      const float new_cost = cost_trav + (surface_area(c1) / sa_p) * (cost_isect * (float)n1) +
                             surface_area(c2) / sa_p * (cost_isect * (float)n2);
      if (new_cost < cost) {
        best1 = c1; best2 = c2;
        cost = new_cost;
      }
    }
    if (cost == initial_cost) median = true;
  } else {
    median = true;
  }
  if (median) {
    const float center = (get(pbox.p_min, axis) + get(pbox.p_max, axis)) / 2.0f;
    best1 = pbox; best2 = pbox;
    put(best1.p_max, axis, center);
    put(best2.p_min, axis, center);
  }
  w.split = 1;
  child_box[2 * (size_t)(nd - a)] = best1;
  child_box[2 * (size_t)(nd - a) + 1] = best2;
}

// membership of each primitive in its node's first child (BVH.cpp:175-216)
__global__ void k_flags(const int* __restrict__ perm, const int* __restrict__ pnode, const float4* __restrict__ cen,
                        const NodeWork* work, const yc_aabb* child_box, int* flag, int n, int a, int b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nd = pnode[i];
  int f = 0;
  if (nd >= a && nd < b && work[nd].split) {
    const yc_aabb b1 = child_box[2 * (size_t)(nd - a)], b2 = child_box[2 * (size_t)(nd - a) + 1];
    if (surface_area(b1) == 0.0f) f = 0;
    else if (surface_area(b2) == 0.0f) f = 1;
    else {
      const float4 c = cen[perm[i]];
      f = (c.x < b1.p_min.x || c.x > b1.p_max.x || c.y < b1.p_min.y || c.y > b1.p_max.y || c.z < b1.p_min.z ||
           c.z > b1.p_max.z) ? 0 : 1;
    }
  }
  flag[i] = f;
}

// exclusive scan of n ints in tiles of 1024 (tile sums scanned in one block, then added)
__global__ void k_scan_tiles(const int* in, int* out, int* tile_sum, int n) {
  __shared__ int s_sum[32];
  const int i = blockIdx.x * 1024 + threadIdx.x;
  const int v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = v;
  for (int off = 1; off < 32; off <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += u;
  }
  if (lane == 31) s_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int w = s_sum[lane];
    for (int off = 1; off < 32; off <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += u;
    }
    s_sum[lane] = w;
  }
  __syncthreads();
  if (i < n) out[i] = incl - v + (warp > 0 ? s_sum[warp - 1] : 0);
  if (threadIdx.x == 1023) tile_sum[blockIdx.x] = s_sum[31];
}

__global__ void k_scan_sums(int* tile_sum, int tiles) {   // one block: exclusive scan in place
  __shared__ int s_sum[32];
  const int per = (tiles + blockDim.x - 1) / blockDim.x;
  const int i0 = threadIdx.x * per;
  int sum = 0;
  for (int k = 0; k < per; ++k)
    if (i0 + k < tiles) sum += tile_sum[i0 + k];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int incl = sum;
  for (int off = 1; off < 32; off <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += v;
  }
  if (lane == 31) s_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int v = lane < (int)(blockDim.x >> 5) ? s_sum[lane] : 0;
    for (int off = 1; off < 32; off <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, off);
      if (lane >= off) v += u;
    }
    s_sum[lane] = v;
  }
  __syncthreads();
  int run = incl - sum + (warp > 0 ? s_sum[warp - 1] : 0);
  for (int k = 0; k < per; ++k)
    if (i0 + k < tiles) {
      const int x = tile_sum[i0 + k];
      tile_sum[i0 + k] = run;
      run += x;
    }
}

__global__ void k_scan_add(int* out, const int* tile_sum, int n) {
  const int i = blockIdx.x * 1024 + threadIdx.x;
  if (i < n) out[i] += tile_sum[blockIdx.x];
}

// child slots of a level by the tiled scan: the split flags of its nodes, then (after
// k_scan_tiles / k_scan_sums) each splitting node's slot and the level's split count
__global__ void k_split_flags(const NodeWork* work, int* flag, int a, int b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (a + i < b) flag[i] = work[a + i].split;
}
__global__ void k_slots_finish(const int* flag, const int* tile_sum, int* child_of, int count, int* total) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const int slot = child_of[i] + tile_sum[i >> 10];
  child_of[i] = flag[i] ? slot : -1;
  if (i == count - 1) *total = slot + flag[i];
}

// per splitting node: the first child's count, the children's nodes and segments
__global__ void k_children(yc_bvh_node* nodes, NodeWork* work, const yc_aabb* child_box, const int* child_of,
                           const int* pos, const int* flag, int a, int b, int next) {
  const int nd = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (nd >= b) return;
  NodeWork& w = work[nd];
  if (!w.split) return;
  const int e1 = w.e - 1;
  w.n1 = (pos[e1] + flag[e1]) - pos[w.s];
  const int c = next + 2 * child_of[nd - a];
  nodes[nd].child_idx = c;
  fresh(nodes[c], child_box[2 * (size_t)(nd - a)]);
  fresh(nodes[c + 1], child_box[2 * (size_t)(nd - a) + 1]);
  work[c].s = w.s;
  work[c].e = w.s + w.n1;
  work[c + 1].s = w.s + w.n1;
  work[c + 1].e = w.e;
}

// stable partition of every splitting node's segment; the other primitives stay put
__global__ void k_scatter(const int* __restrict__ perm, const int* __restrict__ pnode, const NodeWork* work,
                          const yc_bvh_node* nodes, const int* pos, const int* flag, int* perm_out, int* pnode_out,
                          int n, int a, int b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int nd = pnode[i];
  if (nd < a || nd >= b || !work[nd].split) {
    perm_out[i] = perm[i];
    pnode_out[i] = nd;
    return;
  }
  const NodeWork& w = work[nd];
  const int before1 = pos[i] - pos[w.s];   // first-child members before i in the segment
  const int c = nodes[nd].child_idx;
  int dst, child;
  if (flag[i]) { dst = w.s + before1; child = c; }
  else { dst = w.s + w.n1 + (i - w.s - before1); child = c + 1; }
  perm_out[dst] = perm[i];
  pnode_out[dst] = child;
}

// bottom-up refit (BVH.cpp:218-247): leaves take the union of their triangles' padded
// boxes, interior nodes the union of their children; empty nodes keep their box
__global__ void k_refit(yc_bvh_node* nodes, const float4* __restrict__ lo, const float4* __restrict__ hi, int a,
                        int b) {
  const int j = a + blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= b) return;
  yc_bvh_node& g = nodes[j];
  if (g.vert_len > 0) {
    float l[3] = {FMAX, FMAX, FMAX}, h[3] = {-FMAX, -FMAX, -FMAX};
    for (int k = 0; k < g.vert_len; ++k) {
      const float4 pl = lo[g.vert_list[k]], ph = hi[g.vert_list[k]];
      l[0] = fminf(pl.x, l[0]); l[1] = fminf(pl.y, l[1]); l[2] = fminf(pl.z, l[2]);
      h[0] = fmaxf(ph.x, h[0]); h[1] = fmaxf(ph.y, h[1]); h[2] = fmaxf(ph.z, h[2]);
    }
    g.aabb.p_min = yc_float4{l[0], l[1], l[2], 1.0f};
    g.aabb.p_max = yc_float4{h[0], h[1], h[2], 1.0f};
  } else if (g.child_idx > 0) {
    const yc_aabb& p = nodes[g.child_idx].aabb;
    const yc_aabb& q = nodes[g.child_idx + 1].aabb;
    g.aabb.p_min = yc_float4{fminf(q.p_min.x, p.p_min.x), fminf(q.p_min.y, p.p_min.y), fminf(q.p_min.z, p.p_min.z),
                             p.p_min.w};
    g.aabb.p_max = yc_float4{fmaxf(q.p_max.x, p.p_max.x), fmaxf(q.p_max.y, p.p_max.y), fmaxf(q.p_max.z, p.p_max.z),
                             p.p_max.w};
  }
}

template <class T>
struct Buf {
  T* p = nullptr;
  size_t n = 0;
  ~Buf() { if (p) cudaFree(p); }
  cudaError_t need(size_t count, cudaStream_t s, bool keep = false) {
    if (count <= n) return cudaSuccess;
    T* q = nullptr;
    const size_t cap = std::max(count, n + n / 2);
    cudaError_t e = cudaMalloc(&q, cap * sizeof(T));
    if (e != cudaSuccess) return e;
    if (keep && p) e = cudaMemcpyAsync(q, p, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
    if (p) { cudaStreamSynchronize(s); cudaFree(p); }
    p = q;
    n = cap;
    return e;
  }
};

#define BB_CHECK(x)                           \
  do {                                        \
    const cudaError_t e_ = (x);               \
    if (e_ != cudaSuccess) return e_;         \
  } while (0)

}  // namespace

cudaError_t bvh_build_device(const yc_triangle* tris_dev, int n, int bins, int leaf_max, cudaStream_t s,
                             std::vector<yc_bvh_node>& out, int& depth, bool& too_deep) {
  out.clear();
  depth = 0;
  too_deep = false;
  if (n <= 0) return cudaSuccess;
  Buf<float4> cen, lo, hi;
  Buf<int> perm, perm2, pnode, pnode2, flag, pos, tiles, root, child_of, hist, total, nflag, ntile;
  Buf<yc_bvh_node> nodes;
  Buf<NodeWork> work;
  Buf<yc_aabb> child_box;
  BB_CHECK(cen.need(n, s)); BB_CHECK(lo.need(n, s)); BB_CHECK(hi.need(n, s));
  BB_CHECK(perm.need(n, s)); BB_CHECK(perm2.need(n, s)); BB_CHECK(pnode.need(n, s)); BB_CHECK(pnode2.need(n, s));
  BB_CHECK(flag.need(n, s)); BB_CHECK(pos.need(n, s));
  const int ntiles = (n + 1023) / 1024;
  BB_CHECK(tiles.need(ntiles, s)); BB_CHECK(root.need(6, s)); BB_CHECK(total.need(1, s));
  const int init_root[6] = {0x7fffffff, 0x7fffffff, 0x7fffffff, (int)0x80000000, (int)0x80000000, (int)0x80000000};
  BB_CHECK(cudaMemcpyAsync(root.p, init_root, sizeof(init_root), cudaMemcpyHostToDevice, s));
  const int gp = (n + BB_TB - 1) / BB_TB;
  k_tri_info<<<gp, BB_TB, 0, s>>>(tris_dev, n, cen.p, lo.p, hi.p, root.p);
  // perm = identity, every primitive in the root
  k_iota<<<gp, BB_TB, 0, s>>>(perm.p, n);
  BB_CHECK(cudaMemsetAsync(pnode.p, 0, n * sizeof(int), s));
  BB_CHECK(nodes.need(1024, s)); BB_CHECK(work.need(1024, s));
  k_root<<<1, 1, 0, s>>>(nodes.p, work.p, root.p, n);
  std::vector<int> level_start = {0};
  int a = 0, b = 1;
  while (a < b) {
    const int cnt = b - a;
    BB_CHECK(hist.need((size_t)cnt * bins, s)); BB_CHECK(child_of.need(cnt, s)); BB_CHECK(child_box.need(2 * (size_t)cnt, s));
    const int gn = (cnt + BB_TB - 1) / BB_TB;
    k_level_clear<<<gn, BB_TB, 0, s>>>(work.p, hist.p, a, b, bins);
    k_bounds<<<gp, BB_TB, 0, s>>>(perm.p, pnode.p, lo.p, hi.p, work.p, n, a, b, leaf_max);
    k_hist<<<gp, BB_TB, 0, s>>>(perm.p, pnode.p, cen.p, nodes.p, work.p, hist.p, n, a, b, bins, leaf_max);
    k_decide<<<gn, BB_TB, 0, s>>>(perm.p, nodes.p, work.p, hist.p, child_box.p, a, b, bins, leaf_max);
    {   // child slots in node order: an exclusive scan of the split flags
      const int ct = (cnt + 1023) / 1024;
      BB_CHECK(nflag.need(cnt, s)); BB_CHECK(ntile.need(ct, s));
      k_split_flags<<<gn, BB_TB, 0, s>>>(work.p, nflag.p, a, b);
      k_scan_tiles<<<ct, 1024, 0, s>>>(nflag.p, child_of.p, ntile.p, cnt);
      k_scan_sums<<<1, 1024, 0, s>>>(ntile.p, ct);
      k_slots_finish<<<gn, BB_TB, 0, s>>>(nflag.p, ntile.p, child_of.p, cnt, total.p);
    }
    int splits = 0;
    BB_CHECK(cudaMemcpyAsync(&splits, total.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    BB_CHECK(cudaStreamSynchronize(s));
    if (splits == 0) break;
    const int next = b;
    BB_CHECK(nodes.need((size_t)b + 2 * splits, s, true));
    BB_CHECK(work.need((size_t)b + 2 * splits, s, true));
    k_flags<<<gp, BB_TB, 0, s>>>(perm.p, pnode.p, cen.p, work.p, child_box.p, flag.p, n, a, b);
    k_scan_tiles<<<ntiles, 1024, 0, s>>>(flag.p, pos.p, tiles.p, n);
    k_scan_sums<<<1, 1024, 0, s>>>(tiles.p, ntiles);
    k_scan_add<<<ntiles, 1024, 0, s>>>(pos.p, tiles.p, n);
    k_children<<<gn, BB_TB, 0, s>>>(nodes.p, work.p, child_box.p, child_of.p, pos.p, flag.p, a, b, next);
    k_scatter<<<gp, BB_TB, 0, s>>>(perm.p, pnode.p, work.p, nodes.p, pos.p, flag.p, perm2.p, pnode2.p, n, a, b);
    std::swap(perm.p, perm2.p);
    std::swap(pnode.p, pnode2.p);
    BB_CHECK(cudaPeekAtLastError());
    a = b;
    b = b + 2 * splits;
    level_start.push_back(a);
    if ((int)level_start.size() > kMaxLevels) {   // a split that moves nothing, forever
      too_deep = true;
      return cudaSuccess;
    }
  }
  const int total_nodes = b;
  level_start.push_back(total_nodes);
  for (int l = (int)level_start.size() - 2; l >= 0; --l) {
    const int la = level_start[l], lb = level_start[l + 1];
    if (lb > la) k_refit<<<(lb - la + BB_TB - 1) / BB_TB, BB_TB, 0, s>>>(nodes.p, lo.p, hi.p, la, lb);
  }
  BB_CHECK(cudaPeekAtLastError());
  out.resize(total_nodes);
  BB_CHECK(cudaMemcpyAsync(out.data(), nodes.p, total_nodes * sizeof(yc_bvh_node), cudaMemcpyDeviceToHost, s));
  BB_CHECK(cudaStreamSynchronize(s));
  depth = (int)level_start.size() - 2;
  return cudaSuccess;
}

}  // namespace yc
