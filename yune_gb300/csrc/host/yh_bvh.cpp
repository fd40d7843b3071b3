// yh_bvh.cpp -- the breadth-first binned BVH of Yune's BVH::createBVH, restated.
//
// The node array this produces is the one src/BVH.cpp:56-173 produces for the same
// triangles, bins and leaf size (tests/test_oracle_pin.py compares the two node by
// node). The arithmetic that decides splits is kept in the reference's order, in
// float, so every comparison takes the same branch:
//   split axis    longest extent of the union of triangle boxes (BVH.cpp:280-314)
//   bin planes    parent box min + (i+1) * (extent / bins)      (BVH.cpp:93-106)
//   bin cost      1/8 + SA(c1)/SA(p) * n1 + SA(c2)/SA(p) * n2    (BVH.cpp:113-115)
//   membership    centroid inside the child-1 box on all three axes, inclusive
//                 (BVH.cpp:175-216); the rest go to child 2
//   fallback      spatial median of the parent box (BVH.cpp:145-160)
//   refit         leaves = union of padded triangle boxes, interior = union of
//                 both children, empty nodes keep their spatial box (BVH.cpp:218-247)
// What differs is the cost of the build. The reference copies a primitive vector per
// node and re-partitions the primitives once per bin (O(bins * n) with allocation).
// Here each node counts its primitives per bin once with a binary search over the
// monotone bin planes and a prefix sum (O(n log bins)), the primitives live in one
// permutation array (a node owns a range of it, split in place in order), and the build
// runs level by level on all host cores: the nodes of a level decide independently
// (large ones with their passes split over threads, exact min/max/count reductions),
// then their children are numbered by a prefix count in node order, so the node array
// is the sequential builder's, bit for bit.
#include "yune_host.h"
#include "host/yh_threads.h"

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cstring>
#include <new>
#include <memory>
#include <thread>
#include <utility>
#include <vector>

namespace {

// More than leaf_max triangles with one centroid can never be separated: every split
// sends them all to the same child and the reference builder does not terminate. Trees
// deeper than this are taken for that case and refused.
constexpr int kMaxLevels = 1024;

struct V3 { float s[4]; };

struct TriInfo {
  float c[3];       // centroid (TriangleCPU::computeCentroid)
  float lo[3], hi[3];  // padded box (TriangleCPU::computeAABB)
};

// An allocator whose resize() leaves new elements uninitialised: node records are
// written in parallel right after they are made.
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U> struct rebind { using other = NoInitAlloc<U>; };
  NoInitAlloc() = default;
  template <class U> NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
  template <class U> void construct(U* p) noexcept { ::new (static_cast<void*>(p)) U; }
  template <class U, class... A> void construct(U* p, A&&... a) { ::new (static_cast<void*>(p)) U(std::forward<A>(a)...); }
};
using NodeVec = std::vector<yc_bvh_node, NoInitAlloc<yc_bvh_node>>;

struct Seg {
  int s, e;   // a node's primitives: perm[s, e)
};

inline float surface_area(const yc_aabb& b) {
  const float d0 = b.p_max.x - b.p_min.x;
  const float d1 = b.p_max.y - b.p_min.y;
  const float d2 = b.p_max.z - b.p_min.z;
  return 2 * (d0 * d1 + d0 * d2 + d1 * d2);
}

inline float& axis_ref(yc_float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
inline float axis_get(const yc_float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

void tri_info(const yc_triangle& t, TriInfo& ti) {
  // centroid = ((v1 + v2) + v3) / 3
  ti.c[0] = ((t.v1.x + t.v2.x) + t.v3.x) / 3.0f;
  ti.c[1] = ((t.v1.y + t.v2.y) + t.v3.y) / 3.0f;
  ti.c[2] = ((t.v1.z + t.v2.z) + t.v3.z) / 3.0f;
  const float* a = &t.v1.x;
  const float* b = &t.v2.x;
  const float* c = &t.v3.x;
  for (int i = 0; i < 3; ++i) {
    ti.lo[i] = std::min(a[i], std::min(b[i], c[i]));
    ti.hi[i] = std::max(a[i], std::max(b[i], c[i]));
    if (ti.hi[i] - ti.lo[i] == 0.0f) ti.hi[i] += 0.2f;   // TriangleCPU.cpp:63-67
  }
}

yc_bvh_node fresh_node(const yc_aabb& box) {
  yc_bvh_node g;
  std::memset(&g, 0, sizeof(g));
  g.aabb = box;
  for (int k = 0; k < 10; ++k) g.vert_list[k] = -1;
  g.child_idx = -2;
  g.vert_len = -1;
  return g;
}

}  // namespace

struct yh_bvh {
  NodeVec nodes;
  int depth = 0;
};

extern "C" int yh_triangle_aabb(const yc_triangle* t, yc_aabb* aabb, yc_float4* centroid) {
  if (!t) return YH_E_INVALID;
  TriInfo ti;
  tri_info(*t, ti);
  if (aabb) {
    aabb->p_min = yc_float4{ti.lo[0], ti.lo[1], ti.lo[2], 1.0f};
    aabb->p_max = yc_float4{ti.hi[0], ti.hi[1], ti.hi[2], 1.0f};
  }
  if (centroid) *centroid = yc_float4{ti.c[0], ti.c[1], ti.c[2], 1.0f};
  return YH_OK;
}

namespace {

// f(i) for i in [0, n) on up to `threads` host threads, taking blocks of `grain` indices
// from a shared counter
template <class F>
void pfor(size_t n, size_t grain, int threads, F f) {
  const int t = (int)std::min<size_t>((size_t)std::max(1, threads), (n + grain - 1) / std::max<size_t>(1, grain));
  if (t <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<size_t> next{0};
  auto work = [&] {
    for (;;) {
      const size_t b = next.fetch_add(grain);
      if (b >= n) break;
      const size_t e = std::min(n, b + grain);
      for (size_t i = b; i < e; ++i) f(i);
    }
  };
  std::vector<std::thread> pool;
  for (int k = 1; k < t; ++k) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
}

// [0, n) cut into `parts` contiguous chunks; f(chunk, begin, end) on a thread each
template <class F>
void chunks(size_t n, int parts, F f) {
  if (parts <= 1) {
    f(0, (size_t)0, n);
    return;
  }
  std::vector<std::thread> pool;
  for (int k = 1; k < parts; ++k) pool.emplace_back([&, k] { f(k, n * k / parts, n * (k + 1) / parts); });
  f(0, (size_t)0, n / parts);
  for (auto& th : pool) th.join();
}

struct Split {
  bool split = false;
  yc_aabb b1, b2;
  int n1 = 0;   // primitives of the first child, at the front of the node's range
};

// One node of BVH::createBVH (BVH.cpp:69-216) over perm[nd.s, nd.e): a leaf keeps its
// primitives; a node that splits reorders its range into the first child's primitives
// then the second's, each in their previous order (the reference's push_back order).
// Nodes of many primitives run their passes over `threads` chunks: box union and bin
// counts are exact in any order, and the membership lists are laid out by chunk offsets.
Split split_node(yc_bvh_node& g, Seg sg, int* perm, int* tmp, const std::vector<TriInfo>& info, int bins,
                 int leaf_max, int threads) {
  Split out;
  const yc_aabb pbox = g.aabb;
  int* prims = perm + sg.s;
  const int nprim = sg.e - sg.s;
  if (nprim == 0) return out;
  if (nprim <= leaf_max) {
    g.vert_len = nprim;
    g.child_idx = -1;
    for (int j = 0; j < nprim; ++j) g.vert_list[j] = prims[j];
    return out;
  }
  const float fmax_ = FLT_MAX;
  const int parts = nprim >= (1 << 16) ? std::min(threads, nprim >> 15) : 1;
  const int np = std::max(parts, 1);
  // per-thread scratch reused from node to node (no allocation per node)
  // (named through pointers below: inside a chunk running on another thread a
  // thread_local name would resolve to that thread's copy)
  thread_local std::vector<std::array<float, 6>> tl_pb;
  thread_local std::vector<float> tl_plane;
  thread_local std::vector<int> tl_ph;
  thread_local std::vector<size_t> tl_n1, tl_off1, tl_off2;
  tl_pb.resize(np);
  std::array<float, 6>* pb = tl_pb.data();
  // split axis: longest extent of the union of the primitives' boxes
  chunks((size_t)nprim, parts, [&](int c, size_t b, size_t e) {
    float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
    for (size_t i = b; i < e; ++i) {
      const int p = prims[i];
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(info[p].lo[k], lo[k]);
        hi[k] = std::max(info[p].hi[k], hi[k]);
      }
    }
    pb[c] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
  });
  float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
  for (int c = 0; c < np; ++c)
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(pb[c][k], lo[k]);
      hi[k] = std::max(pb[c][3 + k], hi[k]);
    }
  int axis = 0;
  float diff = -fmax_;
  for (int k = 0; k < 3; ++k) {
    const float d = hi[k] - lo[k];
    if (d > diff) { diff = d; axis = k; }
  }

  const float cost_isect = 1.0f;
  const float cost_trav = 1 / 8.0f;
  bool median = false;
  yc_aabb best1 = pbox, best2 = pbox;
  if (bins > 2 && nprim > 20) {
    float cost = surface_area(pbox) * cost_isect * (float)nprim;
    const float initial_cost = cost;
    float increment = axis_get(pbox.p_max, axis) - axis_get(pbox.p_min, axis);
    increment /= (float)bins;
    const int nsplit = bins - 1;
    tl_plane.resize(nsplit);
    float* plane = tl_plane.data();
    for (int b = 0; b < nsplit; ++b)
      plane[b] = axis_get(pbox.p_min, axis) + (float)(b + 1) * increment;
    // per primitive: first bin plane it lies below (membership is monotone in b)
    tl_ph.assign((size_t)np * (nsplit + 1), 0);
    int* ph = tl_ph.data();
    const float* bl = &pbox.p_min.x;
    const float* bh = &pbox.p_max.x;
    const float* pl = plane;
    chunks((size_t)nprim, parts, [&](int c, size_t b, size_t e) {
      int* hist = ph + (size_t)c * (nsplit + 1);
      for (size_t i = b; i < e; ++i) {
        const float* cc = info[prims[i]].c;
        bool inside = true;
        for (int k = 0; k < 3; ++k) {
          if (k == axis) { if (cc[k] < bl[k]) inside = false; }
          else if (cc[k] < bl[k] || cc[k] > bh[k]) inside = false;
        }
        int first = nsplit;
        if (inside) first = (int)(std::lower_bound(pl, pl + nsplit, cc[axis]) - pl);
        hist[first]++;
      }
    });
    int* hist = ph;
    for (int c = 1; c < np; ++c)
      for (int b = 0; b <= nsplit; ++b) hist[b] += ph[(size_t)c * (nsplit + 1) + b];
    const float sa_p = surface_area(pbox);
    int below = 0;
    for (int b = 0; b < nsplit; ++b) {
      below += hist[b];
      yc_aabb c1 = pbox, c2 = pbox;
      axis_ref(c1.p_max, axis) = plane[b];
      axis_ref(c2.p_min, axis) = plane[b];
      int n1, n2;
      if (surface_area(c1) == 0.0f) { n1 = 0; n2 = nprim; }
      else if (surface_area(c2) == 0.0f) { n1 = nprim; n2 = 0; }
      else { n1 = below; n2 = nprim - below; }
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
    const float center = (axis_get(pbox.p_min, axis) + axis_get(pbox.p_max, axis)) / 2.0f;
    best1 = pbox; best2 = pbox;
    axis_ref(best1.p_max, axis) = center;
    axis_ref(best2.p_min, axis) = center;
  }
  // populate the two children (BVH.cpp:175-216), keeping the primitives' order
  out.split = true;
  out.b1 = best1;
  out.b2 = best2;
  if (surface_area(best1) == 0.0f) {
    out.n1 = 0;
  } else if (surface_area(best2) == 0.0f) {
    out.n1 = nprim;
  } else {
    const float* l1 = &best1.p_min.x;
    const float* h1 = &best1.p_max.x;
    auto in1 = [&](int p) {
      const float* c = info[p].c;
      for (int k = 0; k < 3; ++k)
        if (c[k] < l1[k] || c[k] > h1[k]) return false;
      return true;
    };
    int* t = tmp + sg.s;
    tl_n1.assign(np, 0);
    size_t* n1 = tl_n1.data();
    chunks((size_t)nprim, parts, [&](int c, size_t b, size_t e) {
      size_t k1 = 0;
      for (size_t i = b; i < e; ++i) k1 += in1(prims[i]) ? 1 : 0;
      n1[c] = k1;
    });
    size_t total1 = 0;
    for (int c = 0; c < np; ++c) total1 += n1[c];
    tl_off1.assign(np, 0);
    tl_off2.assign(np, 0);
    size_t* off1 = tl_off1.data();
    size_t* off2 = tl_off2.data();
    size_t a1 = 0, a2 = total1;
    for (int c = 0; c < np; ++c) {
      const size_t b = (size_t)nprim * c / np, e = (size_t)nprim * (c + 1) / np;
      off1[c] = a1;
      off2[c] = a2;
      a1 += n1[c];
      a2 += (e - b) - n1[c];
    }
    chunks((size_t)nprim, parts, [&](int c, size_t b, size_t e) {
      size_t w1 = off1[c], w2 = off2[c];
      for (size_t i = b; i < e; ++i) {
        const int p = prims[i];
        if (in1(p)) t[w1++] = p;
        else t[w2++] = p;
      }
    });
    chunks((size_t)nprim, parts, [&](int, size_t b, size_t e) {
      std::memcpy(prims + b, t + b, (e - b) * sizeof(int));
    });
    out.n1 = (int)total1;
  }
  return out;
}

}  // namespace

extern "C" int yh_bvh_build(const yc_triangle* tris, int n_tri, int bins, int leaf_max, yh_bvh** out) {
  if (!out || n_tri < 0 || (n_tri > 0 && !tris) || leaf_max < 1 || leaf_max > 10 || bins < 0)
    return YH_E_INVALID;
  *out = nullptr;
  yh_bvh* bvh = new (std::nothrow) yh_bvh;
  if (!bvh) return YH_E_NOMEM;
  const int hw = yh::host_threads();
  try {
    std::vector<TriInfo> info(n_tri);
    const float fmax_ = FLT_MAX;
    yc_aabb root;
    root.p_min = yc_float4{fmax_, fmax_, fmax_, 1.0f};
    root.p_max = yc_float4{-fmax_, -fmax_, -fmax_, 1.0f};
    {
      const int parts = n_tri >= (1 << 16) ? std::min(hw, n_tri >> 15) : 1;
      std::vector<std::array<float, 6>> pb(std::max(parts, 1));
      chunks((size_t)n_tri, parts, [&](int c, size_t b, size_t e) {
        float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
        for (size_t i = b; i < e; ++i) {
          tri_info(tris[i], info[i]);
          for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], info[i].lo[k]);
            hi[k] = std::max(hi[k], info[i].hi[k]);
          }
        }
        pb[c] = {lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]};
      });
      float* lo = &root.p_min.x;
      float* hi = &root.p_max.x;
      for (const auto& q : pb)
        for (int k = 0; k < 3; ++k) {
          lo[k] = std::min(lo[k], q[k]);
          hi[k] = std::max(hi[k], q[3 + k]);
        }
    }

    NodeVec nodes;
    std::vector<Seg, NoInitAlloc<Seg>> seg;
    std::vector<int, NoInitAlloc<int>> node_depth;
    const size_t cap = n_tri > 0 ? (size_t)2 * n_tri + 8 : 8;
    nodes.reserve(cap);
    seg.reserve(cap);
    node_depth.reserve(cap);
    std::vector<int> perm(n_tri), tmp(n_tri);
    pfor((size_t)n_tri, 1 << 16, hw, [&](size_t i) { perm[i] = (int)i; });
    nodes.push_back(fresh_node(root));
    seg.push_back(Seg{0, n_tri});
    node_depth.push_back(0);

    // breadth first, one level at a time: the level's nodes decide independently (few
    // large nodes: each with every thread; many nodes: a node per thread), then their
    // children are appended in node order, which is the reference's numbering
    std::vector<size_t> level_start = {0};
    size_t a = 0, b = 1;
    while (a < b) {
      const size_t cnt = b - a;
      std::vector<Split> sp(cnt);
      if (cnt < (size_t)hw) {
        for (size_t i = 0; i < cnt; ++i)
          sp[i] = split_node(nodes[a + i], seg[a + i], perm.data(), tmp.data(), info, bins, leaf_max, hw);
      } else {
        pfor(cnt, std::max<size_t>(1, cnt / ((size_t)hw * 16)), hw, [&](size_t i) {
          sp[i] = split_node(nodes[a + i], seg[a + i], perm.data(), tmp.data(), info, bins, leaf_max, 1);
        });
      }
      // children slots: two per splitting node, in node order
      std::vector<int> slot(cnt);
      size_t splits = 0;
      for (size_t i = 0; i < cnt; ++i) {
        slot[i] = (int)splits;
        splits += sp[i].split ? 1 : 0;
      }
      if (splits > 0) {
        const int d = node_depth[a] + 1;   // every node of a level has the same depth
        if (d > kMaxLevels) {   // a split that moves nothing, forever (see yh_bvh_build)
          delete bvh;
          return YH_E_RANGE;
        }
        const size_t base = nodes.size();
        nodes.resize(base + 2 * splits);
        seg.resize(base + 2 * splits);
        node_depth.resize(base + 2 * splits);
        pfor(cnt, std::max<size_t>(1, cnt / ((size_t)hw * 16)), hw, [&](size_t i) {
          if (!sp[i].split) return;
          const size_t c = base + 2 * (size_t)slot[i];
          const Seg ps = seg[a + i];
          nodes[a + i].child_idx = (int)c;
          nodes[c] = fresh_node(sp[i].b1);
          nodes[c + 1] = fresh_node(sp[i].b2);
          seg[c] = Seg{ps.s, ps.s + sp[i].n1};
          seg[c + 1] = Seg{ps.s + sp[i].n1, ps.e};
          node_depth[c] = node_depth[c + 1] = d;
        });
      }
      a = b;
      b = nodes.size();
      level_start.push_back(a);
    }

    // bottom-up refit (BVH.cpp:218-247), deepest level first, a level's nodes in parallel
    for (size_t l = level_start.size() - 1; l-- > 0;) {
      const size_t la = level_start[l], lb = level_start[l + 1];
      pfor(lb - la, 256, hw, [&](size_t i) {
        yc_bvh_node& g = nodes[la + i];
        if (g.vert_len > 0) {
          float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
          for (int j = seg[la + i].s; j < seg[la + i].e; ++j)
            for (int k = 0, p = perm[j]; k < 3; ++k) {
              lo[k] = std::min(info[p].lo[k], lo[k]);
              hi[k] = std::max(info[p].hi[k], hi[k]);
            }
          g.aabb.p_min = yc_float4{lo[0], lo[1], lo[2], 1.0f};
          g.aabb.p_max = yc_float4{hi[0], hi[1], hi[2], 1.0f};
        } else if (g.child_idx > 0) {
          const yc_aabb& ca = nodes[g.child_idx].aabb;
          const yc_aabb& cb = nodes[g.child_idx + 1].aabb;
          yc_aabb u = ca;
          u.p_min.x = std::min(cb.p_min.x, ca.p_min.x);
          u.p_min.y = std::min(cb.p_min.y, ca.p_min.y);
          u.p_min.z = std::min(cb.p_min.z, ca.p_min.z);
          u.p_max.x = std::max(cb.p_max.x, ca.p_max.x);
          u.p_max.y = std::max(cb.p_max.y, ca.p_max.y);
          u.p_max.z = std::max(cb.p_max.z, ca.p_max.z);
          g.aabb = u;
        }
      });
    }
    int depth = 0;
    for (size_t i = 0; i < node_depth.size(); ++i) depth = std::max(depth, node_depth[i]);
    bvh->nodes = std::move(nodes);
    bvh->depth = depth;
  } catch (const std::bad_alloc&) {
    delete bvh;
    return YH_E_NOMEM;
  }
  *out = bvh;
  return YH_OK;
}

extern "C" int yh_bvh_node_count(const yh_bvh* b) { return b ? (int)b->nodes.size() : YH_E_INVALID; }
extern "C" int yh_bvh_depth(const yh_bvh* b) { return b ? b->depth : YH_E_INVALID; }
extern "C" int yh_bvh_copy_nodes(const yh_bvh* b, yc_bvh_node* out, int capacity) {
  if (!b || !out) return YH_E_INVALID;
  if (capacity < (int)b->nodes.size()) return YH_E_RANGE;
  std::memcpy(out, b->nodes.data(), b->nodes.size() * sizeof(yc_bvh_node));
  return YH_OK;
}
extern "C" void yh_bvh_free(yh_bvh* b) { delete b; }

// The bottom-up pass of BVH::createBVH (BVH::resizeBvh, src/BVH.cpp:218-247) on an
// existing node array with new triangle positions: leaf boxes are computed in parallel
// (each from its own triangles), then every interior box, in reverse node order, from
// its two children, which come after it in the array.
extern "C" int yh_bvh_refit(const yc_triangle* tris, int n_tri, yc_bvh_node* nodes, int n_node) {
  if (n_tri < 0 || n_node < 0 || (n_tri > 0 && !tris) || (n_node > 0 && !nodes)) return YH_E_INVALID;
  for (int j = 0; j < n_node; ++j) {
    const yc_bvh_node& g = nodes[j];
    if (g.vert_len > 0) {
      if (g.vert_len > 10) return YH_E_RANGE;
      for (int k = 0; k < g.vert_len; ++k)
        if (g.vert_list[k] < 0 || g.vert_list[k] >= n_tri) return YH_E_RANGE;
    } else if (g.child_idx > 0) {
      if (g.child_idx <= j || g.child_idx >= n_node - 1) return YH_E_RANGE;
    }
  }
  const float fmax_ = FLT_MAX;
  pfor((size_t)n_node, 4096, yh::host_threads(), [&](size_t j) {
    yc_bvh_node& g = nodes[j];
    if (g.vert_len <= 0) return;
    float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
    for (int k = 0; k < g.vert_len; ++k) {
      TriInfo ti;
      tri_info(tris[g.vert_list[k]], ti);
      for (int a = 0; a < 3; ++a) {
        lo[a] = std::min(ti.lo[a], lo[a]);
        hi[a] = std::max(ti.hi[a], hi[a]);
      }
    }
    g.aabb.p_min = yc_float4{lo[0], lo[1], lo[2], 1.0f};
    g.aabb.p_max = yc_float4{hi[0], hi[1], hi[2], 1.0f};
  });
  for (int j = n_node - 1; j >= 0; --j) {
    yc_bvh_node& g = nodes[j];
    if (g.vert_len > 0 || g.child_idx <= 0) continue;
    const yc_aabb& ca = nodes[g.child_idx].aabb;
    const yc_aabb& cb = nodes[g.child_idx + 1].aabb;
    yc_aabb u = ca;
    u.p_min.x = std::min(cb.p_min.x, ca.p_min.x);
    u.p_min.y = std::min(cb.p_min.y, ca.p_min.y);
    u.p_min.z = std::min(cb.p_min.z, ca.p_min.z);
    u.p_max.x = std::max(cb.p_max.x, ca.p_max.x);
    u.p_max.y = std::max(cb.p_max.y, ca.p_max.y);
    u.p_max.z = std::max(cb.p_max.z, ca.p_max.z);
    g.aabb = u;
  }
  return YH_OK;
}
