// yh_bvh.cpp -- the breadth-first binned BVH of Yune's BVH::createBVH, restated.
//
// The node array this produces is the one src/BVH.cpp:56-173 produces for the same
// triangles, bins and leaf size (tests/test_host_bvh.py compares the two node by
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
// monotone bin planes and a prefix sum (O(n log bins)), and moves vectors instead of
// copying them.
#include "yune_host.h"

#include <algorithm>
#include <cfloat>
#include <cstring>
#include <new>
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

struct Node {
  yc_bvh_node g;
  std::vector<int> prims;
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
  std::vector<yc_bvh_node> nodes;
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

extern "C" int yh_bvh_build(const yc_triangle* tris, int n_tri, int bins, int leaf_max, yh_bvh** out) {
  if (!out || n_tri < 0 || (n_tri > 0 && !tris) || leaf_max < 1 || leaf_max > 10 || bins < 0)
    return YH_E_INVALID;
  *out = nullptr;
  yh_bvh* bvh = new (std::nothrow) yh_bvh;
  if (!bvh) return YH_E_NOMEM;
  try {
    std::vector<TriInfo> info(n_tri);
    const float fmax_ = FLT_MAX;
    yc_aabb root;
    root.p_min = yc_float4{fmax_, fmax_, fmax_, 1.0f};
    root.p_max = yc_float4{-fmax_, -fmax_, -fmax_, 1.0f};
    for (int i = 0; i < n_tri; ++i) {
      tri_info(tris[i], info[i]);
      float* lo = &root.p_min.x;
      float* hi = &root.p_max.x;
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], info[i].lo[k]);
        hi[k] = std::max(hi[k], info[i].hi[k]);
      }
    }

    const float cost_isect = 1.0f;
    const float cost_trav = 1 / 8.0f;
    std::vector<Node> nodes;
    std::vector<int> node_depth;
    nodes.reserve(n_tri > 0 ? (size_t)(2 * n_tri / std::max(1, leaf_max) + 8) : 8);
    nodes.push_back(Node{fresh_node(root), {}});
    node_depth.push_back(0);
    nodes[0].prims.resize(n_tri);
    for (int i = 0; i < n_tri; ++i) nodes[0].prims[i] = i;

    std::vector<int> hist;
    for (size_t ni = 0; ni < nodes.size(); ++ni) {
      std::vector<int> prims = std::move(nodes[ni].prims);
      const yc_aabb pbox = nodes[ni].g.aabb;
      const int nprim = (int)prims.size();
      if (nprim == 0) continue;
      if (nprim <= leaf_max) {
        nodes[ni].g.vert_len = nprim;
        nodes[ni].g.child_idx = -1;
        for (int j = 0; j < nprim; ++j) nodes[ni].g.vert_list[j] = prims[j];
        nodes[ni].prims = std::move(prims);   // kept for the refit
        continue;
      }
      // split axis: longest extent of the union of the primitives' boxes
      float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
      for (int p : prims)
        for (int k = 0; k < 3; ++k) {
          lo[k] = std::min(info[p].lo[k], lo[k]);
          hi[k] = std::max(info[p].hi[k], hi[k]);
        }
      int axis = 0;
      float diff = -fmax_;
      for (int k = 0; k < 3; ++k) {
        const float d = hi[k] - lo[k];
        if (d > diff) { diff = d; axis = k; }
      }

      bool median = false;
      bool have_split = false;
      yc_aabb best1 = pbox, best2 = pbox;
      if (bins > 2 && nprim > 20) {
        float cost = surface_area(pbox) * cost_isect * (float)nprim;
        const float initial_cost = cost;
        float increment = axis_get(pbox.p_max, axis) - axis_get(pbox.p_min, axis);
        increment /= (float)bins;
        const int nsplit = bins - 1;
        std::vector<float> plane(nsplit);
        for (int b = 0; b < nsplit; ++b)
          plane[b] = axis_get(pbox.p_min, axis) + (float)(b + 1) * increment;
        // per primitive: first bin plane it lies below (membership is monotone in b)
        hist.assign(nsplit + 1, 0);
        const float* bl = &pbox.p_min.x;
        const float* bh = &pbox.p_max.x;
        for (int p : prims) {
          const float* c = info[p].c;
          bool inside = true;
          for (int k = 0; k < 3; ++k) {
            if (k == axis) { if (c[k] < bl[k]) inside = false; }
            else if (c[k] < bl[k] || c[k] > bh[k]) inside = false;
          }
          int first = nsplit;
          if (inside) first = (int)(std::lower_bound(plane.begin(), plane.end(), c[axis]) - plane.begin());
          hist[first]++;
        }
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
            best1 = c1; best2 = c2; have_split = true;
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
        have_split = true;
      }
      (void)have_split;
      // populate the two children (BVH.cpp:175-216)
      std::vector<int> p1, p2;
      if (surface_area(best1) == 0.0f) p2 = prims;
      else if (surface_area(best2) == 0.0f) p1 = prims;
      else {
        const float* l1 = &best1.p_min.x;
        const float* h1 = &best1.p_max.x;
        for (int p : prims) {
          const float* c = info[p].c;
          bool in1 = true;
          for (int k = 0; k < 3; ++k)
            if (c[k] < l1[k] || c[k] > h1[k]) { in1 = false; break; }
          (in1 ? p1 : p2).push_back(p);
        }
      }
      const int cidx = (int)nodes.size();
      nodes[ni].g.child_idx = cidx;
      const int d = node_depth[ni] + 1;
      if (d > kMaxLevels) {   // a split that moves nothing, forever (see yh_bvh_build)
        delete bvh;
        return YH_E_RANGE;
      }
      nodes.push_back(Node{fresh_node(best1), std::move(p1)});
      nodes.push_back(Node{fresh_node(best2), std::move(p2)});
      node_depth.push_back(d);
      node_depth.push_back(d);
    }

    // bottom-up refit (BVH.cpp:218-247)
    for (int j = (int)nodes.size() - 1; j >= 0; --j) {
      yc_bvh_node& g = nodes[j].g;
      if (g.vert_len > 0) {
        float lo[3] = {fmax_, fmax_, fmax_}, hi[3] = {-fmax_, -fmax_, -fmax_};
        for (int p : nodes[j].prims)
          for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(info[p].lo[k], lo[k]);
            hi[k] = std::max(info[p].hi[k], hi[k]);
          }
        g.aabb.p_min = yc_float4{lo[0], lo[1], lo[2], 1.0f};
        g.aabb.p_max = yc_float4{hi[0], hi[1], hi[2], 1.0f};
      } else if (g.child_idx > 0) {
        const yc_aabb& a = nodes[g.child_idx].g.aabb;
        const yc_aabb& b = nodes[g.child_idx + 1].g.aabb;
        yc_aabb u = a;
        u.p_min.x = std::min(b.p_min.x, a.p_min.x);
        u.p_min.y = std::min(b.p_min.y, a.p_min.y);
        u.p_min.z = std::min(b.p_min.z, a.p_min.z);
        u.p_max.x = std::max(b.p_max.x, a.p_max.x);
        u.p_max.y = std::max(b.p_max.y, a.p_max.y);
        u.p_max.z = std::max(b.p_max.z, a.p_max.z);
        g.aabb = u;
      }
    }
    bvh->nodes.resize(nodes.size());
    int depth = 0;
    for (size_t i = 0; i < nodes.size(); ++i) {
      bvh->nodes[i] = nodes[i].g;
      depth = std::max(depth, node_depth[i]);
    }
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
