// repack.cpp -- turns the caller's TriangleGPU / BVHNodeGPU arrays into the device
// layout described in yc_scene.h (host side, once per upload).
//
// The reference walks BVHNodeGPU directly: a node is processed as a leaf when
// child_idx == -1 and vert_len > 0, otherwise its children child_idx and child_idx + 1
// are box-tested, each only when vert_len > 0 || child_idx > 0 (traverseBVH,
// kernels/legacy/udpt.cl:298-321). The repack keeps exactly that structure: each
// reference interior node becomes one 64-byte node carrying its children's boxes, each
// reference leaf becomes a contiguous run of its vert_list triangles (in vert_list
// order) in the 48-byte stream, and a child the reference never queues becomes
// LINK_NONE.
// Equal-t ties: the reference accepts a triangle only when its t is strictly smaller
// than the current length, so among triangles at the same t the first one it visits
// wins. Its node array is built breadth first (src/BVH.cpp:65-165) and its queue is
// processed in index order, so that first one lies in the leaf with the smallest node
// index, at the smallest vert_list slot. Each stream slot carries that rank
// (node index * 16 + slot) as a tie-break key, so the depth-first walk picks the same
// triangle. With no BVH (bvh_size == 0) the reference tests every triangle in index
// order (udpt.cl:280-284); that case becomes a chain of nodes with unbounded boxes whose
// leaves hold the triangles in index order.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../ym_math.h"
#include "yc_repack.h"
#include "yc_sah.h"
#include "host/yh_threads.h"

namespace yc {

namespace {

struct Builder {
  const yc_triangle* tris;
  int n_tri;
  const yc_bvh_node* nodes;
  int n_node;
  F4Vec out_nodes;
  F4Vec out_tris;
  int depth = 0;

  // order_base: visiting rank of the leaf in the reference traversal; the triangle's
  // tie-break key is order_base + its slot.
  int emit_leaf(const int* list, int count, int order_base) {
    const int first = (int)(out_tris.size() / 3);
    for (int k = 0; k < count; ++k) {
      const yc_triangle& t = tris[list[k]];
      float4 a, b, c;
      a.x = t.v1.x; a.y = t.v1.y; a.z = t.v1.z;
      int id = list[k];
      std::memcpy(&a.w, &id, 4);
      const int key = order_base + k;
      b.x = t.v2.x - t.v1.x; b.y = t.v2.y - t.v1.y; b.z = t.v2.z - t.v1.z;
      std::memcpy(&b.w, &key, 4);
      c.x = t.v3.x - t.v1.x; c.y = t.v3.y - t.v1.y; c.z = t.v3.z - t.v1.z; c.w = 0.0f;
      out_tris.push_back(a);
      out_tris.push_back(b);
      out_tris.push_back(c);
    }
    return ~((first << 4) | count);
  }
  // the same records as emit_leaf, written at stream slot `first` of a pre-sized stream
  int fill_leaf(const int* list, int count, int order_base, int first) {
    for (int k = 0; k < count; ++k) {
      const yc_triangle& t = tris[list[k]];
      float4 a, b, c;
      a.x = t.v1.x; a.y = t.v1.y; a.z = t.v1.z;
      int id = list[k];
      std::memcpy(&a.w, &id, 4);
      const int key = order_base + k;
      b.x = t.v2.x - t.v1.x; b.y = t.v2.y - t.v1.y; b.z = t.v2.z - t.v1.z;
      std::memcpy(&b.w, &key, 4);
      c.x = t.v3.x - t.v1.x; c.y = t.v3.y - t.v1.y; c.z = t.v3.z - t.v1.z; c.w = 0.0f;
      float4* o = &out_tris[3 * ((size_t)first + k)];
      o[0] = a;
      o[1] = b;
      o[2] = c;
    }
    return ~((first << 4) | count);
  }
};

// f(i) for i in [0, n) on the host's cores, in contiguous chunks (f must write only
// its own outputs)
template <class F>
void parallel_for(size_t n, F f) {
  const size_t hw = (size_t)yh::host_threads();
  const size_t t = std::min(hw, std::max<size_t>(1, n / 4096));
  if (t <= 1) {
    for (size_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> pool;
  for (size_t k = 0; k < t; ++k)
    pool.emplace_back([&, k] {
      for (size_t i = n * k / t; i < n * (k + 1) / t; ++i) f(i);
    });
  for (auto& th : pool) th.join();
}

bool is_leaf(const yc_bvh_node& n) { return (float)n.child_idx == -1.0f && n.vert_len > 0; }

// One two-child node of yc_scene.h: per axis the pair (child 0, child 1) of lower bounds,
// then the pair of upper bounds, so that each 64-bit half of a float4 is the pair one
// packed f32x2 operation takes; then the two links.
void write_node2(float4* o, const float lo0[3], const float hi0[3], const float lo1[3], const float hi1[3], int l0,
                 int l1) {
  for (int k = 0; k < 3; ++k) o[k] = float4{lo0[k], lo1[k], hi0[k], hi1[k]};
  float4 l;
  std::memcpy(&l.x, &l0, 4);
  std::memcpy(&l.y, &l1, 4);
  l.z = l.w = 0.0f;
  o[3] = l;
}
bool is_queued(const yc_bvh_node& n) { return n.vert_len > 0 || n.child_idx > 0; }

// ---- SAH hierarchy over the reference leaves ----
// Each reference leaf keeps its triangles, their order and its tie-break rank; only the
// interior nodes above the leaves are rebuilt, by a binned surface-area-heuristic split
// of the leaves' box centroids (up to 256 bins per axis; each side of a split costs its
// box area times its triangles). A node's box is the union of the
// leaf boxes below it, so it contains every box the reference tree places below it and
// a ray that reaches a leaf in the reference passes every box on the way down here too.
// The arithmetic (bins, areas, costs, min / max order) is yc_sah.h's, and a split keeps
// the leaves' order on each side (a stable partition), so the device repack
// (repack_dev.cu) builds the same hierarchy bit for bit.
struct LeafItem {
  float lo[3], hi[3];
  float c[3];
  int w;   // the leaf's triangles (its cost in the SAH; integer sums are exact in any order)
  int link;
};

// A child reference of the in-memory binary tree: a leaf (node < 0, link = its leaf
// link) or an interior node (index into SahBuilder::bins), with its box.
struct BinRef {
  int node;
  int link;
  int count;   // leaves below (1 for a leaf)
  float lo[3], hi[3];
};
struct BinNode {
  BinRef c[2];
};

// Subtrees of more than kParallelItems leaves are built on their own thread while threads
// are free: a subtree's splits depend only on its own items, and the emitted layout only
// on the tree's shape, so the result is the sequential build's. Interior nodes take their
// slots in `bins` (exactly items - 1 of them) from an atomic counter.
constexpr int kParallelItems = 1 << 15;

struct SahBuilder {
  std::vector<LeafItem>& items;
  std::vector<BinNode> bins;
  std::atomic<int> max_depth{0};
  std::atomic<int> next_node{0};
  std::atomic<int> threads{1};
  int max_threads = yh::host_threads();

  SahBuilder(std::vector<LeafItem>& it) : items(it), bins(it.size() > 1 ? it.size() - 1 : 0) {}

  static float area(const float lo[3], const float hi[3]) { return sah_area(lo[0], lo[1], lo[2], hi[0], hi[1], hi[2]); }

  // stable partition of items [b, e): the leaves with left(item) first, each side in its
  // old order; returns the first of the right side (a scratch vector per thread holds them)
  template <class P>
  int stable_split(int b, int e, P left) {
    thread_local std::vector<LeafItem> right;
    right.clear();
    int w = b;
    for (int i = b; i < e; ++i) {
      if (left(items[i])) items[w++] = items[i];
      else right.push_back(items[i]);
    }
    std::copy(right.begin(), right.end(), items.begin() + w);
    return w;
  }

  static constexpr int NB = SAH_NB;

  // box and centroid box of items [b, e), and the per-axis bins of their centroids:
  // min, max and counts, which are exact in any order, so the chunks of a large range
  // are reduced on their own threads and merged
  struct RangeStats {
    float lo[3], hi[3], clo[3], chi[3];
    int cnt[3][NB];
    int wsum[3][NB];
    float blo[3][NB][3], bhi[3][NB][3];
  };
  static void init_box(float lo[3], float hi[3]) {
    for (int k = 0; k < 3; ++k) { lo[k] = INFINITY; hi[k] = -INFINITY; }
  }
  void bounds(int b, int e, RangeStats& st) const {
    init_box(st.lo, st.hi);
    init_box(st.clo, st.chi);
    for (int i = b; i < e; ++i)
      for (int k = 0; k < 3; ++k) {
        st.lo[k] = sah_min(st.lo[k], items[i].lo[k]);
        st.hi[k] = sah_max(st.hi[k], items[i].hi[k]);
        st.clo[k] = sah_min(st.clo[k], items[i].c[k]);
        st.chi[k] = sah_max(st.chi[k], items[i].c[k]);
      }
  }
  // bins of [b, e) on the axes with a positive centroid extent, against the node's
  // centroid box (clo, ext)
  // bins for a range of n leaves: 256 for large ranges, fewer (at least 8 per leaf) for
  // small ones, where the binning of every node would otherwise cost more than its items
  static int bins_for(int n) { return sah_bins_for(n); }
  void binning(int b, int e, const float clo[3], const float ext[3], RangeStats& st, int nb) const {
    for (int k = 0; k < 3; ++k)
      for (int q = 0; q < nb; ++q) {
        st.cnt[k][q] = 0;
        st.wsum[k][q] = 0;
        init_box(st.blo[k][q], st.bhi[k][q]);
      }
    float scale[3];
    for (int k = 0; k < 3; ++k) scale[k] = ext[k] > 0.0f ? nb / ext[k] : 0.0f;
    for (int i = b; i < e; ++i)
      for (int k = 0; k < 3; ++k) {
        if (!(ext[k] > 0.0f)) continue;
        const int q = sah_bin(items[i].c[k], clo[k], scale[k], nb);
        st.cnt[k][q]++;
        st.wsum[k][q] += items[i].w;
        for (int a = 0; a < 3; ++a) {
          st.blo[k][q][a] = sah_min(st.blo[k][q][a], items[i].lo[a]);
          st.bhi[k][q][a] = sah_max(st.bhi[k][q][a], items[i].hi[a]);
        }
      }
  }
  // f(chunk b, chunk e, stats) over [b, e) in chunks on threads, merged into st
  template <class F>
  void chunked(int b, int e, RangeStats& st, bool boxes, F f) {
    const int n = e - b;
    int t = (int)std::min<long>(max_threads, n / (1 << 16));
    if (t > 1 && threads.load() < max_threads) {
      std::vector<RangeStats> part(t);
      std::vector<std::thread> pool;
      for (int k = 1; k < t; ++k)
        pool.emplace_back([&, k] { f(b + (int)((long)n * k / t), b + (int)((long)n * (k + 1) / t), part[k]); });
      f(b, b + n / t, part[0]);
      for (auto& th : pool) th.join();
      st = part[0];
      for (int c = 1; c < t; ++c) {
        const RangeStats& o = part[c];
        if (boxes) {
          for (int k = 0; k < 3; ++k) {
            st.lo[k] = sah_min(st.lo[k], o.lo[k]); st.hi[k] = sah_max(st.hi[k], o.hi[k]);
            st.clo[k] = sah_min(st.clo[k], o.clo[k]); st.chi[k] = sah_max(st.chi[k], o.chi[k]);
          }
        } else {
          for (int k = 0; k < 3; ++k)
            for (int q = 0; q < NB; ++q) {
              st.cnt[k][q] += o.cnt[k][q];
              st.wsum[k][q] += o.wsum[k][q];
              for (int a = 0; a < 3; ++a) {
                st.blo[k][q][a] = sah_min(st.blo[k][q][a], o.blo[k][q][a]);
                st.bhi[k][q][a] = sah_max(st.bhi[k][q][a], o.bhi[k][q][a]);
              }
            }
        }
      }
    } else {
      f(b, e, st);
    }
  }

  // the subtree over items [b, e)
  BinRef build(int b, int e, int depth) {
    BinRef r;
    RangeStats st;
    chunked(b, e, st, true, [&](int cb, int ce, RangeStats& o) { bounds(cb, ce, o); });
    float clo[3], chi[3];
    for (int k = 0; k < 3; ++k) {
      r.lo[k] = st.lo[k];
      r.hi[k] = st.hi[k];
      clo[k] = st.clo[k];
      chi[k] = st.chi[k];
    }
    for (int m = max_depth.load(); depth > m && !max_depth.compare_exchange_weak(m, depth);) {}
    if (e - b == 1) {
      r.node = -1;
      r.link = items[b].link;
      r.count = 1;
      return r;
    }
    // binned SAH
    float ext3[3];
    for (int k = 0; k < 3; ++k) ext3[k] = chi[k] - clo[k];
    const int nb = bins_for(e - b);
    chunked(b, e, st, false, [&](int cb, int ce, RangeStats& o) { binning(cb, ce, clo, ext3, o, nb); });
    int best_axis = -1, best_split = -1;
    float best_cost = INFINITY;
    for (int k = 0; k < 3; ++k) {
      const float ext = ext3[k];
      if (!(ext > 0.0f)) continue;
      const int* cnt = st.cnt[k];
      const float (*blo)[3] = st.blo[k];
      const float (*bhi)[3] = st.bhi[k];
      float rlo[NB][3], rhi[NB][3];
      int rcnt[NB];
      int rw[NB];
      float alo[3] = {INFINITY, INFINITY, INFINITY}, ahi[3] = {-INFINITY, -INFINITY, -INFINITY};
      int ac = 0;
      int aw = 0;
      for (int q = nb - 1; q >= 0; --q) {
        for (int a = 0; a < 3; ++a) { alo[a] = sah_min(alo[a], blo[q][a]); ahi[a] = sah_max(ahi[a], bhi[q][a]); }
        ac += cnt[q];
        aw += st.wsum[k][q];
        for (int a = 0; a < 3; ++a) { rlo[q][a] = alo[a]; rhi[q][a] = ahi[a]; }
        rcnt[q] = ac;
        rw[q] = aw;
      }
      float llo[3] = {INFINITY, INFINITY, INFINITY}, lhi[3] = {-INFINITY, -INFINITY, -INFINITY};
      int lc = 0;
      int lw = 0;
      for (int q = 0; q < nb - 1; ++q) {
        for (int a = 0; a < 3; ++a) { llo[a] = sah_min(llo[a], blo[q][a]); lhi[a] = sah_max(lhi[a], bhi[q][a]); }
        lc += cnt[q];
        lw += st.wsum[k][q];
        const int rc = rcnt[q + 1];
        if (lc == 0 || rc == 0) continue;
        const float cost = area(llo, lhi) * (float)lw + area(rlo[q + 1], rhi[q + 1]) * (float)rw[q + 1];
        if (cost < best_cost) { best_cost = cost; best_axis = k; best_split = q; }
      }
    }
    int mid;
    if (best_axis < 0) {
      mid = (b + e) / 2;   // coincident centroids: split the list in half
    } else {
      const float ext = chi[best_axis] - clo[best_axis];
      const float scale = nb / ext;
      auto left = [&](const LeafItem& it) { return sah_bin(it.c[best_axis], clo[best_axis], scale, nb) <= best_split; };
      mid = stable_split(b, e, left);
      if (mid == b || mid == e) mid = (b + e) / 2;
    }
    const int node = next_node.fetch_add(1);
    BinRef c0, c1;
    if (e - b > kParallelItems && threads.load() < max_threads) {
      threads.fetch_add(1);
      std::thread left([&] { c0 = build(b, mid, depth + 1); });
      c1 = build(mid, e, depth + 1);
      left.join();
      threads.fetch_sub(1);
    } else {
      c0 = build(b, mid, depth + 1);
      c1 = build(mid, e, depth + 1);
    }
    bins[node].c[0] = c0;
    bins[node].c[1] = c1;
    r.node = node;
    r.count = e - b;
    r.link = 0;
    return r;
  }

  // two-child layout of yc_scene.h, nodes in pre-order; returns the link of r. A
  // subtree of n leaves holds n - 1 nodes, so each child's first node is known and large
  // subtrees are written on threads of their own (the same layout as a sequential walk).
  int emit_binary(const BinRef& r, F4Vec& out) {
    if (r.node < 0) return r.link;
    const size_t base = out.size() / 4;
    out.resize(out.size() + 4 * (size_t)(r.count - 1));
    return emit_binary_at(r, out.data(), (int)base);
  }
  int emit_binary_at(const BinRef& r, float4* out, int node) {
    if (r.node < 0) return r.link;
    const BinNode& bn = bins[r.node];
    const BinRef& a = bn.c[0];
    const BinRef& b = bn.c[1];
    const int left_nodes = a.node < 0 ? 0 : a.count - 1;
    int c0, c1;
    if (r.count > kParallelItems && threads.load() < max_threads) {
      threads.fetch_add(1);
      std::thread left([&] { c0 = emit_binary_at(a, out, node + 1); });
      c1 = emit_binary_at(b, out, node + 1 + left_nodes);
      left.join();
      threads.fetch_sub(1);
    } else {
      c0 = emit_binary_at(a, out, node + 1);
      c1 = emit_binary_at(b, out, node + 1 + left_nodes);
    }
    write_node2(&out[4 * (size_t)node], a.lo, a.hi, b.lo, b.hi, c0, c1);
    return node;
  }

  // four-child layout (yc_scene.h, wide nodes): the children of a binary node are
  // replaced, largest surface area first, by their own children until four remain.
  // depth_out: wide levels below r.
  int emit_wide(const BinRef& r, F4Vec& out, int& depth_out) const {
    depth_out = 0;
    if (r.node < 0) return r.link;
    BinRef kids[4];
    int nk = 2;
    kids[0] = bins[r.node].c[0];
    kids[1] = bins[r.node].c[1];
    while (nk < 4) {
      int pick = -1;
      float best = -1.0f;
      for (int i = 0; i < nk; ++i)
        if (kids[i].node >= 0 && area(kids[i].lo, kids[i].hi) > best) { best = area(kids[i].lo, kids[i].hi); pick = i; }
      if (pick < 0) break;
      const BinNode& bn = bins[kids[pick].node];
      kids[pick] = bn.c[0];
      kids[nk++] = bn.c[1];
    }
    const int node = (int)(out.size() / 8);
    out.resize(out.size() + 8);
    int links[4] = {LINK_NONE, LINK_NONE, LINK_NONE, LINK_NONE};
    for (int i = 0; i < nk; ++i) {
      int d = 0;
      links[i] = emit_wide(kids[i], out, d);
      depth_out = std::max(depth_out, d + 1);
    }
    float4* o = &out[8 * (size_t)node];
    float v[6][4];
    for (int i = 0; i < 4; ++i)
      for (int k = 0; k < 3; ++k) {
        v[2 * k][i] = i < nk ? kids[i].lo[k] : 0.0f;
        v[2 * k + 1][i] = i < nk ? kids[i].hi[k] : 0.0f;
      }
    for (int f = 0; f < 6; ++f) o[f] = float4{v[f][0], v[f][1], v[f][2], v[f][3]};
    float4 l;
    std::memcpy(&l.x, &links[0], 4);
    std::memcpy(&l.y, &links[1], 4);
    std::memcpy(&l.z, &links[2], 4);
    std::memcpy(&l.w, &links[3], 4);
    o[6] = l;
    o[7] = float4{0.0f, 0.0f, 0.0f, 0.0f};
    return node;
  }
};

// the reference node array's checks (in parallel; the message names the first bad node)
int check_nodes(const yc_bvh_node* nodes, int n_node, int n_tri, std::string& err) {
  auto node_error = [&](int i, std::string* msg) {
    const yc_bvh_node& n = nodes[i];
    if (n.vert_len > 10) {
      if (msg) *msg = "BVH node " + std::to_string(i) + " has vert_len > 10";
      return true;
    }
    if (is_leaf(n)) {
      for (int k = 0; k < n.vert_len; ++k)
        if (n.vert_list[k] < 0 || n.vert_list[k] >= n_tri) {
          if (msg) *msg = "BVH leaf " + std::to_string(i) + " references triangle " + std::to_string(n.vert_list[k]);
          return true;
        }
    } else if (is_queued(n) || i == 0) {
      if (n.child_idx <= 0 || n.child_idx + 1 >= n_node) {
        if (msg) *msg = "BVH node " + std::to_string(i) + " has child_idx " + std::to_string(n.child_idx) + " out of range";
        return true;
      }
    }
    return false;
  };
  std::atomic<int> first_bad{n_node};
  parallel_for((size_t)n_node, [&](size_t i) {
    if (node_error((int)i, nullptr))
      for (int m = first_bad.load(); (int)i < m && !first_bad.compare_exchange_weak(m, (int)i);) {}
  });
  if (first_bad.load() < n_node) {
    node_error(first_bad.load(), &err);
    return -1;
  }
  return 0;
}

// the leaves the reference traversal can reach, in node-index order, the first stream
// slot of each (the slots their triangles take one leaf after another) and the slot total
void reachable_leaves(const yc_bvh_node* nodes, int n_node, std::vector<int>& leaf_node, std::vector<int>& leaf_first,
                      size_t& slots) {
  std::vector<char> reach(n_node, 0);
  reach[0] = 1;
  slots = 0;
  for (int i = 0; i < n_node; ++i) {
    if (!reach[i]) continue;
    const yc_bvh_node& n = nodes[i];
    if (is_leaf(n)) {
      leaf_node.push_back(i);
      leaf_first.push_back((int)slots);
      slots += (size_t)n.vert_len;
    } else if (is_queued(n) || i == 0) {
      for (int c = 0; c < 2; ++c)
        if (is_queued(nodes[n.child_idx + c])) reach[n.child_idx + c] = 1;
    }
  }
}

}  // namespace

int check_materials(const yc_triangle* tris, int n_tri, int n_mat, std::string& err) {
  std::atomic<int> first_bad{n_tri};
  parallel_for((size_t)n_tri, [&](size_t i) {
    if (tris[i].matID < 0 || tris[i].matID >= n_mat)
      for (int m = first_bad.load(); (int)i < m && !first_bad.compare_exchange_weak(m, (int)i);) {}
  });
  if (first_bad.load() < n_tri) {
    err = "triangle " + std::to_string(first_bad.load()) + " has matID out of range";
    return -1;
  }
  return 0;
}

int plan_device_repack(const yc_bvh_node* nodes, int n_node, int n_tri, DevRepackPlan& plan, std::string& err) {
  plan = DevRepackPlan();
  if (n_tri == 0 || n_node == 0) return 0;
  if (check_nodes(nodes, n_node, n_tri, err)) return -1;
  if (n_node >= (1 << 27)) { err = "BVH too large for the 27-bit tie-break rank"; return -1; }
  const yc_bvh_node& root = nodes[0];
  if (is_leaf(root)) return 0;
  reachable_leaves(nodes, n_node, plan.leaf_node, plan.leaf_first, plan.slots);
  if (plan.leaf_node.size() < 2) return 0;
  if (plan.slots >= (size_t)(1 << 27)) { err = "scene too large for the 27-bit stream index"; return -1; }
  plan.root_lo = float4{root.aabb.p_min.x, root.aabb.p_min.y, root.aabb.p_min.z, 0.0f};
  plan.root_hi = float4{root.aabb.p_max.x, root.aabb.p_max.y, root.aabb.p_max.z, 0.0f};
  return 1;
}

int repack_scene(const yc_triangle* tris, int n_tri, const yc_bvh_node* nodes, int n_node, int tree_mode,
                 Repacked& out, std::string& err) {
  Builder b{tris, n_tri, nodes, n_node, {}, {}, 0};
  out = Repacked();
  const float INF = INFINITY;
  // shading records: normalize(vn1..vn3) and the material index
  out.shade.resize((size_t)n_tri * 4);
  parallel_for((size_t)n_tri, [&](size_t i) {
    const yc_triangle& t = tris[i];
    const yc_float4* vn[3] = {&t.vn1, &t.vn2, &t.vn3};
    for (int k = 0; k < 3; ++k) {
      const ym::f4 n = ym::normalize(ym::mk(vn[k]->x, vn[k]->y, vn[k]->z, vn[k]->w));
      out.shade[4 * (size_t)i + k] = float4{n.x, n.y, n.z, n.w};
    }
    float mid;
    int m = t.matID;
    std::memcpy(&mid, &m, 4);
    out.shade[4 * (size_t)i + 3] = float4{mid, 0.0f, 0.0f, 0.0f};
  });

  if (n_tri == 0) {
    out.root_link = LINK_NONE;
    out.root_test = 0;
    out.depth = 0;
    return 0;
  }
  if (n_node == 0) {
    // brute force: chain of unbounded nodes, leaves of up to 15 triangles in index order
    const int per = 15;
    const int n_leaf = (n_tri + per - 1) / per;
    std::vector<int> ids(n_tri);
    for (int i = 0; i < n_tri; ++i) ids[i] = i;
    if (n_leaf == 1) {
      out.root_link = b.emit_leaf(ids.data(), n_tri, 0);
    } else {
      for (int l = 0; l < n_leaf - 1; ++l) {
        const int leaf = b.emit_leaf(ids.data() + l * per, per, l * per);
        int next;
        if (l == n_leaf - 2) {
          const int rest = n_tri - (l + 1) * per;
          next = b.emit_leaf(ids.data() + (l + 1) * per, rest, (l + 1) * per);
        } else {
          next = (int)(b.out_nodes.size() / 4) + 1;
        }
        const float lo[3] = {-INF, -INF, -INF}, hi[3] = {INF, INF, INF};
        const size_t at = b.out_nodes.size();
        b.out_nodes.resize(at + 4);
        write_node2(&b.out_nodes[at], lo, hi, lo, hi, leaf, next);
      }
      out.root_link = 0;
    }
    out.root_test = 0;
    out.depth = 2;
    out.nodes.swap(b.out_nodes);
    out.tris.swap(b.out_tris);
    return 0;
  }

  if (check_nodes(nodes, n_node, n_tri, err)) return -1;
  const yc_bvh_node& root = nodes[0];
  out.root_test = 1;
  out.root_lo = float4{root.aabb.p_min.x, root.aabb.p_min.y, root.aabb.p_min.z, 0.0f};
  out.root_hi = float4{root.aabb.p_max.x, root.aabb.p_max.y, root.aabb.p_max.z, 0.0f};
  if (n_node >= (1 << 27)) { err = "BVH too large for the 27-bit tie-break rank"; return -1; }
  if (is_leaf(root)) {
    out.root_link = b.emit_leaf(root.vert_list, root.vert_len, 0);
    out.depth = 0;
    out.tris.swap(b.out_tris);
    return 0;
  }
  if (tree_mode == TREE_SAH_OVER_LEAVES || tree_mode == TREE_WIDE4) {
    // the leaves the reference traversal can reach, in node-index order, and the first
    // stream slot of each (then the stream and the leaf items are filled in parallel,
    // exactly as emit_leaf would append them one after another)
    std::vector<int> leaf_node, leaf_first;
    size_t slots = 0;
    reachable_leaves(nodes, n_node, leaf_node, leaf_first, slots);
    if (leaf_node.empty()) { out.root_link = LINK_NONE; out.depth = 0; return 0; }
    if (slots >= (size_t)(1 << 27)) { err = "scene too large for the 27-bit stream index"; return -1; }
    std::vector<LeafItem> items(leaf_node.size());
    b.out_tris.resize(slots * 3);
    parallel_for(leaf_node.size(), [&](size_t j) {
      const int i = leaf_node[j];
      const yc_bvh_node& n = nodes[i];
      LeafItem& it = items[j];
      const float* plo = &n.aabb.p_min.x;
      const float* phi = &n.aabb.p_max.x;
      for (int k = 0; k < 3; ++k) {
        it.lo[k] = plo[k];
        it.hi[k] = phi[k];
        it.c[k] = sah_centroid(plo[k], phi[k]);
      }
      it.link = b.fill_leaf(n.vert_list, n.vert_len, i * 16, leaf_first[j]);
      it.w = n.vert_len;
    });
    SahBuilder sb{items};
    const BinRef root_ref = sb.build(0, (int)items.size(), 0);
    if (tree_mode == TREE_WIDE4) {
      int d = 0;
      out.root_link = sb.emit_wide(root_ref, b.out_nodes, d);
      out.wide = 1;
      out.depth = 3 * d;   // up to three entries pushed per wide level
    } else {
      out.root_link = sb.emit_binary(root_ref, b.out_nodes);
      out.depth = sb.max_depth + 1;
    }
    out.nodes.swap(b.out_nodes);
    out.tris.swap(b.out_tris);
    return 0;
  }
  // breadth-first over interior nodes; packed index assigned on first visit
  std::vector<int> packed_of(n_node, -1);
  std::vector<int> level(n_node, 0);
  std::vector<int> order;
  order.reserve(n_node);
  order.push_back(0);
  packed_of[0] = 0;
  for (size_t q = 0; q < order.size(); ++q) {
    const int ni = order[q];
    const yc_bvh_node& n = nodes[ni];
    for (int c = 0; c < 2; ++c) {
      const int ci = n.child_idx + c;
      const yc_bvh_node& ch = nodes[ci];
      if (is_queued(ch) && !is_leaf(ch)) {
        if (packed_of[ci] >= 0) { err = "BVH is not a tree (node reached twice)"; return -1; }
        packed_of[ci] = (int)order.size();
        level[ci] = level[ni] + 1;
        order.push_back(ci);
        if ((int)order.size() > n_node) { err = "BVH has a cycle"; return -1; }
      }
    }
  }
  b.out_nodes.resize(order.size() * 4);
  int depth = 0;
  for (size_t q = 0; q < order.size(); ++q) {
    const yc_bvh_node& n = nodes[order[q]];
    depth = std::max(depth, level[order[q]] + 1);
    int link[2];
    const yc_aabb* box[2];
    for (int c = 0; c < 2; ++c) {
      const int ci = n.child_idx + c;
      const yc_bvh_node& ch = nodes[ci];
      box[c] = &ch.aabb;
      if (!is_queued(ch)) link[c] = LINK_NONE;
      else if (is_leaf(ch)) link[c] = b.emit_leaf(ch.vert_list, ch.vert_len, ci * 16);
      else link[c] = packed_of[ci];
    }
    write_node2(&b.out_nodes[4 * q], &box[0]->p_min.x, &box[0]->p_max.x, &box[1]->p_min.x, &box[1]->p_max.x, link[0],
                link[1]);
    if ((b.out_tris.size() / 3) >= (size_t)(1 << 27)) { err = "scene too large for the 27-bit stream index"; return -1; }
  }
  out.root_link = 0;
  out.depth = depth;
  out.nodes.swap(b.out_nodes);
  out.tris.swap(b.out_tris);
  return 0;
}

}  // namespace yc
