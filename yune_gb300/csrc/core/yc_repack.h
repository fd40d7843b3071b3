// yc_repack.h -- host-side repack of a scene into the device layout of yc_scene.h.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <memory>
#include <utility>
#include <vector>

#include "yc_scene.h"

namespace yc {

// An allocator whose resize() leaves new elements uninitialised (float4 records are
// written in parallel right after, so their pages are first touched by the filling threads
// instead of by a sequential zero fill).
template <class T>
struct NoInitAlloc : std::allocator<T> {
  template <class U> struct rebind { using other = NoInitAlloc<U>; };
  NoInitAlloc() = default;
  template <class U> NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
  template <class U> void construct(U* p) noexcept { ::new (static_cast<void*>(p)) U; }
  template <class U, class... A> void construct(U* p, A&&... a) { ::new (static_cast<void*>(p)) U(std::forward<A>(a)...); }
};
using F4Vec = std::vector<float4, NoInitAlloc<float4>>;

struct Repacked {
  F4Vec nodes;   // 4 per two-child node, 8 per four-child node
  F4Vec tris;    // 3 per stream slot
  F4Vec shade;   // 4 per original triangle
  int root_link = LINK_NONE;
  int root_test = 0;
  int depth = 0;               // stack entries a walk can need
  int wide = 0;                // 1: four-child nodes
  float4 root_lo{0, 0, 0, 0}, root_hi{0, 0, 0, 0};
};

// tree_mode: how the interior nodes above the reference leaves are laid out
enum { TREE_REFERENCE = 0, TREE_SAH_OVER_LEAVES = 1, TREE_WIDE4 = 2 };

// Returns 0, or -1 with a message when the node array is not a tree the reference
// traversal could walk (child indices out of range, vert_len > 10, ...).
int repack_scene(const yc_triangle* tris, int n_tri, const yc_bvh_node* nodes, int n_node, int tree_mode,
                 Repacked& out, std::string& err);

// -1 with err naming the first triangle whose matID is outside [0, n_mat) (checked on the
// host's threads), else 0
int check_materials(const yc_triangle* tris, int n_tri, int n_mat, std::string& err);

// The host half of the device repack of TREE_SAH_OVER_LEAVES (repack_dev.cu): the node
// array's checks (those of repack_scene) and the reachable leaves with their first
// stream slots. Returns 1 when the scene takes the device repack (two reachable leaves or
// more), 0 when it does not (no triangles, no BVH, a leaf at the root, fewer than two
// reachable leaves: repack_scene is then immediate), -1 with err for a node array the
// upload rejects.
struct DevRepackPlan {
  std::vector<int> leaf_node, leaf_first;   // reachable leaves in node-index order, first slots
  size_t slots = 0;                         // stream slots in all
  float4 root_lo{0, 0, 0, 0}, root_hi{0, 0, 0, 0};
};
int plan_device_repack(const yc_bvh_node* nodes, int n_node, int n_tri, DevRepackPlan& plan, std::string& err);

// repack_dev.cu: the repack of a planned scene on the device, on stream s: nodes receives
// the leaves - 1 two-child nodes (4 float4 each), stream the plan's slots (3 float4 each),
// shade the triangles' shading records (4 float4 each), depth the stack entries a walk
// can need -- byte for byte what repack_scene gives for TREE_SAH_OVER_LEAVES. The
// temporaries (the caller's arrays copied over, the leaf items, the split tasks) are freed
// before it returns. Returns 0, or -2 (a device allocation failed) or -1 with err.
int repack_device(const yc_triangle* tris_host, int n_tri, const yc_bvh_node* nodes_host, int n_node,
                  const DevRepackPlan& plan, float4* nodes, float4* stream, float4* shade, int& depth, cudaStream_t s,
                  std::string& err);

// walk_host.cpp: the device walk's work on explicit rays (9 floats each) replayed one ray
// at a time on the host, without the warp's speculative leaves: child boxes and triangles
// tested, and each ray's closest (any = false) or first (any = true) triangle and t.
int walk_counts_host(const Repacked& rp, const float* rays9, int n, bool any, uint64_t* boxes, uint64_t* tris,
                     int* tri_out, float* t_out, std::string& err);

}  // namespace yc
