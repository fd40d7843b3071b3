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

// walk_host.cpp: the device walk's work on explicit rays (9 floats each) replayed one ray
// at a time on the host, without the warp's speculative leaves: child boxes and triangles
// tested, and each ray's closest (any = false) or first (any = true) triangle and t.
int walk_counts_host(const Repacked& rp, const float* rays9, int n, bool any, uint64_t* boxes, uint64_t* tris,
                     int* tri_out, float* t_out, std::string& err);

}  // namespace yc
