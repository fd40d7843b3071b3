// yc_scene.h -- device layout of an uploaded scene (shared by host and device code).
//
// One scene in HBM is five read-only arrays, all 16-byte aligned and fetched with
// 128-bit loads:
//   nodes   two-child layout: 4 x float4 (64 B) per interior node, holding the boxes
//           of its two children (the 32 B a box test reads) and their links:
//             n0 = (c0.lo.x, c1.lo.x, c0.hi.x, c1.hi.x)
//             n1 = (c0.lo.y, c1.lo.y, c0.hi.y, c1.hi.y)
//             n2 = (c0.lo.z, c1.lo.z, c0.hi.z, c1.hi.z)
//             n3 = (link0, link1, 0, 0) as int bits
//           (each 64-bit half is the (child 0, child 1) pair one packed f32x2 operation
//           of the box test takes)
//           link >= 0: interior node index; link < 0: leaf, ~link = (first stream slot
//           << 4) | triangle count (a reference leaf holds at most 10); LINK_NONE: a
//           child the reference never queues (vert_len <= 0 and child_idx <= 0,
//           udpt.cl:316).
//           four-child layout (wide = 1): 8 x float4 (128 B) per node, the boxes of
//           its four children as lo.x[4], hi.x[4], lo.y[4], hi.y[4], lo.z[4], hi.z[4],
//           then the four links (LINK_NONE for an empty slot) and 16 unused bytes.
//   tris    3 x float4 (48 B) per stream slot, leaves' triangles contiguous:
//             (v1.xyz, original index), (e1 = v2 - v1, tie-break rank), (e2 = v3 - v1, 0)
//           with the index and rank as int bits; the rank orders triangles at equal t
//           the way the reference's breadth-first walk meets them (see repack.cpp)
//           e1/e2 are the subtractions rayTriangleIntersection does (udpt.cl:328-329),
//           done once on the host in FP32, which gives the same bits.
//   shade   4 x float4 (64 B) per original triangle: normalize(vn1..vn3) (udpt.cl:377-379,
//           the same FP32 operations) and (matID, 0, 0, 0).
//   mats    Material records as uploaded (80 B each).
//   lights  quad lights (128 B each).
#pragma once

#include <stdint.h>

#include "yune_types.h"

namespace yc {

constexpr int LINK_NONE = 0x7fffffff;
constexpr int MAX_LIGHTS = 16;

struct DevScene {
  const float4* nodes;
  const float4* tris;
  const float4* shade;
  const yc_material* mats;
  const yc_quad_light* lights;
  const float2* on_ab;   // per material: the Oren-Nayar A and B of its sigma^2 (oren_nayar_ab)
  int n_lights;
  int n_tri;
  int n_mat;
  int root_link;       // link of the reference root node 0
  int wide;            // 1: four-child nodes (8 x float4 each), 0: two-child nodes
  int root_test;       // 1: test the root box first (traverseBVH, udpt.cl:295); 0: brute force
  int depth;           // interior levels below the root (stack slots needed)
  int pad_;
  float4 root_lo, root_hi;
};

}  // namespace yc
