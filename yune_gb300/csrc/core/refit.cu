// refit.cu -- refit of an uploaded scene for moving geometry, on the device
// (yc_refit_scene).
//
// Yune refits its BVH after a build with BVH::resizeBvh (src/BVH.cpp:218-247): every leaf
// box becomes the union of its triangles' boxes (TriangleCPU::computeAABB,
// src/TriangleCPU.cpp:51-71: per axis the minimum and maximum of the three vertices, the
// maximum raised by 0.2 where the two are equal), every interior box the union of its
// children's. Here the same pass runs on the repacked scene where it lies in HBM, for new
// vertex positions of the same triangles: the stream records (v1, e1 = v2 - v1,
// e2 = v3 - v1) and the shading records are rewritten from the new triangles, then the
// child boxes of every node, level by level from the deepest: a leaf child's box from its
// triangles, an interior child's box as the union of that child's own child boxes (written
// by the previous level). Leaf boxes are then exactly the reference's refitted leaf boxes
// (min and max are exact in any order), and every interior box contains the leaves below
// it, so the walk's hits are those of the reference tree refitted by resizeBvh. The
// hierarchy (its topology, leaves and tie-break ranks) is kept.
//
// Compiled with -fmad=false like the rest of the core.
#include <cuda_runtime.h>

#include "../ym_math.h"
#include "yc_internal.h"

namespace yc {

constexpr int REFIT_TB = 256;

struct Box3 {
  float lo[3], hi[3];
};

__device__ __forceinline__ void box_empty(Box3& b) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = __int_as_float(0x7f800000);
    b.hi[k] = -__int_as_float(0x7f800000);
  }
}
__device__ __forceinline__ void box_join(Box3& b, const float lo[3], const float hi[3]) {
  for (int k = 0; k < 3; ++k) {
    b.lo[k] = fminf(b.lo[k], lo[k]);
    b.hi[k] = fmaxf(b.hi[k], hi[k]);
  }
}

// TriangleCPU::computeAABB of triangle t
__device__ __forceinline__ void tri_box(const yc_triangle& t, float lo[3], float hi[3]) {
  const float a[3] = {t.v1.x, t.v1.y, t.v1.z}, b[3] = {t.v2.x, t.v2.y, t.v2.z}, c[3] = {t.v3.x, t.v3.y, t.v3.z};
  for (int k = 0; k < 3; ++k) {
    lo[k] = fminf(a[k], fminf(b[k], c[k]));
    hi[k] = fmaxf(a[k], fmaxf(b[k], c[k]));
    if (__fsub_rn(hi[k], lo[k]) == 0.0f) hi[k] = __fadd_rn(hi[k], 0.2f);
  }
}

// the box of a leaf: its stream slots [first, first + count)
__device__ __forceinline__ void leaf_box(int link, const float4* stream, const yc_triangle* tris, Box3& b) {
  box_empty(b);
  const int enc = ~link;
  const int first = enc >> 4, count = enc & 15;
  for (int k = 0; k < count; ++k) {
    const int id = __float_as_int(stream[3 * (size_t)(first + k)].w);
    float lo[3], hi[3];
    tri_box(tris[id], lo, hi);
    box_join(b, lo, hi);
  }
}

// the union of a node's child boxes (two-child or four-child layout of yc_scene.h)
__device__ __forceinline__ void node_box(const float4* nodes, int n, bool wide, Box3& b) {
  box_empty(b);
  if (!wide) {
    const float4* nd = nodes + 4 * (size_t)n;
    const float4 x = nd[0], y = nd[1], z = nd[2];
    const int2 l = *reinterpret_cast<const int2*>(nd + 3);
    if (l.x != LINK_NONE) {
      const float lo[3] = {x.x, y.x, z.x}, hi[3] = {x.z, y.z, z.z};
      box_join(b, lo, hi);
    }
    if (l.y != LINK_NONE) {
      const float lo[3] = {x.y, y.y, z.y}, hi[3] = {x.w, y.w, z.w};
      box_join(b, lo, hi);
    }
    return;
  }
  const float4* nd = nodes + 8 * (size_t)n;
  const float4 lx = nd[0], hx = nd[1], ly = nd[2], hy = nd[3], lz = nd[4], hz = nd[5];
  const int4 l = *reinterpret_cast<const int4*>(nd + 6);
  const float clx[4] = {lx.x, lx.y, lx.z, lx.w}, chx[4] = {hx.x, hx.y, hx.z, hx.w};
  const float cly[4] = {ly.x, ly.y, ly.z, ly.w}, chy[4] = {hy.x, hy.y, hy.z, hy.w};
  const float clz[4] = {lz.x, lz.y, lz.z, lz.w}, chz[4] = {hz.x, hz.y, hz.z, hz.w};
  const int cl[4] = {l.x, l.y, l.z, l.w};
  for (int c = 0; c < 4; ++c)
    if (cl[c] != LINK_NONE) {
      const float lo[3] = {clx[c], cly[c], clz[c]}, hi[3] = {chx[c], chy[c], chz[c]};
      box_join(b, lo, hi);
    }
}

__device__ __forceinline__ void child_box(int link, const float4* nodes, bool wide, const float4* stream,
                                          const yc_triangle* tris, Box3& b) {
  if (link < 0) leaf_box(link, stream, tris, b);
  else node_box(nodes, link, wide, b);
}

// stream records of the new positions: (v1, index), (v2 - v1, rank), (v3 - v1, 0)
__global__ void __launch_bounds__(REFIT_TB) k_refit_stream(const yc_triangle* __restrict__ tris, float4* stream,
                                                           int n_slots) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slots) return;
  float4* r = stream + 3 * (size_t)s;
  const float4 a = r[0];
  const yc_triangle& t = tris[__float_as_int(a.w)];
  r[0] = make_float4(t.v1.x, t.v1.y, t.v1.z, a.w);
  r[1] = make_float4(__fsub_rn(t.v2.x, t.v1.x), __fsub_rn(t.v2.y, t.v1.y), __fsub_rn(t.v2.z, t.v1.z), r[1].w);
  r[2] = make_float4(__fsub_rn(t.v3.x, t.v1.x), __fsub_rn(t.v3.y, t.v1.y), __fsub_rn(t.v3.z, t.v1.z), 0.0f);
}

// shading records: normalize(vn1..vn3) (udpt.cl:377-379) and the material index
__global__ void __launch_bounds__(REFIT_TB) k_refit_shade(const yc_triangle* __restrict__ tris, float4* shade,
                                                          int n_tri) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_tri) return;
  const yc_triangle& t = tris[i];
  const yc_float4* vn[3] = {&t.vn1, &t.vn2, &t.vn3};
  for (int k = 0; k < 3; ++k) {
    const ym::f4 n = ym::normalize(ym::mk(vn[k]->x, vn[k]->y, vn[k]->z, vn[k]->w));
    shade[4 * (size_t)i + k] = make_float4(n.x, n.y, n.z, n.w);
  }
  shade[4 * (size_t)i + 3] = make_float4(__int_as_float(t.matID), 0.0f, 0.0f, 0.0f);
}

// the child boxes of the nodes order[0..n): every child's nodes are already refitted
__global__ void __launch_bounds__(REFIT_TB) k_refit_level(const int* __restrict__ order, int n, float4* nodes,
                                                          bool wide, const float4* __restrict__ stream,
                                                          const yc_triangle* __restrict__ tris) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int node = order[i];
  if (!wide) {
    float4* nd = nodes + 4 * (size_t)node;
    const int2 l = *reinterpret_cast<const int2*>(nd + 3);
    Box3 b0, b1;
    box_empty(b0);
    box_empty(b1);
    if (l.x != LINK_NONE) child_box(l.x, nodes, false, stream, tris, b0);
    if (l.y != LINK_NONE) child_box(l.y, nodes, false, stream, tris, b1);
    float4 o[3];
    for (int k = 0; k < 3; ++k) o[k] = nd[k];
    if (l.x != LINK_NONE) { o[0].x = b0.lo[0]; o[1].x = b0.lo[1]; o[2].x = b0.lo[2]; o[0].z = b0.hi[0]; o[1].z = b0.hi[1]; o[2].z = b0.hi[2]; }
    if (l.y != LINK_NONE) { o[0].y = b1.lo[0]; o[1].y = b1.lo[1]; o[2].y = b1.lo[2]; o[0].w = b1.hi[0]; o[1].w = b1.hi[1]; o[2].w = b1.hi[2]; }
    for (int k = 0; k < 3; ++k) nd[k] = o[k];
    return;
  }
  float4* nd = nodes + 8 * (size_t)node;
  const int4 l = *reinterpret_cast<const int4*>(nd + 6);
  const int cl[4] = {l.x, l.y, l.z, l.w};
  float v[6][4];
  for (int f = 0; f < 6; ++f) {
    const float4 q = nd[f];
    v[f][0] = q.x; v[f][1] = q.y; v[f][2] = q.z; v[f][3] = q.w;
  }
  for (int c = 0; c < 4; ++c) {
    if (cl[c] == LINK_NONE) continue;
    Box3 b;
    child_box(cl[c], nodes, true, stream, tris, b);
    for (int k = 0; k < 3; ++k) {
      v[2 * k][c] = b.lo[k];
      v[2 * k + 1][c] = b.hi[k];
    }
  }
  for (int f = 0; f < 6; ++f) nd[f] = make_float4(v[f][0], v[f][1], v[f][2], v[f][3]);
}

// the scene box the walk tests first: the union of the root's child boxes (or of the root
// leaf's triangles)
__global__ void k_refit_root(int root_link, const float4* nodes, bool wide, const float4* stream,
                             const yc_triangle* tris, float4* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  Box3 b;
  child_box(root_link, nodes, wide, stream, tris, b);
  out[0] = make_float4(b.lo[0], b.lo[1], b.lo[2], 0.0f);
  out[1] = make_float4(b.hi[0], b.hi[1], b.hi[2], 0.0f);
}

int launch_refit(const RefitPlan& plan, const yc_triangle* tris_dev, int n_tri, float4* nodes, float4* stream,
                 int n_slots, float4* shade, bool wide, int root_link, bool refit_nodes, float4* root_out,
                 cudaStream_t s) {
  if (n_slots > 0) k_refit_stream<<<(n_slots + REFIT_TB - 1) / REFIT_TB, REFIT_TB, 0, s>>>(tris_dev, stream, n_slots);
  if (n_tri > 0) k_refit_shade<<<(n_tri + REFIT_TB - 1) / REFIT_TB, REFIT_TB, 0, s>>>(tris_dev, shade, n_tri);
  if (refit_nodes) {
    for (size_t lv = 0; lv + 1 < plan.level_off.size(); ++lv) {   // deepest level first
      const int b = plan.level_off[lv], e = plan.level_off[lv + 1];
      if (e > b)
        k_refit_level<<<(e - b + REFIT_TB - 1) / REFIT_TB, REFIT_TB, 0, s>>>(plan.order + b, e - b, nodes, wide,
                                                                             stream, tris_dev);
    }
    if (root_link != LINK_NONE) k_refit_root<<<1, 32, 0, s>>>(root_link, nodes, wide, stream, tris_dev, root_out);
  }
  return cudaPeekAtLastError() == cudaSuccess ? 0 : -1;
}

}  // namespace yc
