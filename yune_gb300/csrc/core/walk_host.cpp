// walk_host.cpp -- the traversal's algorithmic work, counted on the host (yc_walk_counts).
//
// The device walk (yc_traverse.cuh) runs a warp's rays together: a lane that reaches a
// leaf keeps it aside and goes on opening nodes until every lane has a leaf, so a ray may
// open boxes that a walk of its own would have culled, and the device counters
// (yc_stats: ext_boxes, any_tris, ...) count that speculative work too. This file replays
// one ray at a time in the device walk's order -- the nearer child first, the same
// distance cull (a child is skipped when its entry lies beyond the closest hit by more than
// 2^-10 relative), the reference's slab and Moller-Trumbore arithmetic -- without the
// speculation, and counts the child boxes and triangles the ray itself needs: the
// algorithmic bytes of the traversal roofline. It also returns each ray's result, which
// must equal the device walk's and the reference's.
//
// Host code compiled with -ffp-contract=off: every float expression rounds as the device
// code's __fadd_rn / __fmul_rn forms do.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "yc_repack.h"

namespace yc {

namespace {

float ocl_min(float x, float y) { return (y < x) ? y : x; }
float ocl_fmax(float x, float y) {
  if (x != x) return y;
  if (y != y) return x;
  return (x < y) ? y : x;
}

struct HostRay {
  float o[3], d[3], inv[3];
  bool exact;
};

// rayAabbIntersection with the reference's NaN-skipping slab arithmetic
bool box_ref(const HostRay& r, const float lo[3], const float hi[3], float& tentry) {
  float t_max = INFINITY, t_min = -INFINITY;
  for (int k = 0; k < 3; ++k) {
    const float mn = (lo[k] - r.o[k]) * r.inv[k], mx = (hi[k] - r.o[k]) * r.inv[k];
    if (!(mn != mn)) {
      t_min = ocl_fmax(ocl_min(mn, mx), t_min);
      t_max = ocl_min(ocl_fmax(mn, mx), t_max);
    }
    if (k == 1 && t_max < t_min) {
      tentry = t_min;
      return false;
    }
  }
  tentry = t_min;
  return t_max > ocl_fmax(t_min, 0.0f);
}

// the device's box_fast (finite reciprocals): the same result as box_ref, with the cull
bool box_fast(const HostRay& r, const float lo[3], const float hi[3], float cull_up, bool clamp, float& tentry) {
  float a[3], b[3];
  for (int k = 0; k < 3; ++k) {
    a[k] = (lo[k] - r.o[k]) * r.inv[k];
    b[k] = (hi[k] - r.o[k]) * r.inv[k];
  }
  const float t0 = std::fmax(std::fmax(std::fmin(a[0], b[0]), std::fmin(a[1], b[1])), std::fmin(a[2], b[2]));
  const float t1 = std::fmin(std::fmin(std::fmax(a[0], b[0]), std::fmax(a[1], b[1])),
                             std::fmin(std::fmax(a[2], b[2]), cull_up));
  const float t0c = std::fmax(t0, 0.0f);
  tentry = clamp ? t0c : t0;
  return t1 > t0c;
}

float cull_bound(float best) { return best * 1.0009765625f; }
float cull_up(float best) {
  const float cb = cull_bound(best);
  if (std::isinf(cb)) return cb;
  int32_t i;
  std::memcpy(&i, &cb, 4);
  ++i;
  float r;
  std::memcpy(&r, &i, 4);
  return r;
}

// rayTriangleIntersection on a stream slot (v1, e1, e2), the device's tri_test
bool tri_test(const HostRay& r, const float4& a, const float4& b, const float4& c, float best, int best_rank,
              float& t_out) {
  const float px = r.d[1] * c.z - r.d[2] * c.y;
  const float py = r.d[2] * c.x - r.d[0] * c.z;
  const float pz = r.d[0] * c.y - r.d[1] * c.x;
  const float det = ((b.x * px + b.y * py) + b.z * pz) + 0.0f;
  const float inv_det = 1.0f / det;
  const float sx = r.o[0] - a.x, sy = r.o[1] - a.y, sz = r.o[2] - a.z;
  const float u = (((px * sx + py * sy) + pz * sz) + 0.0f) * inv_det;
  if (u < 0.0f || u > 1.0f) return false;
  const float qx = sy * b.z - sz * b.y;
  const float qy = sz * b.x - sx * b.z;
  const float qz = sx * b.y - sy * b.x;
  const float v = (((qx * r.d[0] + qy * r.d[1]) + qz * r.d[2]) + 0.0f) * inv_det;
  if (v < 0.0f || u + v > 1.0f) return false;
  const float t = (((c.x * qx + c.y * qy) + c.z * qz) + 0.0f) * inv_det;
  int rank;
  std::memcpy(&rank, &b.w, 4);
  if (t > 0.0f && (t < best || (t == best && rank < best_rank))) {
    t_out = t;
    return true;
  }
  return false;
}

}  // namespace

int walk_counts_host(const Repacked& rp, const float* rays9, int n, bool any, uint64_t* boxes_out,
                     uint64_t* tris_out, int* tri_out, float* t_out, std::string& err) {
  if (rp.wide > 1) {
    err = "the host replay walks two-child and four-child float nodes (tree modes 0, 1 and 2)";
    return -1;
  }
  uint64_t boxes = 0, tris = 0;
  std::vector<std::pair<int, float>> stack;
  for (int i = 0; i < n; ++i) {
    const float* q = rays9 + 9 * (size_t)i;
    HostRay r;
    for (int k = 0; k < 3; ++k) {
      r.o[k] = q[k];
      r.d[k] = q[4 + k];
      r.inv[k] = 1.0f / r.d[k];
    }
    r.exact = std::isinf(r.inv[0]) || std::isinf(r.inv[1]) || std::isinf(r.inv[2]);
    float best = q[8];
    int best_tri = -1, best_rank = -1;
    int link = rp.root_link;
    if (link != LINK_NONE && rp.root_test) {
      const float lo[3] = {rp.root_lo.x, rp.root_lo.y, rp.root_lo.z}, hi[3] = {rp.root_hi.x, rp.root_hi.y, rp.root_hi.z};
      float te;
      const bool h = r.exact ? box_ref(r, lo, hi, te) : box_fast(r, lo, hi, INFINITY, false, te);
      if (!h) link = LINK_NONE;
    }
    float link_t = -INFINITY;
    stack.clear();
    auto pop = [&]() {
      while (!stack.empty()) {
        const std::pair<int, float> e = stack.back();
        stack.pop_back();
        if (!(e.second > cull_bound(best))) {
          link_t = e.second;
          return e.first;
        }
      }
      return (int)LINK_NONE;
    };
    bool stop = false;
    while (!stop && link != LINK_NONE) {
      if (!any && link_t > cull_bound(best)) {   // a hit found since this subtree was chosen
        link = pop();
        continue;
      }
      if (link < 0) {   // leaf: its triangles in stream order
        const int enc = ~link;
        const int count = enc & 15;
        const float4* tp = rp.tris.data() + 3 * (size_t)(enc >> 4);
        for (int k = 0; k < count && !stop; ++k) {
          ++tris;
          float t;
          if (tri_test(r, tp[3 * k], tp[3 * k + 1], tp[3 * k + 2], best, best_rank, t)) {
            best = t;
            std::memcpy(&best_tri, &tp[3 * k].w, 4);
            std::memcpy(&best_rank, &tp[3 * k + 1].w, 4);
            if (any) stop = true;
          }
        }
        link = stop ? (int)LINK_NONE : pop();
        continue;
      }
      if (rp.wide) {   // four-child node (yc_scene.h): lo.x[4], hi.x[4], ..., links; visit4's order
        const float4* nd = rp.nodes.data() + 8 * (size_t)link;
        boxes += 4;
        const float* f = reinterpret_cast<const float*>(nd);
        int cl[4];
        std::memcpy(cl, &nd[6], 16);
        const float cb = cull_bound(best), up = cull_up(best);
        float t[4];
        int l[4];
        for (int c = 0; c < 4; ++c) {
          const float lo[3] = {f[c], f[8 + c], f[16 + c]}, hi[3] = {f[4 + c], f[12 + c], f[20 + c]};
          float te;
          bool h = !r.exact ? box_fast(r, lo, hi, up, !any, te) : (box_ref(r, lo, hi, te) && !(te > cb));
          h = h && cl[c] != LINK_NONE;
          t[c] = h ? te : INFINITY;
          l[c] = h ? cl[c] : (int)LINK_NONE;
        }
        auto cx = [&](int a, int b) {
          if (t[b] < t[a]) { std::swap(t[a], t[b]); std::swap(l[a], l[b]); }
        };
        cx(0, 1); cx(2, 3); cx(0, 2); cx(1, 3); cx(1, 2);
        if (l[0] == LINK_NONE) {
          link = pop();
          continue;
        }
        for (int c = 3; c >= 1; --c)
          if (l[c] != LINK_NONE) stack.emplace_back(l[c], t[c]);
        link_t = t[0];
        link = l[0];
        continue;
      }
      // two-child node (yc_scene.h): per axis (lo pair, hi pair), then the links
      const float4* nd = rp.nodes.data() + 4 * (size_t)link;
      boxes += 2;
      const float lo0[3] = {nd[0].x, nd[1].x, nd[2].x}, lo1[3] = {nd[0].y, nd[1].y, nd[2].y};
      const float hi0[3] = {nd[0].z, nd[1].z, nd[2].z}, hi1[3] = {nd[0].w, nd[1].w, nd[2].w};
      int l0, l1;
      std::memcpy(&l0, &nd[3].x, 4);
      std::memcpy(&l1, &nd[3].y, 4);
      float t0, t1;
      bool h0, h1;
      if (!r.exact) {
        const float up = cull_up(best);
        h0 = box_fast(r, lo0, hi0, up, !any, t0);
        h1 = box_fast(r, lo1, hi1, up, !any, t1);
      } else {
        h0 = box_ref(r, lo0, hi0, t0);
        h1 = box_ref(r, lo1, hi1, t1);
        const float cb = cull_bound(best);
        h0 = h0 && !(t0 > cb);
        h1 = h1 && !(t1 > cb);
      }
      h0 = h0 && l0 != LINK_NONE;
      h1 = h1 && l1 != LINK_NONE;
      if (h0 && h1) {
        const bool swap = t1 < t0;
        stack.emplace_back(swap ? l0 : l1, swap ? t0 : t1);
        link_t = swap ? t1 : t0;
        link = swap ? l1 : l0;
      } else if (h0) {
        link_t = t0;
        link = l0;
      } else if (h1) {
        link_t = t1;
        link = l1;
      } else {
        link = pop();
      }
    }
    if (tri_out) tri_out[i] = best_tri;
    if (t_out) t_out[i] = best_tri >= 0 ? best : q[8];
  }
  *boxes_out = boxes;
  *tris_out = tris;
  return 0;
}

}  // namespace yc
