// yc_traverse.cuh -- BVH traversal for sm_103a: while-while depth-first walk over the
// repacked two-child or four-child nodes with a per-thread stack in shared memory.
//
// The tests themselves are the reference's, operation for operation, so the accepted
// triangles and their t are bit-identical to traverseBVH + rayTriangleIntersection
// (kernels/legacy/udpt.cl:288-390). What changes is the order of the walk: the
// reference visits, breadth first, every box the ray's half-line crosses and keeps the
// first triangle with the smallest t; here the nearer child is visited first and a
// child is skipped once its entry distance lies beyond the closest hit found so far (by
// a margin of 2^-10 relative, so rounding of the entry distance can never hide a
// triangle the reference would accept). Between triangles at exactly the same t the
// reference keeps the first it visits; every stream slot carries that visiting rank and
// an equal-t candidate replaces the current one only when its rank is lower, so the
// closest triangle and its t are the reference's bit for bit.
//
// The translation unit is compiled with -fmad=false: no multiply-add is fused, as in
// the reference arithmetic.
#pragma once

#include <stdint.h>

#include "yc_scene.h"

namespace yc {

struct RayIn {
  float ox, oy, oz, tmax;
  float dx, dy, dz;
};

struct HitOut {
  float t, u, v;
  int tri;   // original triangle index, -1 when nothing closer than tmax
};

// work done by walks: child boxes tested (two per two-child node, four per four-child
// node) and triangles tested
struct WalkCount {
  unsigned nodes = 0, tris = 0;
};

// ---- packed pairs: the f32x2 operations of sm_100 and later apply the IEEE
// round-to-nearest operation to each 32-bit half of a 64-bit register, so one packed
// operation gives exactly the bits of the two scalar operations it replaces, at one
// instruction issue. The two-child node stores its bounds as (child 0, child 1) pairs.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void up2(f32x2 v, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ float lo2(f32x2 v) {
  float a, b;
  up2(v, a, b);
  return a;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}

// OpenCL `min` (y if y < x, otherwise x); NaN-sensitive like the reference.
__device__ __forceinline__ float ocl_min(float x, float y) { return (y < x) ? y : x; }
// OpenCL `fmax` (NaN operand ignored; ties keep x).
__device__ __forceinline__ float ocl_fmax(float x, float y) {
  if (x != x) return y;
  if (y != y) return x;
  return (x < y) ? y : x;
}

// rayAabbIntersection (udpt.cl:392-431) exactly, for rays with a zero or subnormal
// direction component (1/d = inf can make (p - o) * inv NaN, and the reference then
// skips that axis). Returns hit and the entry distance.
__device__ __forceinline__ bool box_ref(float ox, float oy, float oz, float ix, float iy, float iz,
                                        float lx, float hx, float ly, float hy, float lz, float hz,
                                        float& tentry) {
  float t_max = __int_as_float(0x7f800000), t_min = -__int_as_float(0x7f800000);
  float mn = __fmul_rn(__fsub_rn(lx, ox), ix), mx = __fmul_rn(__fsub_rn(hx, ox), ix);
  if (!(mn != mn)) { t_min = ocl_fmax(ocl_min(mn, mx), t_min); t_max = ocl_min(ocl_fmax(mn, mx), t_max); }
  mn = __fmul_rn(__fsub_rn(ly, oy), iy); mx = __fmul_rn(__fsub_rn(hy, oy), iy);
  if (!(mn != mn)) { t_min = ocl_fmax(ocl_min(mn, mx), t_min); t_max = ocl_min(ocl_fmax(mn, mx), t_max); }
  if (t_max < t_min) { tentry = t_min; return false; }
  mn = __fmul_rn(__fsub_rn(lz, oz), iz); mx = __fmul_rn(__fsub_rn(hz, oz), iz);
  if (!(mn != mn)) { t_min = ocl_fmax(ocl_min(mn, mx), t_min); t_max = ocl_min(ocl_fmax(mn, mx), t_max); }
  tentry = t_min;
  return t_max > ocl_fmax(t_min, 0.0f);
}

// rayAabbIntersection on the slab values a = (lo - o) * inv and b = (hi - o) * inv of each
// axis (computed by the caller, possibly two boxes at a time with packed operations):
// box_ref's NaN-skipping arithmetic
__device__ __forceinline__ bool box_ref_ab(float ax, float bx, float ay, float by, float az, float bz,
                                           float& tentry) {
  float t_max = __int_as_float(0x7f800000), t_min = -__int_as_float(0x7f800000);
  if (!(ax != ax)) { t_min = ocl_fmax(ocl_min(ax, bx), t_min); t_max = ocl_min(ocl_fmax(ax, bx), t_max); }
  if (!(ay != ay)) { t_min = ocl_fmax(ocl_min(ay, by), t_min); t_max = ocl_min(ocl_fmax(ay, by), t_max); }
  if (t_max < t_min) { tentry = t_min; return false; }
  if (!(az != az)) { t_min = ocl_fmax(ocl_min(az, bz), t_min); t_max = ocl_min(ocl_fmax(az, bz), t_max); }
  tentry = t_min;
  return t_max > ocl_fmax(t_min, 0.0f);
}

// minimum and maximum of three (the three-operand PTX forms of sm_100 measured no
// faster here)
__device__ __forceinline__ float max3f(float a, float b, float c) { return fmaxf(fmaxf(a, b), c); }
__device__ __forceinline__ float min3f(float a, float b, float c) { return fminf(fminf(a, b), c); }

// The same test when every 1/d is finite: no operand can be NaN, so min/max are the
// hardware FMNMX, and the reference's result is t_max > max(t_min, 0). The distance
// cull is folded in: `cull_up` is the smallest float above the cull bound (+inf when
// there is none), so min(t_max, cull_up) > max(t_min, 0) holds exactly when the box is
// hit and its entry distance is within the bound (a negative t_min, an origin inside
// the box, is never culled). tentry, which orders the children, is max(t_min, 0) when
// `clamp` (closest-hit walks: children around the origin tie and keep their order, which
// measured fewer triangle tests) and t_min otherwise (any-hit walks: the child reaching
// furthest behind the origin first, which measured fewer box tests).
__device__ __forceinline__ bool box_fast(float ox, float oy, float oz, float ix, float iy, float iz,
                                         float lx, float hx, float ly, float hy, float lz, float hz,
                                         float cull_up, bool clamp, float& tentry) {
  const float ax = __fmul_rn(__fsub_rn(lx, ox), ix), bx = __fmul_rn(__fsub_rn(hx, ox), ix);
  const float ay = __fmul_rn(__fsub_rn(ly, oy), iy), by = __fmul_rn(__fsub_rn(hy, oy), iy);
  const float az = __fmul_rn(__fsub_rn(lz, oz), iz), bz = __fmul_rn(__fsub_rn(hz, oz), iz);
  const float t0 = max3f(fminf(ax, bx), fminf(ay, by), fminf(az, bz));
  const float t1 = min3f(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), cull_up));
  const float t0c = fmaxf(t0, 0.0f);
  tentry = clamp ? t0c : t0;
  return t1 > t0c;
}

// box_fast on slab values (see box_ref_ab)
__device__ __forceinline__ bool box_fast_ab(float ax, float bx, float ay, float by, float az, float bz,
                                            float cull_up, bool clamp, float& tentry) {
  const float t0 = max3f(fminf(ax, bx), fminf(ay, by), fminf(az, bz));
  const float t1 = min3f(fmaxf(ax, bx), fmaxf(ay, by), fminf(fmaxf(az, bz), cull_up));
  const float t0c = fmaxf(t0, 0.0f);
  tentry = clamp ? t0c : t0;
  return t1 > t0c;
}

struct TriHit {
  float t, u, v;
};

// rayTriangleIntersection (udpt.cl:326-390): Moller-Trumbore with the reference's
// operation order; the `+ 0.0f` is the w-lane product of the float4 dot (0 * 0), which
// only turns a -0 sum into +0, as the reference's four-lane dot does.
__device__ __forceinline__ bool tri_test(float ox, float oy, float oz, float dx, float dy, float dz,
                                         const float4& a, const float4& b, const float4& c, float best,
                                         int best_rank, TriHit& out) {
  // e1 = b.xyz, e2 = c.xyz, v1 = a.xyz
  const float px = __fsub_rn(__fmul_rn(dy, c.z), __fmul_rn(dz, c.y));
  const float py = __fsub_rn(__fmul_rn(dz, c.x), __fmul_rn(dx, c.z));
  const float pz = __fsub_rn(__fmul_rn(dx, c.y), __fmul_rn(dy, c.x));
  const float det = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(b.x, px), __fmul_rn(b.y, py)), __fmul_rn(b.z, pz)), 0.0f);
  const float inv_det = __frcp_rn(det);
  const float sx = __fsub_rn(ox, a.x), sy = __fsub_rn(oy, a.y), sz = __fsub_rn(oz, a.z);
  const float u = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(px, sx), __fmul_rn(py, sy)), __fmul_rn(pz, sz)), 0.0f), inv_det);
  if (u < 0.0f || u > 1.0f) return false;
  const float qx = __fsub_rn(__fmul_rn(sy, b.z), __fmul_rn(sz, b.y));
  const float qy = __fsub_rn(__fmul_rn(sz, b.x), __fmul_rn(sx, b.z));
  const float qz = __fsub_rn(__fmul_rn(sx, b.y), __fmul_rn(sy, b.x));
  const float v = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(qx, dx), __fmul_rn(qy, dy)), __fmul_rn(qz, dz)), 0.0f), inv_det);
  if (v < 0.0f || __fadd_rn(u, v) > 1.0f) return false;
  const float t = __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(c.x, qx), __fmul_rn(c.y, qy)), __fmul_rn(c.z, qz)), 0.0f), inv_det);
  if (t > 0.0f && (t < best || (t == best && __float_as_int(b.w) < best_rank))) {
    out.t = t; out.u = u; out.v = v;
    return true;
  }
  return false;
}

// Cull factor for the distance test: a child is skipped when its entry distance exceeds
// the best t by more than 2^-10 relative.
__device__ __forceinline__ float cull_bound(float best) { return best * 1.0009765625f; }
// the smallest float above cull_bound(best) (best > 0), +inf when the bound is +inf
__device__ __forceinline__ float cull_up(float best) {
  const float cb = cull_bound(best);
  return isinf(cb) ? cb : __int_as_float(__float_as_int(cb) + 1);
}

// ---- resumable walk for the persistent kernels ----
// The state of one ray's walk, so a warp can run its lanes' walks step by step and hand
// a lane a new ray as soon as its walk ends (the replenishing persistent warps of Aila
// and Laine, "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009).
struct Walk {
  const float4* nodes;   // the scene of this ray (lanes of one warp may walk different scenes)
  const float4* tris;
  float dx, dy, dz;
  float ox_, oy_, oz_, ix_, iy_, iz_;   // origin and 1/direction
  __device__ __forceinline__ float ox() const { return ox_; }
  __device__ __forceinline__ float oy() const { return oy_; }
  __device__ __forceinline__ float oz() const { return oz_; }
  __device__ __forceinline__ float ix() const { return ix_; }
  __device__ __forceinline__ float iy() const { return iy_; }
  __device__ __forceinline__ float iz() const { return iz_; }
  // each component twice, the operand of the packed box tests (built where it is used:
  // a register pair per component would hold six more registers through the walk)
  __device__ __forceinline__ f32x2 ox2() const { return pk2(ox_, ox_); }
  __device__ __forceinline__ f32x2 oy2() const { return pk2(oy_, oy_); }
  __device__ __forceinline__ f32x2 oz2() const { return pk2(oz_, oz_); }
  __device__ __forceinline__ f32x2 ix2() const { return pk2(ix_, ix_); }
  __device__ __forceinline__ f32x2 iy2() const { return pk2(iy_, iy_); }
  __device__ __forceinline__ f32x2 iz2() const { return pk2(iz_, iz_); }
  float best, bu, bv;
  float best_up;         // cull_up(best)
  int best_tri, best_rank;
  int link, sp;
  float link_t;          // entry distance of the subtree `link` (checked again before it is opened)
  bool exact;
};

__device__ __forceinline__ void walk_begin(const DevScene& sc, const RayIn& r, Walk& w) {
  w.nodes = sc.nodes;
  w.tris = sc.tris;

  w.dx = r.dx; w.dy = r.dy; w.dz = r.dz;
  const float ix = __frcp_rn(r.dx), iy = __frcp_rn(r.dy), iz = __frcp_rn(r.dz);
  w.exact = isinf(ix) || isinf(iy) || isinf(iz);
  w.ox_ = r.ox; w.oy_ = r.oy; w.oz_ = r.oz;
  w.ix_ = ix; w.iy_ = iy; w.iz_ = iz;
  w.best = r.tmax; w.bu = 0.0f; w.bv = 0.0f;
  w.best_up = cull_up(r.tmax);
  w.best_tri = -1; w.best_rank = -1;
  w.sp = 0;
  w.link = sc.root_link;
  w.link_t = -__int_as_float(0x7f800000);
  if (w.link != LINK_NONE && sc.root_test) {
    float te;
    const bool h = w.exact ? box_ref(w.ox(), w.oy(), w.oz(), w.ix(), w.iy(), w.iz(), sc.root_lo.x, sc.root_hi.x, sc.root_lo.y,
                                     sc.root_hi.y, sc.root_lo.z, sc.root_hi.z, te)
                           : box_fast(w.ox(), w.oy(), w.oz(), w.ix(), w.iy(), w.iz(), sc.root_lo.x, sc.root_hi.x, sc.root_lo.y,
                                      sc.root_hi.y, sc.root_lo.z, sc.root_hi.z, __int_as_float(0x7f800000), false, te);
    if (!h) w.link = LINK_NONE;
  }
}

// Triangles of one leaf (the reference's vert_list run, yc_scene.h); returns true when
// an any-hit walk (any = true) has found its hit.
__device__ __forceinline__ bool walk_leaf(Walk& w, int link, WalkCount& wc, bool any) {
  const int enc = ~link;
  const int count = enc & 15;
  const float4* tp = w.tris + 3 * (size_t)(enc >> 4);
  for (int k = 0; k < count; ++k) {
    ++wc.tris;
    const float4 a = __ldg(tp + 3 * k + 0);
    const float4 b = __ldg(tp + 3 * k + 1);
    const float4 c = __ldg(tp + 3 * k + 2);
    TriHit th;
    if (tri_test(w.ox(), w.oy(), w.oz(), w.dx, w.dy, w.dz, a, b, c, w.best, w.best_rank, th)) {
      w.best = th.t;
      w.best_up = cull_up(th.t);
      w.bu = th.u;
      w.bv = th.v;
      w.best_tri = __float_as_int(a.w);
      w.best_rank = __float_as_int(b.w);
      if (any) return true;
    }
  }
  return false;
}

// A walk's stack of (subtree link, entry distance) pairs, at most `cap` deep: entries
// [0, n_smem) in this thread's column of the block's shared memory (stride: the block
// size), deeper ones in its column of a global spill area (stride: the grid's threads).
// A short shared part leaves more of the SM's unified L1 and shared memory to the node
// and triangle fetches; n_smem == cap (g unused) keeps the whole stack in shared memory.
struct WalkStack {
  int* s;
  int* g;
  int stride, gstride, n_smem, cap;
  __device__ __forceinline__ void put(int i, int link, float t) const {
    if (i < n_smem) {
      s[(2 * i) * stride] = link;
      s[(2 * i + 1) * stride] = __float_as_int(t);
    } else {
      const size_t j = (size_t)(2 * (i - n_smem)) * gstride;
      g[j] = link;
      g[j + gstride] = __float_as_int(t);
    }
  }
  __device__ __forceinline__ float t_at(int i) const {
    return __int_as_float(i < n_smem ? s[(2 * i + 1) * stride] : g[(size_t)(2 * (i - n_smem) + 1) * gstride]);
  }
  __device__ __forceinline__ int link_at(int i) const {
    return i < n_smem ? s[(2 * i) * stride] : g[(size_t)(2 * (i - n_smem)) * gstride];
  }
};

// pops the next subtree whose entry is still within reach (LINK_NONE: the walk ends)
__device__ __forceinline__ int walk_pop(Walk& w, const WalkStack& st) {
  while (w.sp > 0) {
    --w.sp;
    const float te = st.t_at(w.sp);
    if (!(te > cull_bound(w.best))) {
      w.link_t = te;
      return st.link_at(w.sp);
    }
  }
  return LINK_NONE;
}

// the pending subtree, unless a hit found since it was chosen puts it out of reach
__device__ __forceinline__ int walk_recheck(Walk& w, int link, const WalkStack& st) {
  if (link != LINK_NONE && w.link_t > cull_bound(w.best)) return walk_pop(w, st);
  return link;
}

// One interior node of the two-child layout: returns the next node (the nearer child
// hit, the other one pushed), or the next subtree popped from the stack when neither
// child is hit. LINK_NONE: the walk is over (or the stack bound was reached).
__device__ __forceinline__ int visit2(Walk& w, bool any, int link, const WalkStack& st, WalkCount& wc,
                                      bool& overflow) {
  const float4* nd = w.nodes + 4 * (size_t)link;
  const ulonglong2 nx = __ldg(reinterpret_cast<const ulonglong2*>(nd + 0));   // (lo pair, hi pair)
  const ulonglong2 ny = __ldg(reinterpret_cast<const ulonglong2*>(nd + 1));
  const ulonglong2 nz = __ldg(reinterpret_cast<const ulonglong2*>(nd + 2));
  const int2 n3 = __ldg(reinterpret_cast<const int2*>(nd + 3));
  wc.nodes += 2;
  // (lo - o) * inv and (hi - o) * inv of both children, two packed operations per bound
  float ax0, ax1, bx0, bx1, ay0, ay1, by0, by1, az0, az1, bz0, bz1;
  up2(mul2(sub2(nx.x, w.ox2()), w.ix2()), ax0, ax1);
  up2(mul2(sub2(nx.y, w.ox2()), w.ix2()), bx0, bx1);
  up2(mul2(sub2(ny.x, w.oy2()), w.iy2()), ay0, ay1);
  up2(mul2(sub2(ny.y, w.oy2()), w.iy2()), by0, by1);
  up2(mul2(sub2(nz.x, w.oz2()), w.iz2()), az0, az1);
  up2(mul2(sub2(nz.y, w.oz2()), w.iz2()), bz0, bz1);
  float t0, t1;
  bool h0, h1;
  if (!w.exact) {   // hit and within the cull bound
    h0 = box_fast_ab(ax0, bx0, ay0, by0, az0, bz0, w.best_up, !any, t0);
    h1 = box_fast_ab(ax1, bx1, ay1, by1, az1, bz1, w.best_up, !any, t1);
  } else {
    h0 = box_ref_ab(ax0, bx0, ay0, by0, az0, bz0, t0);
    h1 = box_ref_ab(ax1, bx1, ay1, by1, az1, bz1, t1);
    const float cb = cull_bound(w.best);
    h0 = h0 && !(t0 > cb);
    h1 = h1 && !(t1 > cb);
  }
  h0 = h0 && n3.x != LINK_NONE;
  h1 = h1 && n3.y != LINK_NONE;
  if (h0 && h1) {
    const bool swap = t1 < t0;
    if (w.sp >= st.cap) { overflow = true; w.sp = 0; return LINK_NONE; }
    st.put(w.sp, swap ? n3.x : n3.y, swap ? t0 : t1);
    ++w.sp;
    w.link_t = swap ? t1 : t0;
    return swap ? n3.y : n3.x;
  }
  if (h0) { w.link_t = t0; return n3.x; }
  if (h1) { w.link_t = t1; return n3.y; }
  return walk_pop(w, st);
}

// (t, link) compare-exchange: the smaller entry distance first
__device__ __forceinline__ void cx(float& ta, int& la, float& tb, int& lb) {
  if (tb < ta) {
    const float t = ta; ta = tb; tb = t;
    const int l = la; la = lb; lb = l;
  }
}

// One interior node of the four-child layout (yc_scene.h, wide nodes): the four child
// boxes are tested with the reference's slab arithmetic, the hits sorted by entry
// distance, the nearest returned and the others pushed farthest first.
__device__ __forceinline__ int visit4(Walk& w, bool any, int link, const WalkStack& st, WalkCount& wc,
                                      bool& overflow) {
  const float INF = __int_as_float(0x7f800000);
  const float4* nd = w.nodes + 8 * (size_t)link;
  const float4 lx = __ldg(nd + 0), hx = __ldg(nd + 1);
  const float4 ly = __ldg(nd + 2), hy = __ldg(nd + 3);
  const float4 lz = __ldg(nd + 4), hz = __ldg(nd + 5);
  const int4 ln = __ldg(reinterpret_cast<const int4*>(nd + 6));
  wc.nodes += 4;
  const float cb = cull_bound(w.best);
  float t[4];
  int l[4];
  const float clx[4] = {lx.x, lx.y, lx.z, lx.w}, chx[4] = {hx.x, hx.y, hx.z, hx.w};
  const float cly[4] = {ly.x, ly.y, ly.z, ly.w}, chy[4] = {hy.x, hy.y, hy.z, hy.w};
  const float clz[4] = {lz.x, lz.y, lz.z, lz.w}, chz[4] = {hz.x, hz.y, hz.z, hz.w};
  const int cl[4] = {ln.x, ln.y, ln.z, ln.w};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float te;
    bool h = !w.exact ? box_fast(w.ox(), w.oy(), w.oz(), w.ix(), w.iy(), w.iz(), clx[c], chx[c], cly[c], chy[c], clz[c], chz[c],
                                 w.best_up, !any, te)
                      : box_ref(w.ox(), w.oy(), w.oz(), w.ix(), w.iy(), w.iz(), clx[c], chx[c], cly[c], chy[c], clz[c], chz[c], te);
    h = h && cl[c] != LINK_NONE && !(te > cb);
    t[c] = h ? te : INF;
    l[c] = h ? cl[c] : LINK_NONE;
  }
  // sorting network for four entries; misses (t = inf, LINK_NONE) end up last
  cx(t[0], l[0], t[1], l[1]);
  cx(t[2], l[2], t[3], l[3]);
  cx(t[0], l[0], t[2], l[2]);
  cx(t[1], l[1], t[3], l[3]);
  cx(t[1], l[1], t[2], l[2]);
  if (l[0] == LINK_NONE) return walk_pop(w, st);
  const int extra = (l[1] != LINK_NONE) + (l[2] != LINK_NONE) + (l[3] != LINK_NONE);
  if (w.sp + extra > st.cap) { overflow = true; w.sp = 0; return LINK_NONE; }
#pragma unroll
  for (int c = 3; c >= 1; --c) {
    if (l[c] != LINK_NONE) {
      st.put(w.sp, l[c], t[c]);
      ++w.sp;
    }
  }
  w.link_t = t[0];
  return l[0];
}

// One step of the walk, the while-while loop with postponed leaves of Aila and Laine
// ("Understanding the Efficiency of Ray Traversal on GPUs", 2009, and its 2012
// addendum): interior nodes are visited until every lane of the warp still walking has
// reached a leaf; a lane that meets its first leaf keeps it aside and goes on with the
// next subtree, so the lanes test triangles together instead of one after another.
// Returns true when the walk has ended (w.link == LINK_NONE); `overflow` is set when the
// stack bound was reached (the walk then ends early). Leaves are kept aside before the
// hits inside them lower the culling distance, so the walk may open a few more boxes
// than a leaf-first order would; it never skips one that can hold a closer hit.
// `any` selects the any-hit walk (it stops at the first hit); callers that know the kind
// at compile time use walk_step<ANY, WIDE>, the mixed trace loop passes it per lane.
template <bool WIDE>
__device__ __forceinline__ bool walk_step_k(Walk& w, bool any, const WalkStack& st, WalkCount& wc, bool& overflow) {
  // (an any-hit walk keeps its segment length until it stops: nothing to check again)
  int link = any ? w.link : walk_recheck(w, w.link, st);
  int leaf = LINK_NONE;
  while (link >= 0 && link != LINK_NONE) {
    link = WIDE ? visit4(w, any, link, st, wc, overflow) : visit2(w, any, link, st, wc, overflow);
    if (link < 0 && link != LINK_NONE && leaf == LINK_NONE) {
      leaf = link;
      link = walk_pop(w, st);
    }
    if (!__any_sync(__activemask(), leaf == LINK_NONE)) break;
  }
  if (leaf == LINK_NONE && link < 0 && link != LINK_NONE) {
    leaf = link;
    link = walk_pop(w, st);
  }
  while (leaf != LINK_NONE) {
    if (walk_leaf(w, leaf, wc, any)) { w.sp = 0; w.link = LINK_NONE; return true; }
    leaf = LINK_NONE;
    if (!any) link = walk_recheck(w, link, st);
    if (link < 0 && link != LINK_NONE) {   // a second leaf met by the speculative walk
      leaf = link;
      link = walk_pop(w, st);
    }
  }
  w.link = link;
  return link == LINK_NONE;
}

template <bool ANY, bool WIDE>
__device__ __forceinline__ bool walk_step(Walk& w, const WalkStack& st, WalkCount& wc, bool& overflow) {
  return walk_step_k<WIDE>(w, ANY, st, wc, overflow);
}

}  // namespace yc
