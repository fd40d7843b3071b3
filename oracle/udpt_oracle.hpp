// udpt_oracle.hpp -- CPU restatement of Yune's unidirectional path tracer.
//
// TEST INFRASTRUCTURE. This is the checker for the CUDA core: only tests, the smoke
// check and the benchmark's CPU-baseline leg use it. It is never linked into the
// product library.
//
// It follows kernels/legacy/udpt.cl function by function (line numbers cited on each
// function) and adds three switches the benchmark configurations need:
//   mis            the MIS branch of evaluateDirectLighting (udpt.cl:9, 570-608)
//   rr_threshold   RR_THRESHOLD (udpt.cl:6; 6 as shipped)
//   max_depth      bound of the GI loop (udpt.cl:463; 100000 as shipped)
//   brdf_model     0: Lambert of udpt.cl:621-622; 1: Oren-Nayar whenever the diffuse
//                  lobe is taken with probability 1, as kernels/legacy/
//                  udpt-primitives.cl:673-725 does
//   mis_lobe_fix   0 reproduces udpt.cl exactly: with MIS on, a shadow ray that is
//                  blocked leaves brdf_prob = 0 and a BRDF ray that then reaches the
//                  light divides by it (udpt.cl:540, 559, 604). 1 draws the lobe at
//                  that point instead, so the estimate stays finite.
//   heap_size      capacity of the breadth-first candidate queue (HEAP_SIZE, udpt.cl:8);
//                  the traversal stops when it fills, as the reference does, and the
//                  overflow is reported.
// The light sources are a buffer instead of the __constant array of udpt.cl:97-106.
#pragma once

#include <cstdint>
#include <vector>

#include "../include/yune_types.h"
#include "oracle_math.hpp"

namespace orc {

struct Config {
  int mis = 0;
  int rr_threshold = 6;
  int max_depth = 100000;
  int brdf_model = 0;
  int mis_lobe_fix = 0;
  int heap_size = 1500;
  int gi_check = 1;
};

struct Counters {
  uint64_t rays = 0;          // traceRay calls (every kind)
  uint64_t primary = 0, extension = 0, shadow = 0, mis = 0;
  uint64_t heap_overflow = 0;  // traversals cut short by a full queue
};

template <class R>
struct Scene {
  const yc_triangle* tris = nullptr;
  int n_tri = 0;
  const yc_material* mats = nullptr;
  int n_mat = 0;
  const yc_bvh_node* nodes = nullptr;
  int n_node = 0;
  const yc_quad_light* lights = nullptr;
  int n_light = 0;
};

template <class R> inline V4<R> ld(const yc_float4& f) { return V4<R>{(R)f.x, (R)f.y, (R)f.z, (R)f.w}; }

template <class R> struct Ray { V4<R> origin, dir; R length; bool is_shadow; };
template <class R> struct Hit { int tri = -1, light = -1; V4<R> hit_point{0, 0, 0, 1}; V4<R> normal{0, 0, 0, 0}; };

template <class R>
struct Tracer {
  using O = Ops<R>;
  const Scene<R>& sc;
  const Config& cfg;
  Counters& cnt;
  std::vector<int> queue;

  static constexpr float PI_F = 3.14159265359f;
  static constexpr float INV_PI_F = 0.31830988618f;
  static constexpr float EPS_F = 0.0001f;

  Tracer(const Scene<R>& s, const Config& c, Counters& k) : sc(s), cfg(c), cnt(k), queue(c.heap_size > 0 ? c.heap_size + 1 : 2) {}

  // Optional record of the rays that walk a BVH (measurement of the traversal's
  // algorithmic work, replayed on the host): 8 floats each, origin xyz, direction xyz,
  // segment length and kind (0 camera ray, 1 extension ray: closest hit; 2 shadow ray,
  // 3 MIS ray: any hit). A shadow ray that a light closes first, and a MIS ray whose
  // closest light is not the sampled one, settle without a walk (as the CUDA core settles
  // them) and are not recorded. rec_kind is set by the caller of trace() and consumed.
  std::vector<float>* rec = nullptr;
  int rec_kind = -1, rec_light = -1;

  static R draw(uint32_t& seed) { seed = ym::xor_shift(seed); return O::u01(seed); }

  // rayAabbIntersection, udpt.cl:392-431
  bool ray_aabb(const Ray<R>& ray, const yc_aabb& bb) const {
    R t_max = (R)INFINITY, t_min = -(R)INFINITY;
    const R inv[3] = {O::div(R(1), ray.dir.x), O::div(R(1), ray.dir.y), O::div(R(1), ray.dir.z)};
    const R o[3] = {ray.origin.x, ray.origin.y, ray.origin.z};
    const R lo[3] = {(R)bb.p_min.x, (R)bb.p_min.y, (R)bb.p_min.z};
    const R hi[3] = {(R)bb.p_max.x, (R)bb.p_max.y, (R)bb.p_max.z};
    for (int k = 0; k < 3; ++k) {
      const R mn = O::mul(O::sub(lo[k], o[k]), inv[k]);
      const R mx = O::mul(O::sub(hi[k], o[k]), inv[k]);
      if (!O::isnan(mn)) {
        t_min = O::fmax(O::min(mn, mx), t_min);
        t_max = O::min(O::fmax(mn, mx), t_max);
      }
      if (k == 1 && t_max < t_min) return false;
    }
    return t_max > O::fmax(t_min, R(0));
  }

  // rayTriangleIntersection, udpt.cl:326-390 (Moller-Trumbore, no culling)
  bool ray_tri(Ray<R>& ray, Hit<R>& hit, int idx) const {
    const yc_triangle& T = sc.tris[idx];
    const V4<R> v1 = ld<R>(T.v1);
    const V4<R> e1 = ld<R>(T.v2) - v1;
    const V4<R> e2 = ld<R>(T.v3) - v1;
    const V4<R> pvec = cross(ray.dir, e2);
    const R det = dot(e1, pvec);
    const R inv_det = O::div(R(1), det);
    const V4<R> dist = ray.origin - v1;
    const R u = O::mul(dot(pvec, dist), inv_det);
    if (u < 0.0 || u > R(1)) return false;
    const V4<R> qvec = cross(dist, e1);
    const R v = O::mul(dot(qvec, ray.dir), inv_det);
    if (v < 0.0 || O::add(u, v) > 1.0) return false;
    const R t = O::mul(dot(e2, qvec), inv_det);
    if (t > 0 && t < ray.length) {
      ray.length = t;
      const V4<R> N1 = normalize(ld<R>(T.vn1));
      const V4<R> N2 = normalize(ld<R>(T.vn2));
      const V4<R> N3 = normalize(ld<R>(T.vn3));
      const R w = O::sub(O::sub(R(1), u), v);
      hit.hit_point = ray.origin + ray.dir * t;
      hit.normal = normalize((N1 * w + N2 * u) + N3 * v);
      hit.tri = idx;
      hit.light = -1;
      return true;
    }
    return false;
  }

  // traverseBVH, udpt.cl:288-324: breadth-first queue, no ordering, no distance cull.
  // The loop checks the length only before a node's two children are pushed, so when
  // the last free entry takes both, the second lands one past the end (udpt.cl:298,315-
  // 319); the loop stops there and never reads it. The queue has that one spare entry.
  bool traverse(Ray<R>& ray, Hit<R>& hit) {
    const yc_bvh_node* bvh = sc.nodes;
    bool intersect = false;
    if (!ray_aabb(ray, bvh[0].aabb)) return false;
    int len = 1;
    queue[0] = 0;
    const int cap = cfg.heap_size;
    int i = 0;
    for (; i < len && len < cap; ++i) {
      const yc_bvh_node& n = bvh[queue[i]];
      const float c_idx = (float)n.child_idx;
      if (c_idx == -1 && n.vert_len > 0) {
        for (int j = 0; j < n.vert_len; ++j) {
          intersect |= ray_tri(ray, hit, n.vert_list[j]);
          if (ray.is_shadow && intersect) return true;
        }
        continue;
      }
      for (int j = (int)c_idx; j < c_idx + 2; ++j) {
        if ((bvh[j].vert_len > 0 || bvh[j].child_idx > 0) && ray_aabb(ray, bvh[j].aabb)) {
          queue[len] = j;
          len++;
        }
      }
    }
    if (len >= cap && i < len) cnt.heap_overflow++;
    return intersect;
  }

  // traceRay, udpt.cl:240-286
  bool trace(Ray<R>& ray, Hit<R>& hit) {
    cnt.rays++;
    bool flag = false;
    for (int i = 0; i < sc.n_light; ++i) {
      const yc_quad_light& L = sc.lights[i];
      const V4<R> nrm = ld<R>(L.normal);
      const R DdotN = dot(ray.dir, nrm);
      if ((double)O::fabs(DdotN) > 0.0001) {
        const V4<R> pos = ld<R>(L.pos);
        const R t = O::div(dot(nrm, pos - ray.origin), DdotN);
        if (t > 0.0 && t < ray.length) {
          V4<R> temp = ray.origin + ray.dir * t;
          temp = temp - pos;
          const V4<R> el = ld<R>(L.edge_l), ew = ld<R>(L.edge_w);
          R proj1 = dot(temp, el);
          R proj2 = dot(temp, ew);
          const R la = length(el), lb = length(ew);
          proj1 = O::div(proj1, la);
          proj2 = O::div(proj2, lb);
          if ((proj1 >= 0.0 && proj2 >= 0.0) && (proj1 <= la && proj2 <= lb)) {
            ray.length = t;
            hit.hit_point = ray.origin + ray.dir * t;
            hit.light = i;
            hit.tri = -1;
            flag = true;
          }
        }
      }
    }
    if (rec && rec_kind >= 0 && sc.n_node > 0) {
      const bool walked = rec_kind < 2 || (rec_kind == 2 && !flag) || (rec_kind == 3 && flag && hit.light == rec_light);
      if (walked) {
        const float r8[8] = {(float)ray.origin.x, (float)ray.origin.y, (float)ray.origin.z, (float)ray.dir.x,
                             (float)ray.dir.y, (float)ray.dir.z, (float)ray.length, (float)rec_kind};
        rec->insert(rec->end(), r8, r8 + 8);
      }
    }
    rec_kind = -1;
    if (sc.n_node > 0) flag |= traverse(ray, hit);
    else
      for (int i = 0; i < sc.n_tri; ++i) flag |= ray_tri(ray, hit, i);
    return flag;
  }

  const yc_material& mat_of(const Hit<R>& h) const { return sc.mats[sc.tris[h.tri].matID]; }

  static void frame(V4<R> Nz, V4<R>& Nx, V4<R>& Ny) {
    if (O::fabs(Nz.y) > O::fabs(Nz.z)) Nx = V4<R>{Nz.y, -Nz.x, R(0), R(0)};
    else Nx = V4<R>{Nz.z, R(0), -Nz.x, R(0)};
    Nx = normalize(Nx);
    Ny = normalize(cross(Nz, Nx));
  }

  // reflect, udpt.cl:949-961
  static V4<R> reflect(V4<R> w_i, const Hit<R>& h) {
    V4<R> n = h.normal;
    if (dot(w_i, n) < 0) n = n * R(-1);
    V4<R> r = (O::mul(R(2), dot(w_i, n))) * n - w_i;
    return normalize(r);
  }

  // refract, udpt.cl:963-990
  V4<R> refract(V4<R> w_i, const Hit<R>& h) const {
    V4<R> n = h.normal;
    R n1, n2;
    const yc_material& m = mat_of(h);
    if (dot(w_i, n) < 0) { n1 = (R)m.n; n2 = R(1); n = n * R(-1); }
    else { n1 = R(1); n2 = (R)m.n; }
    const V4<R> wt_perp = O::div(n1, n2) * (dot(w_i, n) * n - w_i);
    const R lp = length(wt_perp);
    const V4<R> wt_par = O::sqrt(O::sub(R(1), O::mul(lp, lp))) * (-n);
    return normalize(wt_perp + wt_par);
  }

  // evalFresnelReflectance, udpt.cl:992-1031
  R fresnel(V4<R> w_i, const Hit<R>& h, R& ior_factor) const {
    V4<R> n = h.normal;
    R n1, n2;
    const yc_material& m = mat_of(h);
    if (dot(w_i, n) < 0) { n1 = (R)m.n; n2 = R(1); n = n * R(-1); }
    else { n1 = R(1); n2 = (R)m.n; }
    const R cosI = dot(w_i, n);
    const R sinI = O::sqrt(O::sub(R(1), O::mul(cosI, cosI)));
    const R sinT = O::div(O::mul(n1, sinI), n2);
    const R cosT = O::sqrt(O::sub(R(1), O::mul(sinT, sinT)));
    if (sinT >= R(1) && n1 > n2) return R(1);
    const R r0 = O::div(O::add(O::add((R)m.ks.x, (R)m.ks.y), (R)m.ks.z), R(3));
    ior_factor = O::div(O::mul(n2, n2), O::mul(n1, n1));
    const R c = (n1 > n2) ? cosI : cosT;
    return O::add(r0, O::mul(O::sub(R(1), r0), O::sub(R(1), O::pow(c, R(5)))));
  }

  // sampleFresnelIncidence, udpt.cl:912-947
  void sample_fresnel(Ray<R>& ray, const Hit<R>& h, V4<R> w_i, R& ior_factor, uint32_t& seed) const {
    const yc_material& m = mat_of(h);
    if (m.is_transmissive) {
      const R pdf = fresnel(w_i, h, ior_factor);
      if (pdf == 1.0) { ray.dir = reflect(w_i, h); ior_factor = R(1); }
      else {
        seed = ym::xor_shift(seed);
        const R r = O::u01(seed);
        if (r < pdf) { ray.dir = reflect(w_i, h); ior_factor = R(1); }
        else ray.dir = refract(w_i, h);
      }
    } else {
      ior_factor = R(1);
      ray.dir = reflect(w_i, h);
    }
    ray.length = (R)INFINITY;
    ray.is_shadow = false;
    ray.origin = h.hit_point + ray.dir * (R)EPS_F;
  }

  // rows (Nx.k, Ny.k, Nz.k, p.k) of the normal-to-world matrix applied to (x, y, z, 0)
  static V4<R> to_world(V4<R> Nx, V4<R> Ny, V4<R> Nz, V4<R> p, V4<R> d) {
    V4<R> out;
    out.x = dot(V4<R>{Nx.x, Ny.x, Nz.x, p.x}, d);
    out.y = dot(V4<R>{Nx.y, Ny.y, Nz.y, p.y}, d);
    out.z = dot(V4<R>{Nx.z, Ny.z, Nz.z, p.z}, d);
    out.w = R(0);
    return normalize(out);
  }

  // phongSampleHemisphere, udpt.cl:700-771
  void sample_phong(Ray<R>& ray, R& pdf, V4<R> w_i, const Hit<R>& h, uint32_t& seed) const {
    V4<R> Nz = normalize(reflect(w_i, h)), Nx, Ny;
    frame(Nz, Nx, Ny);
    const R r1 = draw(seed);
    const R r2 = draw(seed);
    const yc_material& m = mat_of(h);
    const int pe = (int)((R)m.px + (R)m.py);
    const R phi = O::mul(O::mul(R(2), (R)PI_F), r2);
    const R costheta = O::pow(r1, O::div(R(1), (R)(pe + 1)));
    R sintheta = O::sub(R(1), O::pow(r1, O::div(R(2), (R)(pe + 1))));
    sintheta = O::sqrt(sintheta);
    const V4<R> d{O::mul(sintheta, O::cos(phi)), O::mul(sintheta, O::sin(phi)), costheta, R(0)};
    ray.dir = to_world(Nx, Ny, Nz, h.hit_point, d);
    ray.origin = h.hit_point + ray.dir * (R)EPS_F;
    ray.is_shadow = false;
    ray.length = (R)INFINITY;
    if (dot(ray.dir, h.normal) < 0) pdf = R(0);
    else pdf = (R)((double)(pe + 1) * 0.5 * (double)INV_PI_F * (double)O::pow(costheta, (R)pe));
  }

  // cosineWeightedHemisphere, udpt.cl:843-910
  void sample_cosine(Ray<R>& ray, R& pdf, const Hit<R>& h, uint32_t& seed) const {
    V4<R> Nz = h.normal, Nx, Ny;
    frame(Nz, Nx, Ny);
    const R r1 = draw(seed);
    const R r2 = draw(seed);
    const R phi = O::mul(O::mul(R(2), (R)PI_F), r2);
    const R sinT = O::sqrt(r1);
    const R z = O::sqrt(O::sub(R(1), r1));
    const V4<R> d{O::mul(sinT, O::cos(phi)), O::mul(sinT, O::sin(phi)), z, R(0)};
    ray.dir = to_world(Nx, Ny, Nz, h.hit_point, d);
    ray.origin = h.hit_point + ray.dir * (R)EPS_F;
    ray.is_shadow = false;
    ray.length = (R)INFINITY;
    pdf = O::mul(z, (R)INV_PI_F);
  }

  // calcPhongPDF, udpt.cl:1033-1045
  R phong_pdf(V4<R> w_i, V4<R> w_o, const Hit<R>& h) const {
    V4<R> rd = O::mul(R(2), dot(w_o, h.normal)) * h.normal - w_o;
    rd = normalize(rd);
    const R costheta = O::fmax(R(0), O::cos(dot(rd, w_i)));
    const yc_material& m = mat_of(h);
    const R pe = O::add((R)m.px, (R)m.py);
    return (R)((double)O::add(pe, R(1)) * 0.5 * (double)INV_PI_F * (double)O::pow(costheta, pe));
  }
  // calcCosPDF, udpt.cl:1047-1050
  static R cos_pdf(V4<R> w_i, V4<R> n) { return O::mul(O::fmax(dot(w_i, n), R(0)), (R)INV_PI_F); }

  // sampleGlossyPdf, udpt.cl:1062-1119
  bool sample_glossy(const Hit<R>& h, uint32_t& seed, R& prob) {
    const R r = draw(seed);
    const yc_material& m = mat_of(h);
    const V4<R> ks = ld<R>(m.ks), kd = ld<R>(m.kd);
    if (length3(ks) == R(0)) { prob = R(1); return false; }
    if (length3(kd) == R(0) || O::add(O::add(kd.x, kd.y), kd.z) == R(0)) { prob = R(1); return true; }
    const V4<R> sum = ks + kd;
    const R mx = O::max(sum.x, O::max(sum.y, sum.z));
    R pd, ps;
    if (mx == sum.x) { pd = kd.x; ps = ks.x; }
    else if (mx == sum.y) { pd = kd.y; ps = ks.y; }
    else { pd = kd.z; ps = ks.z; }
    if (r < pd) { prob = pd; return false; }
    if (r < O::add(pd, ps) && r >= pd) { prob = ps; return true; }
    prob = R(0);
    return false;
  }

  // toShadingSpace and the trig helpers, udpt-primitives.cl:1147-1210
  static V4<R> to_shading(V4<R> w, const Hit<R>& h) {
    V4<R> Nz = h.normal, Nx, Ny;
    frame(Nz, Nx, Ny);
    const V4<R> r1{Nx.x, Nx.y, Nx.z, dot(h.hit_point, Nx)};
    const V4<R> r2{Ny.x, Ny.y, Ny.z, dot(h.hit_point, Ny)};
    const V4<R> r3{Nz.x, Nz.y, Nz.z, dot(h.hit_point, Nz)};
    const V4<R> r4{R(0), R(0), R(0), R(1)};
    return V4<R>{dot(r1, w), dot(r2, w), dot(r3, w), dot(r4, w)};
  }
  static R sin_theta(V4<R> w) { return O::sqrt(O::sub(R(1), O::mul(w.z, w.z))); }
  static R cos_phi(V4<R> w) {
    const R st = sin_theta(w);
    if (st <= (R)EPS_F && st >= -(R)EPS_F) return R(0);
    return O::fmin(O::fmax(O::div(w.x, st), R(-1)), R(1));
  }
  static R sin_phi(V4<R> w) {
    const R st = sin_theta(w);
    if (st <= (R)EPS_F && st >= -(R)EPS_F) return R(0);
    return O::fmin(O::fmax(O::div(w.y, st), R(-1)), R(1));
  }
  // OrenNayarBRDF, udpt-primitives.cl:696-725 (alpha_x holds sigma^2)
  V4<R> oren_nayar(V4<R> w_i, V4<R> w_o, const Hit<R>& h) const {
    w_i = to_shading(w_i, h);
    w_o = to_shading(w_o, h);
    const yc_material& m = mat_of(h);
    R costerm = R(0);
    if (sin_theta(w_i) >= (R)EPS_F && sin_theta(w_o) >= (R)EPS_F)
      costerm = O::fmax(R(0), O::add(O::mul(cos_phi(w_i), cos_phi(w_o)), O::mul(sin_phi(w_i), sin_phi(w_o))));
    R sin_alpha, tan_beta;
    if (O::fabs(w_i.z) < O::fabs(w_o.z)) { sin_alpha = sin_theta(w_i); tan_beta = O::div(sin_theta(w_o), O::fabs(w_o.z)); }
    else { sin_alpha = sin_theta(w_o); tan_beta = O::div(sin_theta(w_i), O::fabs(w_i.z)); }
    const R s2 = (R)m.alpha_x;
    const R A = (R)(1 - ((double)s2 / (2 * ((double)s2 + 0.33))));
    const R B = (R)(0.45 * (double)s2 / ((double)s2 + 0.09));
    return (ld<R>(m.kd) * (R)INV_PI_F) * O::add(A, O::mul(B, O::mul(O::mul(costerm, sin_alpha), tan_beta)));
  }

  // evaluateBRDF, udpt.cl:611-630 (+ udpt-primitives.cl:673-694 when brdf_model = 1)
  V4<R> brdf(V4<R> w_i, V4<R> w_o, const Hit<R>& h, bool glossy, R rr_prob) const {
    const V4<R> refl = normalize(reflect(w_i, h));
    const yc_material& m = mat_of(h);
    if (!glossy) {
      if (cfg.brdf_model == 1 && rr_prob == R(1)) return oren_nayar(w_i, w_o, h);
      return (ld<R>(m.kd) * (R)INV_PI_F) / rr_prob;
    }
    const R cos_alpha = O::pow(O::fmax(dot(w_o, refl), R(0)), O::add((R)m.px, (R)m.py));
    const int pe = (int)((R)m.px + (R)m.py);
    return ((((ld<R>(m.ks) * cos_alpha) * (R)(pe + 2)) * (R)INV_PI_F) * R(0.5f)) / rr_prob;
  }

  // sampleLights, udpt.cl:632-698. Returns -1 when no light is picked (also when the
  // CDF walk falls off the end, which udpt.cl leaves undefined).
  int sample_lights(const Hit<R>& h, R& light_pdf, V4<R>& w_i, uint32_t& seed) {
    const int n = sc.n_light;
    R sum = R(0);
    R weights[16];
    V4<R> w_is[16];
    for (int i = 0; i < n; ++i) {
      const yc_quad_light& L = sc.lights[i];
      const R r1 = draw(seed);
      const R r2 = draw(seed);
      V4<R> t = ((ld<R>(L.pos) + r1 * ld<R>(L.edge_l)) + r2 * ld<R>(L.edge_w)) - h.hit_point;
      const R distance = dot(t, t);
      w_is[i] = t;
      t = normalize(t);
      const V4<R> ln = ld<R>(L.normal);
      const R cf = O::mul(O::max(dot(t, h.normal), R(0)), O::max(dot(-t, ln), R(0)));
      if (cf <= 0.0) { weights[i] = R(0); continue; }
      const R area = O::mul(length(ld<R>(L.edge_l)), length(ld<R>(L.edge_w)));
      if (n == 1) {
        w_i = w_is[i];
        light_pdf = O::div(R(1), area);
        light_pdf = O::mul(light_pdf, O::div(distance, O::fmax(dot(-t, ln), R(0))));
        return i;
      }
      weights[i] = O::div(O::mul(O::mul(length(ld<R>(L.ke)), cf), area), distance);
      sum = O::add(sum, weights[i]);
    }
    if (sum == R(0)) return -1;
    const R r1 = draw(seed);
    R cum = R(0);
    for (int i = 0; i < n; ++i) {
      const R wgt = O::div(weights[i], sum);
      if (r1 >= cum && r1 < O::add(cum, wgt)) {
        const yc_quad_light& L = sc.lights[i];
        const R area = O::mul(length(ld<R>(L.edge_l)), length(ld<R>(L.edge_w)));
        w_i = w_is[i];
        light_pdf = O::div(wgt, area);
        light_pdf = O::mul(light_pdf, O::div(dot(w_i, w_i), O::fmax(dot(-normalize(w_i), ld<R>(L.normal)), R(0))));
        return i;
      }
      cum = O::add(cum, wgt);
    }
    return -1;
  }

  // evaluateDirectLighting, udpt.cl:535-609
  V4<R> direct(V4<R> w_o, const Hit<R>& h, uint32_t& seed) {
    const V4<R> emission = ld<R>(mat_of(h).ke);
    V4<R> light_sample{R(0), R(0), R(0), R(0)};
    V4<R> w_i;
    R light_pdf = R(0), brdf_prob = R(0);
    bool glossy = false;
    const int j = sample_lights(h, light_pdf, w_i, seed);
    if (j == -1 || light_pdf <= 0.0) return emission;
    R len = length(w_i);
    len = O::sub(len, (R)ym::mul(EPS_F, 1.5f));
    w_i = normalize(w_i);
    Ray<R> sray{h.hit_point + w_i * (R)EPS_F, w_i, len, true};
    Hit<R> shit;
    cnt.shadow++;
    rec_kind = 2;
    const bool occluded = trace(sray, shit);
    const V4<R> lke = ld<R>(sc.lights[j].ke);
    if (!occluded) {
      glossy = sample_glossy(h, seed, brdf_prob);
      if (brdf_prob == R(0)) return emission;
      light_sample = (brdf(w_i, w_o, h, glossy, brdf_prob) * lke) * O::fmax(dot(w_i, h.normal), R(0));
      light_sample = light_sample * O::div(R(1), light_pdf);
    }
    if (!cfg.mis) return light_sample + emission;

    if (occluded && cfg.mis_lobe_fix) {
      glossy = sample_glossy(h, seed, brdf_prob);
      if (brdf_prob == R(0)) return light_sample + emission;
    }
    R brdf_pdf = glossy ? phong_pdf(w_i, w_o, h) : cos_pdf(w_i, h.normal);
    R mis_w = light_pdf;
    mis_w = O::div(ym_pown(mis_w), O::add(ym_pown(light_pdf), ym_pown(brdf_pdf)));
    light_sample = light_sample * mis_w;
    Ray<R> bray;
    if (glossy) sample_phong(bray, brdf_pdf, w_o, h, seed);
    else sample_cosine(bray, brdf_pdf, h, seed);
    if (brdf_pdf <= 0.0) return light_sample + emission;
    w_i = bray.dir;
    Hit<R> nh;
    cnt.mis++;
    rec_kind = 3;
    rec_light = j;
    if (!trace(bray, nh) || nh.light != j) return light_sample + emission;
    mis_w = brdf_pdf;
    mis_w = O::div(ym_pown(mis_w), O::add(ym_pown(light_pdf), ym_pown(brdf_pdf)));
    V4<R> brdf_sample = (brdf(w_i, w_o, h, glossy, brdf_prob) * lke) * O::fmax(dot(w_i, h.normal), R(0));
    brdf_sample = brdf_sample * O::div(mis_w, brdf_pdf);
    return (light_sample + brdf_sample) + emission;
  }
  static R ym_pown(R x) { return O::mul(x, x); }   // pown(x, 2), udpt.cl:1149-1152

  static R luminance(V4<R> c) {   // getYluminance, udpt.cl:1121-1124
    return O::add(O::add(O::mul((R)0.212671f, c.x), O::mul((R)0.715160f, c.y)), O::mul((R)0.072169f, c.z));
  }

  // shading, udpt.cl:433-533
  V4<R> shade(Ray<R> ray, uint32_t& seed) {
    Hit<R> hit;
    cnt.primary++;
    rec_kind = 0;
    if (!trace(ray, hit)) return V4<R>{(R)0.4f, (R)0.4f, (R)0.4f, R(1)};
    if (hit.light >= 0) {
      if (dot(ray.dir, ld<R>(sc.lights[hit.light].normal)) < 0) return V4<R>{R(1), R(1), R(1), R(1)};
      return V4<R>{(R)0.1f, (R)0.1f, (R)0.1f, R(1)};
    }
    V4<R> thr{R(1), R(1), R(1), R(1)};
    V4<R> direct_c{R(0), R(0), R(0), R(0)};
    V4<R> indirect{R(0), R(0), R(0), R(0)};
    int matID = sc.tris[hit.tri].matID;
    if (!sc.mats[matID].is_specular) direct_c = direct(-ray.dir, hit, seed);
    if (cfg.gi_check) {
      for (int i = 0; i < cfg.max_depth; ++i) {
        Hit<R> nh;
        Ray<R> nray;
        R pdf = R(1), brdf_prob = R(0), ior = R(1);
        bool glossy = false;
        const bool spec = sc.mats[matID].is_specular != 0;
        if (spec) sample_fresnel(nray, hit, -ray.dir, ior, seed);
        else {
          glossy = sample_glossy(hit, seed, brdf_prob);
          if (brdf_prob == R(0)) break;
          if (glossy) sample_phong(nray, pdf, -ray.dir, hit, seed);
          else sample_cosine(nray, pdf, hit, seed);
        }
        bool traced_hit = false;
        if (!(pdf <= 0.0)) { cnt.extension++; rec_kind = 1; traced_hit = trace(nray, nh); }
        if (pdf <= 0.0 || !traced_hit || nh.light >= 0) {
          if (spec && nh.light >= 0) indirect = indirect + thr * ld<R>(sc.lights[nh.light].ke);
          break;
        }
        indirect = indirect + thr * ld<R>(sc.mats[sc.tris[nh.tri].matID].ke);
        if (spec) thr = thr * ior;
        else thr = ((thr * brdf(nray.dir, -ray.dir, hit, glossy, brdf_prob)) * O::fmax(dot(nray.dir, hit.normal), R(0))) / pdf;
        if (i > cfg.rr_threshold) {
          const R p = O::min(luminance(thr), (R)0.95f);
          const R r = draw(seed);
          if (r >= p) break;
          thr = thr * O::div(R(1), p);
        }
        matID = sc.tris[nh.tri].matID;
        if (!sc.mats[matID].is_specular) indirect = indirect + thr * direct(-nray.dir, nh, seed);
        hit = nh;
        ray = nray;
      }
    }
    return direct_c + indirect;
  }
};

// createRay, udpt.cl:213-238 (the double-precision literals are kept)
template <class R>
inline Ray<R> create_ray(R px, R py, int W, int H, const yc_cam& cam) {
  using O = Ops<R>;
  const R aspect = (R)(((double)W * 1.0) / (double)H);
  V4<R> dir;
  dir.x = (R)((double)aspect * ((2.0 * (double)px / (double)W) - 1));
  dir.y = (R)((2.0 * (double)py / (double)H) - 1);
  dir.z = -(R)cam.view_plane_dist;
  dir.w = R(0);
  Ray<R> r;
  r.dir.x = dot(ld<R>(cam.r1), dir);
  r.dir.y = dot(ld<R>(cam.r2), dir);
  r.dir.z = dot(ld<R>(cam.r3), dir);
  r.dir.w = dot(ld<R>(cam.r4), dir);
  r.dir = normalize(r.dir);
  r.origin = V4<R>{(R)cam.r1.w, (R)cam.r2.w, (R)cam.r3.w, (R)cam.r4.w};
  r.is_shadow = false;
  r.length = (R)INFINITY;
  (void)sizeof(O);
  return r;
}

// pathtracer, udpt.cl:158-211: one sample of pixel (x, y); returns the colour before
// accumulation (NaN replaced by PINK).
template <class R>
inline V4<R> pixel_sample(Tracer<R>& tr, const yc_cam& cam, int x, int y, int W, int H, uint32_t rand) {
  using O = Ops<R>;
  uint32_t seed = (uint32_t)((y + 1) * W + (x + 1));
  seed = rand * seed;
  seed = ym::wang_hash(seed);
  if (seed == 0) seed = ym::wang_hash(seed);
  const R r1 = tr.draw(seed);
  const R r2 = tr.draw(seed);
  Ray<R> ray = create_ray<R>(O::add((R)x, r1), O::add((R)y, r2), W, H, cam);
  V4<R> c = tr.shade(ray, seed);
  if (any_nan(c)) c = V4<R>{(R)0.988f, (R)0.0588f, (R)0.7529f, R(1)};
  return c;
}

// running mean of udpt.cl:196-210
template <class R>
inline V4<R> accumulate(V4<R> c, V4<R> prev, int reset) {
  using O = Ops<R>;
  if (reset == 1) { c.w = R(1); return c; }
  const int n = (int)prev.w;
  c = c + prev * (R)n;
  c = c / (R)(n + 1);
  c.w = (R)(n + 1);
  (void)sizeof(O);
  return c;
}

}  // namespace orc
