// bdpt_mis_oracle.hpp -- CPU statement of the bidirectional path tracer with multiple
// importance sampling (integrator YC_BDPT_MIS). TEST INFRASTRUCTURE, like udpt_oracle.hpp.
//
// bdpt.cl keeps forward and reverse densities on its path vertices but never uses them:
// its connections are summed with the heuristic weight `weight * (1 - ks)` (bdpt.cl:38-39,
// 453, 465, 598-636), so its image is not the one the unidirectional tracer converges to.
// This integrator is the unbiased replacement: every strategy (s light vertices, t eye
// vertices, t >= 2) is weighted by Veach's power heuristic (beta = 2) over the strategies
// that can produce the same path, and the weights are evaluated in O(1) per connection
// from two partial sums kept on each subpath vertex, the recursive form published by
// Georgiev ("Implementing Vertex Connection and Merging", 2012), restricted to
// bidirectional path tracing without light tracing to the camera (t = 1).
//
// Material model: the BRDF of bdpt.cl summed over its lobes, f = kd/pi (Oren-Nayar for
// ks = 0 when brdf_model = 1, udpt-primitives.cl:673-725) + ks (n + 2)/(2 pi) cos^n of the
// angle to the mirror direction (bdpt.cl:718-737), with n = px + py; dielectrics are
// treated by the same rule, as bdpt.cl does. Surfaces are one-sided: a subpath that
// arrives from below the shading normal ends there. Lights: the quad lights, one-sided,
// emitting ke with a cosine pattern, picked with probability proportional to
// (ke.r + ke.g + ke.b) * area.
//
// Random numbers per sample, from the per-pixel stream of the reference prologue:
//   2 (pixel jitter); light subpath: 1 (light) + 2 (point) + 2 (direction), then at each
//   light vertex that continues: 1 (roulette, vertex index > rr_threshold) + 1 (lobe) + 2;
//   eye subpath, at each eye vertex: 1 + 2 (next-event light and point), then when it
//   continues: 1 (roulette, index > rr_threshold) + 1 (lobe) + 2.
// kmax = the longest path in segments (camera to light); the light subpath keeps
// x_0 .. x_{kmax-2}, the eye subpath y_1 .. y_kmax.
#pragma once

#include "bdpt_oracle.hpp"

namespace orc {

template <class R>
struct MisVertex {
  Hit<R> hit;
  V4<R> dir_in{0, 0, 0, 0};   // direction of the ray that reached the vertex
  V4<R> beta{0, 0, 0, 0};     // subpath throughput
  R r = 0, s = 0;             // partial sums of the power-heuristic denominator
};

template <class R>
struct BdptMisTracer : BdptTracer<R> {
  using O = Ops<R>;
  using Base = BdptTracer<R>;
  using Base::sc;
  using Base::cfg;
  using Base::cnt;
  using Base::draw;
  using Base::mat_of;
  using Base::trace;
  using Base::sample_cosine;
  using Base::sample_phong_b;
  using Base::oren_nayar;
  using Base::luminance;
  static constexpr float PI_F = 3.14159265359f;
  static constexpr float INV_PI_F = 0.31830988618f;
  static constexpr float EPS_F = 0.0001f;
  int kmax;

  BdptMisTracer(const Scene<R>& s, const Config& c, Counters& k, int kmax_) : Base(s, c, k, 2), kmax(kmax_) {}

  static R mis(R x) { return O::mul(x, x); }
  // a * b with 0 * inf = 0 (a vanishing density removes the strategy)
  static R mul0(R a, R b) { return (a == R(0) || b == R(0)) ? R(0) : O::mul(a, b); }
  static V4<R> rgb(const yc_float4& c) { return V4<R>{(R)c.x, (R)c.y, (R)c.z, R(0)}; }

  // probability of the diffuse lobe: its share of kd + ks
  static R diffuse_prob(const yc_material& m) {
    const R sd = O::add(O::add((R)m.kd.x, (R)m.kd.y), (R)m.kd.z);
    const R ss = O::add(O::add((R)m.ks.x, (R)m.ks.y), (R)m.ks.z);
    if (ss == R(0)) return R(1);
    if (sd == R(0)) return R(0);
    return O::div(sd, O::add(sd, ss));
  }

  static V4<R> mirror(V4<R> w, V4<R> n) { return normalize(O::mul(R(2), dot(w, n)) * n - w); }

  // BRDF at h between the direction toward the previous subpath vertex and the next one
  V4<R> f_eval(const Hit<R>& h, V4<R> w_prev, V4<R> w_next) const {
    const yc_material& m = mat_of(h);
    const bool glossy = length3(ld<R>(m.ks)) != R(0);
    V4<R> f;
    if (cfg.brdf_model == 1 && !glossy) f = oren_nayar(w_next, w_prev, h);
    else f = ld<R>(m.kd) * (R)INV_PI_F;
    if (glossy) {
      const R ca = O::pow(O::fmax(dot(w_next, mirror(w_prev, h.normal)), R(0)), O::add((R)m.px, (R)m.py));
      const int pe = (int)O::add((R)m.px, (R)m.py);
      f = f + (((ld<R>(m.ks) * ca) * (R)(pe + 2)) * (R)INV_PI_F) * R(0.5f);
    }
    f.w = R(0);
    return f;
  }

  // solid-angle density with which sample_dir picks w_next at h after arriving from w_prev
  R pdf_dir(const Hit<R>& h, V4<R> w_prev, V4<R> w_next) const {
    const yc_material& m = mat_of(h);
    const R cn = dot(w_next, h.normal);
    if (!(cn > R(0))) return R(0);
    const R pd = diffuse_prob(m);
    R p = O::mul(pd, O::mul(cn, (R)INV_PI_F));
    if (pd < R(1)) {
      const int pe = (int)O::add((R)m.px, (R)m.py);
      const R ca = O::fmax(dot(w_next, mirror(w_prev, h.normal)), R(0));
      const R lobe = O::mul(O::mul(O::mul((R)(pe + 1), R(0.5f)), (R)INV_PI_F), O::pow(ca, (R)pe));
      p = O::add(p, O::mul(O::sub(R(1), pd), lobe));
    }
    return p;
  }

  // lobe (1 number), then a cosine or Phong-lobe direction (2 numbers); false when the
  // direction does not leave the surface
  bool sample_dir(const Hit<R>& h, V4<R> w_prev, uint32_t& seed, V4<R>& w_next) {
    const yc_material& m = mat_of(h);
    const R u = draw(seed);
    const R pd = diffuse_prob(m);
    Ray<R> ray;
    R pdf = R(0);
    if (pd >= R(1) || u < pd) {
      sample_cosine(ray, pdf, h, seed);
      w_next = ray.dir;
    } else {
      sample_phong_b(ray, pdf, w_prev, h, seed);
      w_next = ray.dir;
    }
    return dot(w_next, h.normal) > R(0);
  }

  R light_weight(int i) const {
    const yc_quad_light& L = sc.lights[i];
    const R e = O::add(O::add((R)L.ke.x, (R)L.ke.y), (R)L.ke.z);
    return O::mul(e, light_area(i));
  }
  R light_area(int i) const {
    const yc_quad_light& L = sc.lights[i];
    return O::mul(length(ld<R>(L.edge_l)), length(ld<R>(L.edge_w)));
  }
  R light_total() const {
    R t = R(0);
    for (int i = 0; i < sc.n_light; ++i) t = O::add(t, light_weight(i));
    return t;
  }
  // area density of the point a light sample lands on, on light i
  R light_point_pdf(int i) const { return O::div(O::div(light_weight(i), light_total()), light_area(i)); }

  // picks a light (1 number); -1 when no light emits
  int pick_light(uint32_t& seed) {
    const R u = draw(seed);
    const R total = light_total();
    if (!(total > R(0))) return -1;
    R cum = R(0);
    int last = -1;
    for (int i = 0; i < sc.n_light; ++i) {
      const R w = light_weight(i);
      if (!(w > R(0))) continue;
      last = i;
      const R p = O::div(w, total);
      if (u < O::add(cum, p)) return i;
      cum = O::add(cum, p);
    }
    return last;
  }

  V4<R> light_point(int i, uint32_t& seed) {
    const yc_quad_light& L = sc.lights[i];
    const R a = draw(seed);
    const R b = draw(seed);
    return (ld<R>(L.pos) + ld<R>(L.edge_l) * a) + ld<R>(L.edge_w) * b;
  }

  // light subpath x_0 .. x_n into lv; returns n (0: only the light point, or no light)
  int light_path(MisVertex<R>* lv, uint32_t& seed, int& lk, R& p0) {
    lk = pick_light(seed);
    if (lk < 0) return -1;
    const yc_quad_light& L = sc.lights[lk];
    p0 = light_point_pdf(lk);
    Hit<R> h0;
    h0.hit_point = light_point(lk, seed);
    h0.normal = ld<R>(L.normal);
    h0.light = lk;
    lv[0].hit = h0;
    Ray<R> ray;
    R pdf = R(0);
    sample_cosine(ray, pdf, h0, seed);
    const R c0 = dot(ray.dir, h0.normal);
    if (!(c0 > R(0))) return 0;
    R w_f = O::mul(c0, (R)INV_PI_F);
    R c_out = c0;
    R acc = O::div(R(1), mis(p0));
    V4<R> beta{R(1), R(1), R(1), R(0)};
    V4<R> prev = h0.hit_point;
    int n = 0;
    for (int j = 1; j <= kmax - 2; ++j) {
      cnt.extension++;
      Hit<R> h;
      if (!trace(ray, h) || h.light >= 0) break;
      const R cv = -dot(ray.dir, h.normal);
      if (!(cv > R(0))) break;
      const V4<R> dv = h.hit_point - prev;
      const R d2 = dot(dv, dv);
      MisVertex<R>& v = lv[j];
      v.hit = h;
      v.dir_in = ray.dir;
      v.beta = beta;
      v.r = mis(O::div(d2, O::mul(w_f, cv)));
      v.s = mul0(O::mul(v.r, mis(O::div(c_out, d2))), acc);
      n = j;
      if (j + 1 > kmax - 2) break;
      V4<R> cont = beta;
      if (j > cfg.rr_threshold) {
        const R q = O::min(luminance(beta), (R)0.95f);
        if (!(draw(seed) < q)) break;
        cont = beta / q;
      }
      const V4<R> wp = -ray.dir;
      V4<R> wn;
      if (!sample_dir(h, wp, seed, wn)) break;
      w_f = pdf_dir(h, wp, wn);
      if (!(w_f > R(0))) break;
      const R w_r = pdf_dir(h, wn, wp);
      c_out = dot(wn, h.normal);
      acc = O::add(v.r, mul0(v.s, mis(w_r)));
      beta = ((cont * f_eval(h, wp, wn)) * c_out) / w_f;
      prev = h.hit_point;
      ray.origin = h.hit_point + wn * (R)EPS_F;
      ray.dir = wn;
      ray.length = (R)INFINITY;
      ray.is_shadow = false;
    }
    return n;
  }

  // next-event estimate at eye vertex h (strategy s = 1)
  V4<R> nee(const Hit<R>& h, V4<R> wp, V4<R> beta, R r, R s, uint32_t& seed) {
    const V4<R> zero{R(0), R(0), R(0), R(0)};
    const int k = pick_light(seed);
    if (k < 0) return zero;
    const yc_quad_light& L = sc.lights[k];
    const R pk = light_point_pdf(k);
    const V4<R> x = light_point(k, seed);
    const V4<R> v = x - h.hit_point;
    const R d2 = dot(v, v);
    const R dist = O::sqrt(d2);
    const V4<R> dir = v * O::div(R(1), dist);
    const R cy = dot(dir, h.normal);
    const R cl = -dot(dir, ld<R>(L.normal));
    if (!(cy > R(0)) || !(cl > R(0))) return zero;
    Ray<R> sr{h.hit_point + dir * (R)EPS_F, dir, O::sub(dist, (R)ym::mul(EPS_F, 1.5f)), true};
    cnt.shadow++;
    Hit<R> sh;
    if (trace(sr, sh)) return zero;
    const R w_f = pdf_dir(h, wp, dir);
    const R w_r = pdf_dir(h, dir, wp);
    const R ls = mis(O::div(O::mul(w_f, cl), O::mul(d2, pk)));
    const R es = mul0(mis(O::div(O::mul(O::mul(cl, (R)INV_PI_F), cy), d2)), O::add(r, mul0(s, mis(w_r))));
    const R w = O::div(R(1), O::add(O::add(R(1), ls), es));
    const R g = O::div(O::mul(cy, cl), O::mul(d2, pk));
    return ((beta * f_eval(h, wp, dir)) * rgb(L.ke)) * O::mul(g, w);
  }

  // connection of eye vertex h to light vertex L (strategies s >= 2)
  V4<R> connect(const Hit<R>& h, V4<R> wp, V4<R> beta, R r, R s, const MisVertex<R>& L, V4<R> le) {
    const V4<R> zero{R(0), R(0), R(0), R(0)};
    const V4<R> v = L.hit.hit_point - h.hit_point;
    const R d2 = dot(v, v);
    const R dist = O::sqrt(d2);
    const V4<R> dir = v * O::div(R(1), dist);
    const R cy = dot(dir, h.normal);
    const R cl = -dot(dir, L.hit.normal);
    if (!(cy > R(0)) || !(cl > R(0))) return zero;
    Ray<R> sr{h.hit_point + dir * (R)EPS_F, dir, O::sub(dist, O::mul((R)EPS_F, R(2))), true};
    cnt.mis++;   // connection rays are counted in the `mis` slot of the counters
    Hit<R> sh;
    if (trace(sr, sh)) return zero;
    const V4<R> lp = -L.dir_in;
    const V4<R> wl = -dir;
    const R wy_f = pdf_dir(h, wp, dir);
    const R wy_r = pdf_dir(h, dir, wp);
    const R wl_f = pdf_dir(L.hit, lp, wl);
    const R wl_r = pdf_dir(L.hit, wl, lp);
    const R ls = mul0(mis(O::div(O::mul(wy_f, cl), d2)), O::add(L.r, mul0(L.s, mis(wl_r))));
    const R es = mul0(mis(O::div(O::mul(wl_f, cy), d2)), O::add(r, mul0(s, mis(wy_r))));
    const R w = O::div(R(1), O::add(O::add(R(1), ls), es));
    const R g = O::div(O::mul(cy, cl), d2);
    return ((((beta * f_eval(h, wp, dir)) * f_eval(L.hit, lp, wl)) * L.beta) * le) * O::mul(g, w);
  }

  V4<R> shade_m(Ray<R> ray, uint32_t& seed) {
    MisVertex<R> lv[34];
    int lk = -1;
    R p0 = R(0);
    const int nl = light_path(lv, seed, lk, p0);
    V4<R> le{R(0), R(0), R(0), R(0)};
    if (lk >= 0) le = rgb(sc.lights[lk].ke) * O::div((R)PI_F, p0);
    cnt.primary++;
    Hit<R> h;
    if (!trace(ray, h)) return V4<R>{(R)0.4f, (R)0.4f, (R)0.4f, R(1)};
    if (h.light >= 0) {
      if (dot(ray.dir, ld<R>(sc.lights[h.light].normal)) < 0) return V4<R>{R(1), R(1), R(1), R(1)};
      return V4<R>{(R)0.1f, (R)0.1f, (R)0.1f, R(1)};
    }
    V4<R> color{R(0), R(0), R(0), R(1)};
    V4<R> beta{R(1), R(1), R(1), R(0)};
    R r = R(0), s = R(0);
    for (int m = 1;; ++m) {
      const V4<R> wp = -ray.dir;
      if (!(dot(wp, h.normal) > R(0))) break;
      color = color + beta * rgb(mat_of(h).ke);
      if (m + 1 > kmax) break;
      if (lk >= 0) {
        color = color + nee(h, wp, beta, r, s, seed);
        for (int j = 1; j <= nl && m + j + 1 <= kmax; ++j) color = color + connect(h, wp, beta, r, s, lv[j], le);
      }
      V4<R> cont = beta;
      if (m > cfg.rr_threshold) {
        const R q = O::min(luminance(beta), (R)0.95f);
        if (!(draw(seed) < q)) break;
        cont = beta / q;
      }
      V4<R> wn;
      if (!sample_dir(h, wp, seed, wn)) break;
      const R w_f = pdf_dir(h, wp, wn);
      if (!(w_f > R(0))) break;
      const R w_r = pdf_dir(h, wn, wp);
      const R c_out = dot(wn, h.normal);
      const R acc = O::add(r, mul0(s, mis(w_r)));
      const V4<R> bn = ((cont * f_eval(h, wp, wn)) * c_out) / w_f;
      Ray<R> nr{h.hit_point + wn * (R)EPS_F, wn, (R)INFINITY, false};
      cnt.extension++;
      Hit<R> nh;
      if (!trace(nr, nh)) break;
      const V4<R> dv = nh.hit_point - h.hit_point;
      const R d2 = dot(dv, dv);
      if (nh.light >= 0) {   // strategy s = 0
        const yc_quad_light& L = sc.lights[nh.light];
        const R cl = -dot(wn, ld<R>(L.normal));
        if (cl > R(0)) {
          const R r2 = mis(O::div(d2, O::mul(w_f, cl)));
          const R s2 = mul0(O::mul(r2, mis(O::div(c_out, d2))), acc);
          const R es = O::mul(mis(light_point_pdf(nh.light)), O::add(r2, mul0(s2, mis(O::mul(cl, (R)INV_PI_F)))));
          const R w = O::div(R(1), O::add(R(1), es));
          color = color + (bn * rgb(L.ke)) * w;
        }
        break;
      }
      const R cv = -dot(wn, nh.normal);
      if (!(cv > R(0))) break;
      r = mis(O::div(d2, O::mul(w_f, cv)));
      s = mul0(O::mul(r, mis(O::div(c_out, d2))), acc);
      beta = bn;
      h = nh;
      ray = nr;
    }
    return color;
  }
};

// one sample of pixel (x, y): the reference prologue (bdpt.cl:158-189), then shade_m
template <class R>
inline V4<R> pixel_sample_bdpt_mis(BdptMisTracer<R>& tr, const yc_cam& cam, int x, int y, int W, int H,
                                   uint32_t rand) {
  using O = Ops<R>;
  uint32_t seed = (uint32_t)((y + 1) * W + (x + 1));
  seed = rand * seed;
  seed = ym::wang_hash(seed);
  if (seed == 0) seed = ym::wang_hash(seed);
  const R r1 = tr.draw(seed);
  const R r2 = tr.draw(seed);
  Ray<R> ray = create_ray<R>(O::add((R)x, r1), O::add((R)y, r2), W, H, cam);
  V4<R> c = tr.shade_m(ray, seed);
  if (any_nan(c)) c = V4<R>{(R)0.988f, (R)0.0588f, (R)0.7529f, R(1)};
  return c;
}

}  // namespace orc
