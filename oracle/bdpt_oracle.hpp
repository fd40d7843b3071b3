// bdpt_oracle.hpp -- CPU restatement of Yune's naive bidirectional path tracer
// (kernels/legacy/bdpt.cl). TEST INFRASTRUCTURE, like udpt_oracle.hpp.
//
// bdpt.cl shares traceRay, the samplers, sampleLights and evaluateDirectLighting with
// udpt.cl; the functions that differ are restated here:
//   evaluateBRDF       reflection vector without the normal flip (bdpt.cl:718-737)
//   phongSampleHemisphere  lobe axis without the flip (bdpt.cl:807-870)
//   sampleGlossyPdf    the lobe probabilities are raised by (1 - max)/2 when the
//                      channel maximum is below 1, and the path is never absorbed
//                      (bdpt.cl:1048-1105)
//   createLightPath, createEyePath, shading  (bdpt.cl:432-640)
// One departure: when the camera ray hits the light, bdpt.cl keeps extending the eye
// path from a vertex with triangle_ID = -1 (it reads scene_data[-1]) although the pixel
// colour is then fixed to white or grey (bdpt.cl:570-575); the restatement stops the
// eye path there, which leaves the colour unchanged.
#pragma once

#include "udpt_oracle.hpp"

namespace orc {

template <class R>
struct PathVertex {
  Hit<R> hit;
  V4<R> dir{0, 0, 0, 0};
  V4<R> contrib{0, 0, 0, 0};
  R fwd_pdf = 0, rev_pdf = 0;
};

template <class R>
struct BdptTracer : Tracer<R> {
  using O = Ops<R>;
  using Base = Tracer<R>;
  using Base::sc;
  using Base::cfg;
  using Base::cnt;
  using Base::draw;
  using Base::mat_of;
  using Base::trace;
  using Base::frame;
  using Base::to_world;
  using Base::sample_cosine;
  static constexpr float PI_F = 3.14159265359f;
  static constexpr float INV_PI_F = 0.31830988618f;
  static constexpr float EPS_F = 0.0001f;
  int bounces;
  int rr_bdpt;

  BdptTracer(const Scene<R>& s, const Config& c, Counters& k, int b) : Base(s, c, k), bounces(b), rr_bdpt(4) {}

  // evaluateBRDF, bdpt.cl:718-737
  V4<R> brdf_b(V4<R> w_i, V4<R> w_o, const Hit<R>& h, bool glossy, R rr_prob) const {
    V4<R> refl = O::mul(R(2), dot(w_i, h.normal)) * h.normal - w_i;
    refl = normalize(refl);
    const yc_material& m = mat_of(h);
    if (!glossy) return (ld<R>(m.kd) * (R)INV_PI_F) / rr_prob;
    const R cos_alpha = O::pow(O::fmax(dot(w_o, refl), R(0)), O::add((R)m.px, (R)m.py));
    const int pe = (int)((R)m.px + (R)m.py);
    return ((((ld<R>(m.ks) * cos_alpha) * (R)(pe + 2)) * (R)INV_PI_F) * R(0.5f)) / rr_prob;
  }

  // phongSampleHemisphere, bdpt.cl:807-870
  void sample_phong_b(Ray<R>& ray, R& pdf, V4<R> w_i, const Hit<R>& h, uint32_t& seed) const {
    V4<R> Nz = O::mul(R(2), dot(w_i, h.normal)) * h.normal - w_i;
    Nz = normalize(Nz);
    V4<R> Nx, Ny;
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

  // calcPhongPDF (bdpt.cl, same text as udpt.cl:1033-1045)
  R phong_pdf_b(V4<R> w_i, V4<R> w_o, const Hit<R>& h) const { return Base::phong_pdf(w_i, w_o, h); }

  // sampleGlossyPdf, bdpt.cl:1048-1105
  bool sample_glossy_b(const Hit<R>& h, uint32_t& seed, R& prob) {
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
    if (mx < R(1)) {
      const R half = O::div(O::sub(R(1), mx), R(2));
      pd = O::add(pd, half);
      ps = O::add(ps, half);
    }
    if (r < pd) { prob = pd; return false; }
    prob = ps;
    return true;
  }

  // evaluateDirectLighting of bdpt.cl:642-716 (MIS off as shipped; same as udpt.cl with
  // the BDPT BRDF and lobe choice)
  V4<R> direct_b(V4<R> w_o, const Hit<R>& h, uint32_t& seed) {
    const V4<R> emission = ld<R>(mat_of(h).ke);
    V4<R> light_sample{R(0), R(0), R(0), R(0)};
    V4<R> w_i;
    R light_pdf = R(0), brdf_prob = R(0);
    const int j = Base::sample_lights(h, light_pdf, w_i, seed);
    if (j == -1 || light_pdf <= 0.0) return emission;
    R len = length(w_i);
    len = O::sub(len, (R)ym::mul(EPS_F, 1.5f));
    w_i = normalize(w_i);
    Ray<R> sray{h.hit_point + w_i * (R)EPS_F, w_i, len, true};
    Hit<R> shit;
    cnt.shadow++;
    if (!trace(sray, shit)) {
      const bool glossy = sample_glossy_b(h, seed, brdf_prob);
      if (brdf_prob == R(0)) return emission;
      light_sample = (brdf_b(w_i, w_o, h, glossy, brdf_prob) * ld<R>(sc.lights[j].ke)) * O::fmax(dot(w_i, h.normal), R(0));
      light_sample = light_sample * O::div(R(1), light_pdf);
    }
    return light_sample + emission;
  }

  // createLightPath, bdpt.cl:432-511
  int light_path(PathVertex<R>* lp, uint32_t& seed) {
    int len = 1;
    const yc_quad_light& L = sc.lights[0];
    Hit<R> hit;
    hit.normal = ld<R>(L.normal);
    R pdf = R(1);
    seed = ym::xor_shift(seed);
    const R r1 = (R)((double)seed / 4294967295.0);   // seed / (double)UINT_MAX
    const R r2 = draw(seed);
    const V4<R> A = ld<R>(L.edge_l) * r2;
    const V4<R> B = ld<R>(L.edge_w) * r1;
    hit.hit_point = (A + B) + ld<R>(L.pos);
    hit.normal = ld<R>(L.normal);
    lp[0].hit = hit;
    lp[0].hit.light = 0;
    const R area = O::mul(length(ld<R>(L.edge_l)), length(ld<R>(L.edge_w)));
    lp[0].fwd_pdf = O::div(R(1), area);
    lp[0].rev_pdf = R(1);
    lp[0].contrib = ld<R>(L.ke) / lp[0].fwd_pdf;
    Ray<R> ray;
    sample_cosine(ray, pdf, hit, seed);
    if (pdf <= 0.0) return len;
    cnt.extension++;
    if (!trace(ray, hit) || hit.light >= 0) return len;
    lp[1].hit = hit;
    lp[1].dir = ray.dir;
    lp[1].fwd_pdf = pdf;
    lp[1].rev_pdf = R(1);
    const R c1 = O::div(O::max(R(0), dot(lp[0].hit.normal, lp[1].dir)), pdf);
    lp[1].contrib = V4<R>{c1, c1, c1, c1} * lp[0].contrib;
    R brdf_prob = R(0);
    ++len;
    for (int i = 2; i < bounces; ++i) {
      const bool glossy = sample_glossy_b(hit, seed, brdf_prob);
      if (brdf_prob == R(0)) break;
      if (glossy) sample_phong_b(ray, pdf, -lp[i - 1].dir, hit, seed);
      else sample_cosine(ray, pdf, hit, seed);
      cnt.extension++;
      if (!trace(ray, hit) || hit.light >= 0 || pdf <= 0.0) break;
      ++len;
      lp[i].hit = hit;
      lp[i].dir = ray.dir;
      lp[i].fwd_pdf = pdf;
      lp[i].rev_pdf = R(1);
      lp[i].contrib = brdf_b(-lp[i - 1].dir, lp[i].dir, lp[i - 1].hit, glossy, brdf_prob) *
                      O::fmax(R(0), dot(lp[i].dir, lp[i - 1].hit.normal));
      lp[i].contrib = lp[i].contrib / pdf;
      lp[i].contrib = lp[i].contrib * lp[i - 1].contrib;
      if (i > rr_bdpt) {
        const R r = draw(seed);
        const R p = O::min(Base::luminance(lp[i].contrib), (R)0.95f);
        if (r >= p) break;
        lp[i].contrib = lp[i].contrib * O::div(R(1), p);
      }
    }
    return len;
  }

  // createEyePath, bdpt.cl:513-560 (stops after a light hit, see the file comment)
  int eye_path(PathVertex<R>* ep, Ray<R> ray, uint32_t& seed) {
    int len = 1;
    Hit<R> hit;
    ep[0].hit = hit;
    cnt.primary++;
    if (!trace(ray, ep[0].hit)) return len;
    ep[0].dir = ray.dir;
    ep[0].fwd_pdf = R(1);
    ep[0].contrib = V4<R>{R(1), R(1), R(1), R(1)};
    if (ep[0].hit.light >= 0) return len;
    R pdf = R(1), brdf_prob = R(0);
    for (int i = 1; i < bounces; ++i) {
      const bool glossy = sample_glossy_b(ep[i - 1].hit, seed, brdf_prob);
      if (brdf_prob == R(0)) break;
      if (glossy) sample_phong_b(ray, pdf, -ep[i - 1].dir, ep[i - 1].hit, seed);
      else sample_cosine(ray, pdf, ep[i - 1].hit, seed);
      if (pdf <= 0.0) break;
      cnt.extension++;
      if (!trace(ray, hit) || hit.light >= 0) break;
      ++len;
      ep[i].hit = hit;
      ep[i].dir = ray.dir;
      ep[i].fwd_pdf = pdf;
      ep[i].contrib = brdf_b(ep[i].dir, -ep[i - 1].dir, ep[i - 1].hit, glossy, brdf_prob) *
                      O::max(R(0), dot(ep[i].dir, ep[i - 1].hit.normal));
      ep[i].contrib = ep[i].contrib / pdf;
      ep[i].contrib = ep[i].contrib * ep[i - 1].contrib;
      if (i > rr_bdpt) {
        const R r = draw(seed);
        const R p = O::min(Base::luminance(ep[i].contrib), (R)0.95f);
        if (r >= p) break;
        ep[i].contrib = ep[i].contrib * O::div(R(1), p);
      }
    }
    return len;
  }

  // shading, bdpt.cl:562-640
  V4<R> shade_b(Ray<R> ray, uint32_t& seed) {
    PathVertex<R> lp[32], ep[32];
    const int lp_len = light_path(lp, seed);
    const int ep_len = eye_path(ep, ray, seed);
    if (ep[0].hit.light >= 0) {
      if (dot(ray.dir, ld<R>(sc.lights[ep[0].hit.light].normal)) < 0) return V4<R>{R(1), R(1), R(1), R(1)};
      return V4<R>{(R)0.1f, (R)0.1f, (R)0.1f, R(1)};
    }
    if (ep[0].hit.tri < 0) return V4<R>{(R)0.4f, (R)0.4f, (R)0.4f, R(1)};
    V4<R> color{R(0), R(0), R(0), R(1)};
    R weight = R(1), ks = R(0);
    for (int i = 0; i < ep_len; ++i) {
      if (weight == R(0)) break;
      V4<R> sub{R(0), R(0), R(0), R(1)};
      const yc_material& m = mat_of(ep[i].hit);
      const V4<R> spec = ld<R>(m.ks), emission = ld<R>(m.ke);
      ks = O::max(O::max(spec.x, O::max(spec.y, spec.z)), (R)0.1f);
      const V4<R> thr = ep[i].contrib;
      color = color + (thr * (emission + direct_b(-ep[i].dir, ep[i].hit, seed))) * weight;
      for (int j = lp_len - 1; j > 0; --j) {
        Ray<R> dr;
        Hit<R> dh;
        dr.dir = normalize(lp[j].hit.hit_point - ep[i].hit.hit_point);
        dr.origin = ep[i].hit.hit_point + dr.dir * (R)EPS_F;
        R dist = length(lp[j].hit.hit_point - ep[i].hit.hit_point);
        dist = O::mul(dist, dist);
        dr.length = length(lp[j].hit.hit_point - dr.origin);
        dr.is_shadow = true;
        if (dot(dr.dir, ep[i].hit.normal) <= 0 || dot(-dr.dir, lp[j].hit.normal) <= 0) continue;
        cnt.mis++;   // connection rays are counted in the `mis` slot of the counters
        if (!trace(dr, dh)) {
          V4<R> tlp = lp[j].contrib;
          const V4<R> w_i = dr.dir;
          const V4<R> w_o = -ep[i].dir;
          const Hit<R>& h = ep[i].hit;
          const R gf = O::div(O::mul(O::max(dot(w_i, h.normal), R(0)), O::max(dot(-w_i, lp[j].hit.normal), R(0))), dist);
          R prob = R(0);
          bool g = sample_glossy_b(h, seed, prob);
          const V4<R> e2l = brdf_b(w_i, w_o, h, g, prob);
          g = sample_glossy_b(lp[j].hit, seed, prob);
          const V4<R> l2e = brdf_b(-lp[j].dir, -w_i, lp[j].hit, g, prob);
          tlp = tlp * ((gf * e2l) * l2e);
          tlp = tlp * thr;
          sub = sub + tlp;
        }
      }
      color = color + sub * O::mul(weight, O::sub(R(1), ks));
      weight = O::mul(weight, ks);
    }
    return color;
  }
};

// pathtracer of bdpt.cl:158-210 for one pixel
template <class R>
inline V4<R> pixel_sample_bdpt(BdptTracer<R>& tr, const yc_cam& cam, int x, int y, int W, int H, uint32_t rand) {
  using O = Ops<R>;
  uint32_t seed = (uint32_t)((y + 1) * W + (x + 1));
  seed = rand * seed;
  seed = ym::wang_hash(seed);
  if (seed == 0) seed = ym::wang_hash(seed);
  const R r1 = tr.draw(seed);
  const R r2 = tr.draw(seed);
  Ray<R> ray = create_ray<R>(O::add((R)x, r1), O::add((R)y, r2), W, H, cam);
  V4<R> c = tr.shade_b(ray, seed);
  if (any_nan(c)) c = V4<R>{(R)0.988f, (R)0.0588f, (R)0.7529f, R(1)};
  return c;
}

}  // namespace orc
