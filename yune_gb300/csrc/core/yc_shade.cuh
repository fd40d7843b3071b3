// yc_shade.cuh -- per-vertex shading of the wavefront path tracer (device side).
//
// Each function performs the arithmetic of its kernels/legacy/udpt.cl counterpart in
// the same FP32 operation order (cited per function), with the ym:: built-ins, so a
// path consumes the same random numbers and produces the same bits as the CPU oracle.
// Points carry w = 1 and directions w = 0, as in the reference's float4 values; the
// w lanes are kept because the four-lane dot products and the NaN test of the final
// colour see them.
#pragma once

#include "../ym_math.h"
#include "yc_scene.h"

namespace yc {

using ym::f4;

constexpr float PI_F = 3.14159265359f;
constexpr float INV_PI_F = 0.31830988618f;
constexpr float EPS_F = 0.0001f;
// largest float f with (double)f <= 0.0001: |DdotN| > 0.0001 (udpt.cl:247, compared in
// double) holds exactly when |DdotN| > this value
constexpr uint32_t LIGHT_DDOTN_BITS = 0x38D1B717u;

__device__ __forceinline__ f4 ld4(const yc_float4& v) { return ym::mk(v.x, v.y, v.z, v.w); }
__device__ __forceinline__ f4 f4of(float4 v) { return ym::mk(v.x, v.y, v.z, v.w); }
__device__ __forceinline__ float draw(uint32_t& seed) { seed = ym::xor_shift(seed); return ym::u01(seed); }

struct Vtx {
  f4 hp;      // hit point, w = 1
  f4 n;       // shading normal, w = 0
  int mat;
};

// the analytic quad-light loop of traceRay (udpt.cl:244-276); updates len and the hit light
__device__ __forceinline__ void light_test(const DevScene& sc, f4 o, f4 d, float& len, int& light) {
  for (int i = 0; i < sc.n_lights; ++i) {
    const yc_quad_light& L = sc.lights[i];
    const f4 nrm = ld4(L.normal);
    const float DdotN = ym::dot(d, nrm);
    if (ym::fabs(DdotN) > __uint_as_float(LIGHT_DDOTN_BITS)) {
      const f4 pos = ld4(L.pos);
      const float t = ym::div(ym::dot(nrm, pos - o), DdotN);
      if (t > 0.0f && t < len) {
        f4 temp = o + d * t;
        temp = temp - pos;
        const f4 el = ld4(L.edge_l), ew = ld4(L.edge_w);
        float p1 = ym::dot(temp, el);
        float p2 = ym::dot(temp, ew);
        const float la = ym::length(el), lb = ym::length(ew);
        p1 = ym::div(p1, la);
        p2 = ym::div(p2, lb);
        if ((p1 >= 0.0f && p2 >= 0.0f) && (p1 <= la && p2 <= lb)) {
          len = t;
          light = i;
        }
      }
    }
  }
}

__device__ __forceinline__ void frame(f4 Nz, f4& Nx, f4& Ny) {
  if (ym::fabs(Nz.y) > ym::fabs(Nz.z)) Nx = ym::mk(Nz.y, -Nz.x, 0.0f, 0.0f);
  else Nx = ym::mk(Nz.z, 0.0f, -Nz.x, 0.0f);
  Nx = ym::normalize(Nx);
  Ny = ym::normalize(ym::cross(Nz, Nx));
}

// reflect, udpt.cl:949-961
__device__ __forceinline__ f4 reflect(f4 w_i, f4 n) {
  if (ym::dot(w_i, n) < 0.0f) n = n * -1.0f;
  const f4 r = ym::mul(2.0f, ym::dot(w_i, n)) * n - w_i;
  return ym::normalize(r);
}

// refract, udpt.cl:963-990
__device__ __forceinline__ f4 refract(f4 w_i, f4 n, float ior) {
  float n1, n2;
  if (ym::dot(w_i, n) < 0.0f) { n1 = ior; n2 = 1.0f; n = n * -1.0f; }
  else { n1 = 1.0f; n2 = ior; }
  const f4 perp = ym::div(n1, n2) * (ym::dot(w_i, n) * n - w_i);
  const float lp = ym::length(perp);
  const f4 par = ym::sqrt(ym::sub(1.0f, ym::mul(lp, lp))) * (-n);
  return ym::normalize(perp + par);
}

// evalFresnelReflectance, udpt.cl:992-1031
__device__ __forceinline__ float fresnel(f4 w_i, f4 n, const yc_material& m, float& ior_factor) {
  float n1, n2;
  if (ym::dot(w_i, n) < 0.0f) { n1 = m.n; n2 = 1.0f; n = n * -1.0f; }
  else { n1 = 1.0f; n2 = m.n; }
  const float cI = ym::dot(w_i, n);
  const float sI = ym::sqrt(ym::sub(1.0f, ym::mul(cI, cI)));
  const float sT = ym::div(ym::mul(n1, sI), n2);
  const float cT = ym::sqrt(ym::sub(1.0f, ym::mul(sT, sT)));
  if (sT >= 1.0f && n1 > n2) return 1.0f;
  const float r0 = ym::div(ym::add(ym::add(m.ks.x, m.ks.y), m.ks.z), 3.0f);
  ior_factor = ym::div(ym::mul(n2, n2), ym::mul(n1, n1));
  const float c = (n1 > n2) ? cI : cT;
  return ym::add(r0, ym::mul(ym::sub(1.0f, r0), ym::sub(1.0f, ym::pow(c, 5.0f))));
}

// normal-to-world rows (Nx.k, Ny.k, Nz.k, p.k) applied to (x, y, z, 0), then normalised
__device__ __forceinline__ f4 to_world(f4 Nx, f4 Ny, f4 Nz, f4 p, f4 d) {
  f4 o;
  o.x = ym::dot(ym::mk(Nx.x, Ny.x, Nz.x, p.x), d);
  o.y = ym::dot(ym::mk(Nx.y, Ny.y, Nz.y, p.y), d);
  o.z = ym::dot(ym::mk(Nx.z, Ny.z, Nz.z, p.z), d);
  o.w = 0.0f;
  return ym::normalize(o);
}

// phongSampleHemisphere, udpt.cl:700-771 (direction and pdf; origin = hp + dir * EPS)
__device__ __forceinline__ f4 sample_phong(const Vtx& v, const yc_material& m, f4 w_i, uint32_t& seed, float& pdf) {
  const f4 Nz = ym::normalize(reflect(w_i, v.n));
  f4 Nx, Ny;
  frame(Nz, Nx, Ny);
  const float r1 = draw(seed);
  const float r2 = draw(seed);
  const int pe = (int)ym::add(m.px, m.py);
  const float phi = ym::mul(ym::mul(2.0f, PI_F), r2);
  const float ct = ym::pow(r1, ym::div(1.0f, (float)(pe + 1)));
  float st = ym::sub(1.0f, ym::pow(r1, ym::div(2.0f, (float)(pe + 1))));
  st = ym::sqrt(st);
  const f4 d = ym::mk(ym::mul(st, ym::cos(phi)), ym::mul(st, ym::sin(phi)), ct, 0.0f);
  const f4 dir = to_world(Nx, Ny, Nz, v.hp, d);
  if (ym::dot(dir, v.n) < 0.0f) pdf = 0.0f;
  else pdf = (float)((double)(pe + 1) * 0.5 * (double)INV_PI_F * (double)ym::pow(ct, (float)pe));
  return dir;
}

// cosineWeightedHemisphere, udpt.cl:843-910
__device__ __forceinline__ f4 sample_cosine(const Vtx& v, uint32_t& seed, float& pdf) {
  f4 Nx, Ny;
  frame(v.n, Nx, Ny);
  const float r1 = draw(seed);
  const float r2 = draw(seed);
  const float phi = ym::mul(ym::mul(2.0f, PI_F), r2);
  const float sT = ym::sqrt(r1);
  const float z = ym::sqrt(ym::sub(1.0f, r1));
  const f4 d = ym::mk(ym::mul(sT, ym::cos(phi)), ym::mul(sT, ym::sin(phi)), z, 0.0f);
  const f4 dir = to_world(Nx, Ny, v.n, v.hp, d);
  pdf = ym::mul(z, INV_PI_F);
  return dir;
}

// calcPhongPDF, udpt.cl:1033-1045
__device__ __forceinline__ float phong_pdf(f4 w_i, f4 w_o, const Vtx& v, const yc_material& m) {
  f4 rd = ym::mul(2.0f, ym::dot(w_o, v.n)) * v.n - w_o;
  rd = ym::normalize(rd);
  const float ct = ym::fmax(0.0f, ym::cos(ym::dot(rd, w_i)));
  const float pe = ym::add(m.px, m.py);
  return (float)((double)ym::add(pe, 1.0f) * 0.5 * (double)INV_PI_F * (double)ym::pow(ct, pe));
}
// calcCosPDF, udpt.cl:1047-1050
__device__ __forceinline__ float cos_pdf(f4 w_i, f4 n) { return ym::mul(ym::fmax(ym::dot(w_i, n), 0.0f), INV_PI_F); }

// sampleGlossyPdf, udpt.cl:1062-1119
__device__ __forceinline__ bool sample_glossy(const yc_material& m, uint32_t& seed, float& prob) {
  const float r = draw(seed);
  const f4 ks = ld4(m.ks), kd = ld4(m.kd);
  if (ym::length3(ks) == 0.0f) { prob = 1.0f; return false; }
  if (ym::length3(kd) == 0.0f || ym::add(ym::add(kd.x, kd.y), kd.z) == 0.0f) { prob = 1.0f; return true; }
  const f4 sum = ks + kd;
  const float mx = ym::max(sum.x, ym::max(sum.y, sum.z));
  float pd, ps;
  if (mx == sum.x) { pd = kd.x; ps = ks.x; }
  else if (mx == sum.y) { pd = kd.y; ps = ks.y; }
  else { pd = kd.z; ps = ks.z; }
  if (r < pd) { prob = pd; return false; }
  if (r < ym::add(pd, ps) && r >= pd) { prob = ps; return true; }
  prob = 0.0f;
  return false;
}

// toShadingSpace + trig helpers, udpt-primitives.cl:1147-1210
__device__ __forceinline__ f4 to_shading(f4 w, const Vtx& v) {
  f4 Nx, Ny;
  frame(v.n, Nx, Ny);
  const f4 Nz = v.n;
  const f4 r1 = ym::mk(Nx.x, Nx.y, Nx.z, ym::dot(v.hp, Nx));
  const f4 r2 = ym::mk(Ny.x, Ny.y, Ny.z, ym::dot(v.hp, Ny));
  const f4 r3 = ym::mk(Nz.x, Nz.y, Nz.z, ym::dot(v.hp, Nz));
  const f4 r4 = ym::mk(0.0f, 0.0f, 0.0f, 1.0f);
  return ym::mk(ym::dot(r1, w), ym::dot(r2, w), ym::dot(r3, w), ym::dot(r4, w));
}
__device__ __forceinline__ float sin_theta(f4 w) { return ym::sqrt(ym::sub(1.0f, ym::mul(w.z, w.z))); }
__device__ __forceinline__ float cos_phi(f4 w) {
  const float st = sin_theta(w);
  if (st <= EPS_F && st >= -EPS_F) return 0.0f;
  return ym::clamp(ym::div(w.x, st), -1.0f, 1.0f);
}
__device__ __forceinline__ float sin_phi(f4 w) {
  const float st = sin_theta(w);
  if (st <= EPS_F && st >= -EPS_F) return 0.0f;
  return ym::clamp(ym::div(w.y, st), -1.0f, 1.0f);
}
// OrenNayarBRDF, udpt-primitives.cl:696-725 (alpha_x holds sigma^2). A and B (:722-723) depend on
// the material alone and are computed in double precision; oren_nayar_ab (host and
// device) is that computation, done once per material at upload (DevScene::on_ab), so a
// shading step runs no double-precision division.
__host__ __device__ inline float2 oren_nayar_ab(float alpha_x) {
  const double s2 = (double)alpha_x;
  float2 ab;
  ab.x = (float)(1 - (s2 / (2 * (s2 + 0.33))));
  ab.y = (float)(0.45 * s2 / (s2 + 0.09));
  return ab;
}
__device__ __forceinline__ f4 oren_nayar(f4 w_i, f4 w_o, const Vtx& v, const yc_material& m, float2 ab) {
  w_i = to_shading(w_i, v);
  w_o = to_shading(w_o, v);
  float costerm = 0.0f;
  if (sin_theta(w_i) >= EPS_F && sin_theta(w_o) >= EPS_F)
    costerm = ym::fmax(0.0f, ym::add(ym::mul(cos_phi(w_i), cos_phi(w_o)), ym::mul(sin_phi(w_i), sin_phi(w_o))));
  float sa, tb;
  if (ym::fabs(w_i.z) < ym::fabs(w_o.z)) { sa = sin_theta(w_i); tb = ym::div(sin_theta(w_o), ym::fabs(w_o.z)); }
  else { sa = sin_theta(w_o); tb = ym::div(sin_theta(w_i), ym::fabs(w_i.z)); }
  return (ld4(m.kd) * INV_PI_F) * ym::add(ab.x, ym::mul(ab.y, ym::mul(ym::mul(costerm, sa), tb)));
}

// evaluateBRDF, udpt.cl:611-630 (Oren-Nayar for a probability-1 diffuse lobe when
// brdf_model = 1, udpt-primitives.cl:673-686; on_ab: the scene's per-material A and B)
__device__ __forceinline__ f4 brdf(f4 w_i, f4 w_o, const Vtx& v, const yc_material& m, bool glossy, float rr_prob,
                                   int brdf_model, const float2* on_ab) {
  const f4 refl = ym::normalize(reflect(w_i, v.n));
  if (!glossy) {
    if (brdf_model == 1 && rr_prob == 1.0f) return oren_nayar(w_i, w_o, v, m, on_ab[v.mat]);
    return (ld4(m.kd) * INV_PI_F) / rr_prob;
  }
  const float ca = ym::pow(ym::fmax(ym::dot(w_o, refl), 0.0f), ym::add(m.px, m.py));
  const int pe = (int)ym::add(m.px, m.py);
  return ((((ld4(m.ks) * ca) * (float)(pe + 2)) * INV_PI_F) * 0.5f) / rr_prob;
}

// sampleLights, udpt.cl:632-698; -1 when no light is picked
__device__ __forceinline__ int sample_lights(const DevScene& sc, const Vtx& v, uint32_t& seed, float& light_pdf,
                                             f4& w_i) {
  // The reference keeps each light's sample and weight in arrays; here the weights are
  // summed in a first sweep and the chosen light's sample is drawn again in a second
  // sweep that replays the same xorshift stream, so nothing is spilled to local memory
  // and every value is computed by the same operations in the same order.
  const int n = sc.n_lights;
  const uint32_t seed0 = seed;
  float sum = 0.0f;
  for (int i = 0; i < n; ++i) {
    const yc_quad_light& L = sc.lights[i];
    const float r1 = draw(seed);
    const float r2 = draw(seed);
    f4 t = ((ld4(L.pos) + r1 * ld4(L.edge_l)) + r2 * ld4(L.edge_w)) - v.hp;
    const float distance = ym::dot(t, t);
    const f4 ti = t;
    t = ym::normalize(t);
    const f4 ln = ld4(L.normal);
    const float cf = ym::mul(ym::max(ym::dot(t, v.n), 0.0f), ym::max(ym::dot(-t, ln), 0.0f));
    if (cf <= 0.0f) continue;
    const float area = ym::mul(ym::length(ld4(L.edge_l)), ym::length(ld4(L.edge_w)));
    if (n == 1) {
      w_i = ti;
      light_pdf = ym::div(1.0f, area);
      light_pdf = ym::mul(light_pdf, ym::div(distance, ym::fmax(ym::dot(-t, ln), 0.0f)));
      return i;
    }
    sum = ym::add(sum, ym::div(ym::mul(ym::mul(ym::length(ld4(L.ke)), cf), area), distance));
  }
  if (sum == 0.0f) return -1;
  const float r1 = draw(seed);
  float cum = 0.0f;
  uint32_t replay = seed0;
  for (int i = 0; i < n; ++i) {
    const yc_quad_light& L = sc.lights[i];
    const float q1 = draw(replay);
    const float q2 = draw(replay);
    f4 t = ((ld4(L.pos) + q1 * ld4(L.edge_l)) + q2 * ld4(L.edge_w)) - v.hp;
    const float distance = ym::dot(t, t);
    const f4 ti = t;
    t = ym::normalize(t);
    const f4 ln = ld4(L.normal);
    const float cf = ym::mul(ym::max(ym::dot(t, v.n), 0.0f), ym::max(ym::dot(-t, ln), 0.0f));
    const float area = ym::mul(ym::length(ld4(L.edge_l)), ym::length(ld4(L.edge_w)));
    const float weight = cf <= 0.0f ? 0.0f : ym::div(ym::mul(ym::mul(ym::length(ld4(L.ke)), cf), area), distance);
    const float wgt = ym::div(weight, sum);
    if (r1 >= cum && r1 < ym::add(cum, wgt)) {
      w_i = ti;
      light_pdf = ym::div(wgt, area);
      light_pdf = ym::mul(light_pdf, ym::div(ym::dot(w_i, w_i), ym::fmax(ym::dot(-ym::normalize(w_i), ln), 0.0f)));
      return i;
    }
    cum = ym::add(cum, wgt);
  }
  return -1;
}

// ---- the BDPT variants (kernels/legacy/bdpt.cl) ----
// evaluateBRDF, bdpt.cl:718-737: reflection vector without the normal flip
__device__ __forceinline__ f4 brdf_b(f4 w_i, f4 w_o, f4 n, const yc_material& m, bool glossy, float rr_prob) {
  f4 refl = ym::mul(2.0f, ym::dot(w_i, n)) * n - w_i;
  refl = ym::normalize(refl);
  if (!glossy) return (ld4(m.kd) * INV_PI_F) / rr_prob;
  const float ca = ym::pow(ym::fmax(ym::dot(w_o, refl), 0.0f), ym::add(m.px, m.py));
  const int pe = (int)ym::add(m.px, m.py);
  return ((((ld4(m.ks) * ca) * (float)(pe + 2)) * INV_PI_F) * 0.5f) / rr_prob;
}

// phongSampleHemisphere, bdpt.cl:807-870: lobe axis without the normal flip
__device__ __forceinline__ f4 sample_phong_b(const Vtx& v, const yc_material& m, f4 w_i, uint32_t& seed, float& pdf) {
  f4 Nz = ym::mul(2.0f, ym::dot(w_i, v.n)) * v.n - w_i;
  Nz = ym::normalize(Nz);
  f4 Nx, Ny;
  frame(Nz, Nx, Ny);
  const float r1 = draw(seed);
  const float r2 = draw(seed);
  const int pe = (int)ym::add(m.px, m.py);
  const float phi = ym::mul(ym::mul(2.0f, PI_F), r2);
  const float ct = ym::pow(r1, ym::div(1.0f, (float)(pe + 1)));
  float st = ym::sub(1.0f, ym::pow(r1, ym::div(2.0f, (float)(pe + 1))));
  st = ym::sqrt(st);
  const f4 d = ym::mk(ym::mul(st, ym::cos(phi)), ym::mul(st, ym::sin(phi)), ct, 0.0f);
  const f4 dir = to_world(Nx, Ny, Nz, v.hp, d);
  if (ym::dot(dir, v.n) < 0.0f) pdf = 0.0f;
  else pdf = (float)((double)(pe + 1) * 0.5 * (double)INV_PI_F * (double)ym::pow(ct, (float)pe));
  return dir;
}

// sampleGlossyPdf, bdpt.cl:1048-1105: probabilities raised by (1 - max)/2, no absorption
__device__ __forceinline__ bool sample_glossy_b(const yc_material& m, uint32_t& seed, float& prob) {
  const float r = draw(seed);
  const f4 ks = ld4(m.ks), kd = ld4(m.kd);
  if (ym::length3(ks) == 0.0f) { prob = 1.0f; return false; }
  if (ym::length3(kd) == 0.0f || ym::add(ym::add(kd.x, kd.y), kd.z) == 0.0f) { prob = 1.0f; return true; }
  const f4 sum = ks + kd;
  const float mx = ym::max(sum.x, ym::max(sum.y, sum.z));
  float pd, ps;
  if (mx == sum.x) { pd = kd.x; ps = ks.x; }
  else if (mx == sum.y) { pd = kd.y; ps = ks.y; }
  else { pd = kd.z; ps = ks.z; }
  if (mx < 1.0f) {
    const float half = ym::div(ym::sub(1.0f, mx), 2.0f);
    pd = ym::add(pd, half);
    ps = ym::add(ps, half);
  }
  if (r < pd) { prob = pd; return false; }
  prob = ps;
  return true;
}

// getYluminance, udpt.cl:1121-1124
__device__ __forceinline__ float luminance(f4 c) {
  return ym::add(ym::add(ym::mul(0.212671f, c.x), ym::mul(0.715160f, c.y)), ym::mul(0.072169f, c.z));
}

// vertex of a triangle hit: hit point and interpolated normal (udpt.cl:377-383)
__device__ __forceinline__ Vtx tri_vertex(const DevScene& sc, f4 o, f4 d, float t, float u, float v, int tri) {
  Vtx x;
  x.hp = o + d * t;
  const float4* s = sc.shade + 4 * (size_t)tri;
  const f4 N1 = f4of(__ldg(s + 0)), N2 = f4of(__ldg(s + 1)), N3 = f4of(__ldg(s + 2));
  const float w = ym::sub(ym::sub(1.0f, u), v);
  x.n = ym::normalize((N1 * w + N2 * u) + N3 * v);
  x.mat = __float_as_int(__ldg(s + 3).x);
  return x;
}

}  // namespace yc
