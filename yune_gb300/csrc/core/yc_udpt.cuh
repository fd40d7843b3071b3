// yc_udpt.cuh -- the unidirectional path's per-path device logic (kernels/legacy/udpt.cl),
// shared by the per-pass kernels (udpt.cu) and the batch engine (engine.cu).
#pragma once

#include "yc_internal.h"
#include "yc_shade.cuh"

namespace yc {

enum : int {
  S_PRIMARY = 0,     // waiting for the closest hit of the camera ray
  S_NEE_SHADOW = 1,  // waiting for the shadow ray of evaluateDirectLighting
  S_NEE_MIS = 2,     // waiting for the MIS BRDF ray (any-hit up to the sampled light)
  S_EXT = 3,         // waiting for the closest hit of the GI extension ray
  // transient phases
  P_NEE_BEGIN = 8,
  P_NEE_DELIVER = 9,
  P_GI_SAMPLE = 10,
  P_FINISH = 11
};
enum : int {
  F_TARGET_INDIRECT = 1,  // NEE result goes to indirect += thr * DL (udpt.cl:527) else direct = DL
  F_NEE_GLOSSY = 2,       // sample_glossy of the NEE (udpt.cl:559)
  F_SPEC = 4,             // the pending extension ray left a specular vertex
  F_OCCLUDED = 8          // the NEE shadow ray was blocked
};

__device__ __forceinline__ int pack_misc(int state, int flags, int j, int k) {
  return state | (flags << 4) | ((j + 1) << 12) | ((k + 1) << 20);
}

constexpr int LOGIC_TB = 256;

struct LogicCounts {
  unsigned rays = 0, ext = 0, shadow = 0, mis = 0, trav = 0, samples = 0, prim = 0;
};

// ---- raygen: pathtracer prologue + createRay (udpt.cl:158-189, 213-238) ----
// seed of pixel (px, py) for pass seed `rand`, the camera ray, and the closest light
// along it (the light loop of traceRay runs before the BVH, udpt.cl:244-276)
__device__ __forceinline__ void camera_ray(const PassParams& pp, int px, int py, uint32_t rand, uint32_t& seed, f4& o, f4& d,
                           float& len, int& k) {
  const int W = pp.width, H = pp.height;
  seed = (uint32_t)((py + 1) * W + (px + 1));
  seed = rand * seed;
  seed = ym::wang_hash(seed);
  if (seed == 0) seed = ym::wang_hash(seed);
  const float r1 = draw(seed);
  const float r2 = draw(seed);
  const float fx = ym::add((float)px, r1), fy = ym::add((float)py, r2);
  const float aspect = pp.aspect;
  f4 dir;
  dir.x = (float)((double)aspect * ((2.0 * (double)fx / (double)W) - 1));
  dir.y = (float)((2.0 * (double)fy / (double)H) - 1);
  dir.z = -pp.cam.view_plane_dist;
  dir.w = 0.0f;
  d.x = ym::dot(ld4(pp.cam.r1), dir);
  d.y = ym::dot(ld4(pp.cam.r2), dir);
  d.z = ym::dot(ld4(pp.cam.r3), dir);
  d.w = ym::dot(ld4(pp.cam.r4), dir);
  d = ym::normalize(d);
  o = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
  len = __int_as_float(0x7f800000);
  k = -1;
  light_test(pp.sc, o, d, len, k);
}

// Fields of the path record a step rewrote (stored back when the step emits a ray).
enum : unsigned {
  D_THR = 1, D_THR_NEXT = 2, D_DIRECT = 4, D_INDIRECT = 8, D_LS = 16, D_HP = 32, D_NRM = 64, D_WO = 128, D_WI = 256
};

// One step of path p: runs its state machine from the result of its last ray until it
// needs the next one. Returns 1 (closest-hit ray written to the path state), 2 (any-hit
// ray) or 0 (the path finished and its colour went into the accumulator).
// The step loads only the record fields its entry state can read before writing them
// (a camera-ray result reads the ray and the hit; an extension result does not read the
// last vertex's shading frame, light sample or densities; a shadow or MIS result does not
// read the ray it traced) and stores only the fields it changed: the record is the same,
// with fewer bytes moved (pass starts write the misc word and the ray only).
__device__ __forceinline__ int logic_path(const PassParams& pp, int reset, const PathState& ps, int p, LogicCounts& cnt) {
  const DevScene& sc = pp.sc;
  const f4 BG = ym::mk(0.4f, 0.4f, 0.4f, 1.0f);
  const f4 PINK = ym::mk(0.988f, 0.0588f, 0.7529f, 1.0f);
  const float INF = __int_as_float(0x7f800000);
  int emit = 0;
  int4 misc = ps.misc[p];
  uint32_t seed = (uint32_t)misc.x;
  const int pix = misc.y;
  int phase = misc.z & 15;
  int flags = (misc.z >> 4) & 0xff;
  int j = ((misc.z >> 12) & 0xff) - 1;
  int k = ((misc.z >> 20) & 0xff) - 1;
  int bounce = misc.w;
  const bool enter_cam = phase == S_PRIMARY, enter_ext = phase == S_EXT;
  const bool enter_nee = phase == S_NEE_SHADOW || phase == S_NEE_MIS;
  unsigned dirty = 0;
  const float4 Z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  f4 thr = f4of(enter_cam ? Z4 : ps.thr[p]);
  f4 thr_next = f4of(enter_ext ? ps.thr_next[p] : Z4);
  f4 direct = f4of(enter_cam ? Z4 : ps.direct[p]), indirect = f4of(enter_cam ? Z4 : ps.indirect[p]);
  f4 ls = f4of(phase == S_NEE_MIS ? ps.ls[p] : Z4);
  const float4 hp4 = enter_nee ? ps.hp[p] : Z4, n4 = enter_nee ? ps.nrm[p] : Z4;
  const float4 wo4 = enter_nee ? ps.wo[p] : Z4, wi4 = enter_nee ? ps.wi[p] : Z4;
  Vtx V;
  V.hp = ym::mk(hp4.x, hp4.y, hp4.z, 1.0f);
  V.n = ym::mk(n4.x, n4.y, n4.z, 0.0f);
  V.mat = __float_as_int(wi4.w);
  float light_pdf = hp4.w, brdf_prob = n4.w, brdf_pdf = wo4.w;
  f4 wo = ym::mk(wo4.x, wo4.y, wo4.z, -0.0f);
  f4 w_i = ym::mk(wi4.x, wi4.y, wi4.z, 0.0f);
  const float4 ro4 = enter_nee ? Z4 : ps.ro[p], rd4 = enter_nee ? Z4 : ps.rd[p];
  f4 ro = ym::mk(ro4.x, ro4.y, ro4.z, 1.0f);
  f4 rd = ym::mk(rd4.x, rd4.y, rd4.z, rd4.w);
  float tmax = ro4.w;
  const float4 hit = ps.hit[p];
  f4 dl = ym::splat(0.0f);   // result of evaluateDirectLighting being delivered
  f4 color = ym::splat(0.0f);
  bool done = false;

  for (int guard = 0; guard < 64 && !done; ++guard) {
    switch (phase) {
      case S_PRIMARY: {
        const int tri = __float_as_int(hit.w);
        if (tri >= 0) {
          V = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
          thr = ym::mk(1.0f, 1.0f, 1.0f, 1.0f);
          direct = ym::mk(0.0f, 0.0f, 0.0f, 0.0f);
          indirect = direct;
          bounce = 0;
          wo = -rd;
          flags = 0;
          dirty |= D_THR | D_DIRECT | D_INDIRECT | D_HP | D_NRM | D_WO | D_WI;
          if (!sc.mats[V.mat].is_specular) phase = P_NEE_BEGIN;
          else phase = pp.gi_check ? P_GI_SAMPLE : P_FINISH;
          if (phase == P_FINISH) color = direct + indirect;
        } else if (k >= 0) {
          color = (ym::dot(rd, ld4(sc.lights[k].normal)) < 0.0f) ? ym::mk(1.0f, 1.0f, 1.0f, 1.0f)
                                                                 : ym::mk(0.1f, 0.1f, 0.1f, 1.0f);
          phase = P_FINISH;
        } else {
          color = BG;
          phase = P_FINISH;
        }
        break;
      }
      case P_NEE_BEGIN: {   // evaluateDirectLighting up to the shadow ray (udpt.cl:535-553)
        const yc_material& m = sc.mats[V.mat];
        f4 wi_raw;
        j = sample_lights(sc, V, seed, light_pdf, wi_raw);
        dirty |= D_HP;   // light_pdf
        if (j == -1 || light_pdf <= 0.0f) {
          dl = ld4(m.ke);
          phase = P_NEE_DELIVER;
          break;
        }
        float len = ym::length(wi_raw);
        len = ym::sub(len, ym::mul(EPS_F, 1.5f));
        w_i = ym::normalize(wi_raw);
        ro = V.hp + w_i * EPS_F;
        rd = w_i;
        tmax = len;
        flags &= ~(F_NEE_GLOSSY | F_OCCLUDED);
        dirty |= D_WI;
        cnt.rays++; cnt.shadow++;
        int lk = -1;
        float tl = len;
        light_test(sc, ro, rd, tl, lk);
        if (lk >= 0) {   // another light closes the segment: blocked without a BVH walk
          flags |= F_OCCLUDED;
          phase = S_NEE_SHADOW;
          break;
        }
        cnt.trav++;
        phase = S_NEE_SHADOW;
        emit = 2;
        done = true;
        break;
      }
      case S_NEE_SHADOW: {
        ls = ym::splat(0.0f);   // the light sample of this shadow ray (zero while occluded)
        dirty |= D_LS | D_NRM | D_WO;   // ls, brdf_prob, brdf_pdf
        if (hit.x != 0.0f) flags |= F_OCCLUDED;
        const yc_material& m = sc.mats[V.mat];
        const f4 em = ld4(m.ke);
        const f4 lke = ld4(sc.lights[j].ke);
        const bool occluded = (flags & F_OCCLUDED) != 0;
        bool glossy = false;
        brdf_prob = 0.0f;
        if (!occluded) {
          glossy = sample_glossy(m, seed, brdf_prob);
          if (brdf_prob == 0.0f) { dl = em; phase = P_NEE_DELIVER; break; }
          ls = (brdf(w_i, wo, V, m, glossy, brdf_prob, pp.brdf_model, sc.on_ab) * lke) * ym::fmax(ym::dot(w_i, V.n), 0.0f);
          ls = ls * ym::div(1.0f, light_pdf);
        }
        if (!pp.mis) { dl = ls + em; phase = P_NEE_DELIVER; break; }
        if (occluded && pp.mis_lobe_fix) {
          glossy = sample_glossy(m, seed, brdf_prob);
          if (brdf_prob == 0.0f) { dl = ls + em; phase = P_NEE_DELIVER; break; }
        }
        if (glossy) flags |= F_NEE_GLOSSY; else flags &= ~F_NEE_GLOSSY;
        brdf_pdf = glossy ? phong_pdf(w_i, wo, V, m) : cos_pdf(w_i, V.n);
        float mw = light_pdf;
        mw = ym::div(ym::mul(mw, mw), ym::add(ym::mul(light_pdf, light_pdf), ym::mul(brdf_pdf, brdf_pdf)));
        ls = ls * mw;
        f4 bdir;
        if (glossy) bdir = sample_phong(V, m, wo, seed, brdf_pdf);
        else bdir = sample_cosine(V, seed, brdf_pdf);
        if (brdf_pdf <= 0.0f) { dl = ls + em; phase = P_NEE_DELIVER; break; }
        w_i = bdir;
        dirty |= D_WI;
        cnt.rays++; cnt.mis++;
        // closest light along the BRDF ray; only light j can satisfy the test
        ro = V.hp + bdir * EPS_F;
        rd = bdir;
        float tl = INF;
        int lk = -1;
        light_test(sc, ro, rd, tl, lk);
        if (lk != j) { dl = ls + em; phase = P_NEE_DELIVER; break; }
        tmax = tl;
        cnt.trav++;
        phase = S_NEE_MIS;
        emit = 2;
        done = true;
        break;
      }
      case S_NEE_MIS: {
        const yc_material& m = sc.mats[V.mat];
        const f4 em = ld4(m.ke);
        if (hit.x != 0.0f) { dl = ls + em; phase = P_NEE_DELIVER; break; }
        const bool glossy = (flags & F_NEE_GLOSSY) != 0;
        float mw = brdf_pdf;
        mw = ym::div(ym::mul(mw, mw), ym::add(ym::mul(light_pdf, light_pdf), ym::mul(brdf_pdf, brdf_pdf)));
        f4 bs = (brdf(w_i, wo, V, m, glossy, brdf_prob, pp.brdf_model, sc.on_ab) * ld4(sc.lights[j].ke)) *
                ym::fmax(ym::dot(w_i, V.n), 0.0f);
        bs = bs * ym::div(mw, brdf_pdf);
        dl = (ls + bs) + em;
        phase = P_NEE_DELIVER;
        break;
      }
      case P_NEE_DELIVER: {
        if (flags & F_TARGET_INDIRECT) { indirect = indirect + thr * dl; dirty |= D_INDIRECT; }
        else { direct = dl; dirty |= D_DIRECT; }
        if (!pp.gi_check) { color = direct + indirect; phase = P_FINISH; }
        else phase = P_GI_SAMPLE;
        break;
      }
      case P_GI_SAMPLE: {   // one iteration of the GI loop up to its traceRay (udpt.cl:463-488)
        if (bounce >= pp.max_depth) { color = direct + indirect; phase = P_FINISH; break; }
        const yc_material& m = sc.mats[V.mat];
        const bool spec = m.is_specular != 0;
        float pdf = 1.0f, ior = 1.0f, prob = 0.0f;
        bool glossy = false;
        f4 nd;
        if (spec) {
          // sampleFresnelIncidence, udpt.cl:912-947
          if (m.is_transmissive) {
            const float fr = fresnel(wo, V.n, m, ior);
            if (fr == 1.0f) { nd = reflect(wo, V.n); ior = 1.0f; }
            else {
              const float r = draw(seed);
              if (r < fr) { nd = reflect(wo, V.n); ior = 1.0f; }
              else nd = refract(wo, V.n, m.n);
            }
          } else {
            ior = 1.0f;
            nd = reflect(wo, V.n);
          }
        } else {
          glossy = sample_glossy(m, seed, prob);
          if (prob == 0.0f) { color = direct + indirect; phase = P_FINISH; break; }
          if (glossy) nd = sample_phong(V, m, wo, seed, pdf);
          else nd = sample_cosine(V, seed, pdf);
        }
        if (pdf <= 0.0f) { color = direct + indirect; phase = P_FINISH; break; }
        if (spec) thr_next = thr * ior;
        else thr_next = ((thr * brdf(nd, wo, V, m, glossy, prob, pp.brdf_model, sc.on_ab)) * ym::fmax(ym::dot(nd, V.n), 0.0f)) / pdf;
        dirty |= D_THR_NEXT;
        flags = spec ? (flags | F_SPEC) : (flags & ~F_SPEC);
        ro = V.hp + nd * EPS_F;
        rd = nd;
        float tl = INF;
        int lk = -1;
        light_test(sc, ro, rd, tl, lk);
        k = lk;
        tmax = tl;
        cnt.rays++; cnt.ext++; cnt.trav++;
        phase = S_EXT;
        emit = 1;
        done = true;
        break;
      }
      case S_EXT: {   // rest of the GI iteration (udpt.cl:488-529)
        const int tri = __float_as_int(hit.w);
        const bool spec = (flags & F_SPEC) != 0;
        if (tri < 0) {
          if (spec && k >= 0) { indirect = indirect + thr * ld4(sc.lights[k].ke); dirty |= D_INDIRECT; }
          color = direct + indirect;
          phase = P_FINISH;
          break;
        }
        const Vtx NV = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
        indirect = indirect + thr * ld4(sc.mats[NV.mat].ke);
        thr = thr_next;
        dirty |= D_THR | D_INDIRECT | D_HP | D_NRM | D_WO | D_WI;   // new vertex
        if (bounce > pp.rr_threshold) {
          const float pr = ym::min(luminance(thr), 0.95f);
          const float r = draw(seed);
          if (r >= pr) { color = direct + indirect; phase = P_FINISH; break; }
          thr = thr * ym::div(1.0f, pr);
        }
        V = NV;
        wo = -rd;
        ++bounce;
        if (!sc.mats[V.mat].is_specular) { flags |= F_TARGET_INDIRECT; phase = P_NEE_BEGIN; }
        else phase = P_GI_SAMPLE;
        break;
      }
      case P_FINISH:
      default: {
        if (ym::any_nan(color)) color = PINK;
        const float4 prev = pp.accum[pix];
        f4 c = color;
        if (reset == 1) {
          c.w = 1.0f;
        } else {
          const int np = (int)prev.w;
          c = c + f4of(prev) * (float)np;
          c = c / (float)(np + 1);
          c.w = (float)(np + 1);
        }
        pp.accum[pix] = make_float4(c.x, c.y, c.z, c.w);
        cnt.samples++;
        done = true;
        break;
      }
    }
  }
  if (emit) {
    ps.misc[p] = make_int4((int)seed, pix, pack_misc(phase, flags, j, k), bounce);
    if (dirty & D_THR) ps.thr[p] = make_float4(thr.x, thr.y, thr.z, thr.w);
    if (dirty & D_THR_NEXT) ps.thr_next[p] = make_float4(thr_next.x, thr_next.y, thr_next.z, thr_next.w);
    if (dirty & D_DIRECT) ps.direct[p] = make_float4(direct.x, direct.y, direct.z, direct.w);
    if (dirty & D_INDIRECT) ps.indirect[p] = make_float4(indirect.x, indirect.y, indirect.z, indirect.w);
    if (dirty & D_LS) ps.ls[p] = make_float4(ls.x, ls.y, ls.z, ls.w);
    if (dirty & D_HP) ps.hp[p] = make_float4(V.hp.x, V.hp.y, V.hp.z, light_pdf);
    if (dirty & D_NRM) ps.nrm[p] = make_float4(V.n.x, V.n.y, V.n.z, brdf_prob);
    if (dirty & D_WO) ps.wo[p] = make_float4(wo.x, wo.y, wo.z, brdf_pdf);
    if (dirty & D_WI) ps.wi[p] = make_float4(w_i.x, w_i.y, w_i.z, __int_as_float(V.mat));
    ps.ro[p] = make_float4(ro.x, ro.y, ro.z, tmax);
    ps.rd[p] = make_float4(rd.x, rd.y, rd.z, rd.w);
  }
  return emit;
}

}  // namespace yc
