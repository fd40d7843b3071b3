// udpt.cu -- wavefront form of the unidirectional path tracer (kernels/legacy/udpt.cl).
//
// The reference runs one work-item per pixel through `shading` (udpt.cl:433-533),
// calling traceRay 2-3 times per bounce. Here every path is a small state machine in
// HBM (PathState) and a pass is a sequence of rounds:
//   raygen (a)   -> primary rays into the closest-hit queue
//   trace        -> extend kernel (b) on the closest-hit queue, occlusion kernel on the
//                   any-hit queue (NEE shadow rays and MIS BRDF rays, (d))
//   logic        -> advances each path that got a result until it needs its next ray
//                   (shading (c), light sampling and MIS (d), Russian roulette); the new
//                   rays are appended to the next round's queues with one warp ballot +
//                   popc prefix and one atomic per warp (e), so finished paths drop out
//                   and the queues stay dense.
// A path that finishes writes its colour into the running-mean accumulator
// (udpt.cl:193-210). The random numbers of a path are drawn in the reference order,
// from the same per-pixel xorshift stream.
#include <cuda_runtime.h>

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

// ---- raygen: pathtracer prologue + createRay (udpt.cl:158-189, 213-238) ----
__global__ void __launch_bounds__(256) k_raygen(PassParams pp, PathState ps, int* q_closest, RoundCounters* rc,
                                                DevStats* st) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = pp.tile_w * pp.tile_h;
  const bool valid_thread = gid < n;
  int px = 0, py = 0;
  bool active = false;
  if (valid_thread) {
    px = gid % pp.tile_w + pp.off_x;
    py = gid / pp.tile_w + pp.off_y;
    active = px < pp.width && py < pp.height;
  }
  const int W = pp.width, H = pp.height;
  const int pix = py * W + px;
  if (active) {
    uint32_t seed = (uint32_t)((py + 1) * W + (px + 1));
    seed = pp.rand_seed * seed;
    seed = ym::wang_hash(seed);
    if (seed == 0) seed = ym::wang_hash(seed);
    const float r1 = draw(seed);
    const float r2 = draw(seed);
    const float fx = ym::add((float)px, r1), fy = ym::add((float)py, r2);
    const float aspect = (float)(((double)W * 1.0) / (double)H);
    f4 dir;
    dir.x = (float)((double)aspect * ((2.0 * (double)fx / (double)W) - 1));
    dir.y = (float)((2.0 * (double)fy / (double)H) - 1);
    dir.z = -pp.cam.view_plane_dist;
    dir.w = 0.0f;
    f4 d;
    d.x = ym::dot(ld4(pp.cam.r1), dir);
    d.y = ym::dot(ld4(pp.cam.r2), dir);
    d.z = ym::dot(ld4(pp.cam.r3), dir);
    d.w = ym::dot(ld4(pp.cam.r4), dir);
    d = ym::normalize(d);
    const f4 o = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
    float len = __int_as_float(0x7f800000);
    int k = -1;
    light_test(pp.sc, o, d, len, k);
    ps.misc[pix] = make_int4((int)seed, pix, pack_misc(S_PRIMARY, 0, -1, k), 0);
    ps.ro[pix] = make_float4(o.x, o.y, o.z, len);
    ps.rd[pix] = make_float4(d.x, d.y, d.z, d.w);
  }
  // warp-aggregated append of the active pixels to the closest-hit queue
  const unsigned m = __ballot_sync(0xffffffffu, active);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(&rc->n_closest, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (active) q_closest[base + __popc(m & ((1u << lane) - 1))] = pix;
  if (lane == 0 && m) {
    atomicAdd(&st->primary, (unsigned long long)__popc(m));
    atomicAdd(&st->rays, (unsigned long long)__popc(m));
    atomicAdd(&st->traversed, (unsigned long long)__popc(m));
  }
}

void launch_raygen(const PassParams& pp, const PathState& ps, int* q_closest, RoundCounters* rc, DevStats* st,
                   cudaStream_t s) {
  const int n = pp.tile_w * pp.tile_h;
  k_raygen<<<(n + 255) / 256, 256, 0, s>>>(pp, ps, q_closest, rc, st);
}

// ---- logic: one step of every path in the input queues ----
struct Emit {
  int kind;  // 0 none, 1 closest, 2 any-hit
};

__global__ void __launch_bounds__(LOGIC_TB) k_logic(PassParams pp, PathState ps, const int* __restrict__ in_closest,
                                                    const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                    int* out_closest, int* out_any, RoundCounters* rc_out,
                                                    DevStats* st) {
  __shared__ unsigned long long s_cnt[8];   // rays, extension, shadow, mis, traversed, samples
  if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int nc = rc_in->n_closest, na = rc_in->n_any;
  const int n = nc + na;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const DevScene& sc = pp.sc;
  const f4 BG = ym::mk(0.4f, 0.4f, 0.4f, 1.0f);
  const f4 PINK = ym::mk(0.988f, 0.0588f, 0.7529f, 1.0f);
  const float INF = __int_as_float(0x7f800000);

  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int e = wbase + lane;
    int emit = 0;
    int p = -1;
    unsigned c_rays = 0, c_ext = 0, c_shadow = 0, c_mis = 0, c_trav = 0, c_samples = 0;
    if (e < n) {
      p = e < nc ? in_closest[e] : in_any[e - nc];
      int4 misc = ps.misc[p];
      uint32_t seed = (uint32_t)misc.x;
      const int pix = misc.y;
      int phase = misc.z & 15;
      int flags = (misc.z >> 4) & 0xff;
      int j = ((misc.z >> 12) & 0xff) - 1;
      int k = ((misc.z >> 20) & 0xff) - 1;
      int bounce = misc.w;
      f4 thr = f4of(ps.thr[p]), thr_next = f4of(ps.thr_next[p]);
      f4 direct = f4of(ps.direct[p]), indirect = f4of(ps.indirect[p]);
      f4 ls = f4of(ps.ls[p]);
      const float4 hp4 = ps.hp[p], n4 = ps.nrm[p], wo4 = ps.wo[p], wi4 = ps.wi[p];
      Vtx V;
      V.hp = ym::mk(hp4.x, hp4.y, hp4.z, 1.0f);
      V.n = ym::mk(n4.x, n4.y, n4.z, 0.0f);
      V.mat = __float_as_int(wi4.w);
      float light_pdf = hp4.w, brdf_prob = n4.w, brdf_pdf = wo4.w;
      f4 wo = ym::mk(wo4.x, wo4.y, wo4.z, -0.0f);
      f4 w_i = ym::mk(wi4.x, wi4.y, wi4.z, 0.0f);
      const float4 ro4 = ps.ro[p], rd4 = ps.rd[p];
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
            ls = ym::splat(0.0f);
            flags &= ~(F_NEE_GLOSSY | F_OCCLUDED);
            c_rays++; c_shadow++;
            int lk = -1;
            float tl = len;
            light_test(sc, ro, rd, tl, lk);
            if (lk >= 0) {   // another light closes the segment: blocked without a BVH walk
              flags |= F_OCCLUDED;
              phase = S_NEE_SHADOW;
              break;
            }
            c_trav++;
            phase = S_NEE_SHADOW;
            emit = 2;
            done = true;
            break;
          }
          case S_NEE_SHADOW: {
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
              ls = (brdf(w_i, wo, V, m, glossy, brdf_prob, pp.brdf_model) * lke) * ym::fmax(ym::dot(w_i, V.n), 0.0f);
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
            c_rays++; c_mis++;
            // closest light along the BRDF ray; only light j can satisfy the test
            ro = V.hp + bdir * EPS_F;
            rd = bdir;
            float tl = INF;
            int lk = -1;
            light_test(sc, ro, rd, tl, lk);
            if (lk != j) { dl = ls + em; phase = P_NEE_DELIVER; break; }
            tmax = tl;
            c_trav++;
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
            f4 bs = (brdf(w_i, wo, V, m, glossy, brdf_prob, pp.brdf_model) * ld4(sc.lights[j].ke)) *
                    ym::fmax(ym::dot(w_i, V.n), 0.0f);
            bs = bs * ym::div(mw, brdf_pdf);
            dl = (ls + bs) + em;
            phase = P_NEE_DELIVER;
            break;
          }
          case P_NEE_DELIVER: {
            if (flags & F_TARGET_INDIRECT) indirect = indirect + thr * dl;
            else direct = dl;
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
            else thr_next = ((thr * brdf(nd, wo, V, m, glossy, prob, pp.brdf_model)) * ym::fmax(ym::dot(nd, V.n), 0.0f)) / pdf;
            flags = spec ? (flags | F_SPEC) : (flags & ~F_SPEC);
            ro = V.hp + nd * EPS_F;
            rd = nd;
            float tl = INF;
            int lk = -1;
            light_test(sc, ro, rd, tl, lk);
            k = lk;
            tmax = tl;
            c_rays++; c_ext++; c_trav++;
            phase = S_EXT;
            emit = 1;
            done = true;
            break;
          }
          case S_EXT: {   // rest of the GI iteration (udpt.cl:488-529)
            const int tri = __float_as_int(hit.w);
            const bool spec = (flags & F_SPEC) != 0;
            if (tri < 0) {
              if (spec && k >= 0) indirect = indirect + thr * ld4(sc.lights[k].ke);
              color = direct + indirect;
              phase = P_FINISH;
              break;
            }
            const Vtx NV = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            indirect = indirect + thr * ld4(sc.mats[NV.mat].ke);
            thr = thr_next;
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
            if (pp.reset == 1) {
              c.w = 1.0f;
            } else {
              const int np = (int)prev.w;
              c = c + f4of(prev) * (float)np;
              c = c / (float)(np + 1);
              c.w = (float)(np + 1);
            }
            pp.accum[pix] = make_float4(c.x, c.y, c.z, c.w);
            c_samples++;
            done = true;
            break;
          }
        }
      }
      if (emit) {
        ps.misc[p] = make_int4((int)seed, pix, pack_misc(phase, flags, j, k), bounce);
        ps.thr[p] = make_float4(thr.x, thr.y, thr.z, thr.w);
        ps.thr_next[p] = make_float4(thr_next.x, thr_next.y, thr_next.z, thr_next.w);
        ps.direct[p] = make_float4(direct.x, direct.y, direct.z, direct.w);
        ps.indirect[p] = make_float4(indirect.x, indirect.y, indirect.z, indirect.w);
        ps.ls[p] = make_float4(ls.x, ls.y, ls.z, ls.w);
        ps.hp[p] = make_float4(V.hp.x, V.hp.y, V.hp.z, light_pdf);
        ps.nrm[p] = make_float4(V.n.x, V.n.y, V.n.z, brdf_prob);
        ps.wo[p] = make_float4(wo.x, wo.y, wo.z, brdf_pdf);
        ps.wi[p] = make_float4(w_i.x, w_i.y, w_i.z, __int_as_float(V.mat));
        ps.ro[p] = make_float4(ro.x, ro.y, ro.z, tmax);
        ps.rd[p] = make_float4(rd.x, rd.y, rd.z, rd.w);
      }
    }
    // compaction: ballot + popc prefix per queue, one atomic per warp and queue
    const unsigned mc = __ballot_sync(0xffffffffu, emit == 1);
    const unsigned ma = __ballot_sync(0xffffffffu, emit == 2);
    int bc = 0, ba = 0;
    if (lane == 0) {
      if (mc) bc = atomicAdd(&rc_out->n_closest, __popc(mc));
      if (ma) ba = atomicAdd(&rc_out->n_any, __popc(ma));
    }
    bc = __shfl_sync(0xffffffffu, bc, 0);
    ba = __shfl_sync(0xffffffffu, ba, 0);
    const unsigned below = (1u << lane) - 1;
    if (emit == 1) out_closest[bc + __popc(mc & below)] = p;
    if (emit == 2) out_any[ba + __popc(ma & below)] = p;
    // counters
    unsigned v[6] = {c_rays, c_ext, c_shadow, c_mis, c_trav, c_samples};
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      unsigned x = v[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
      if (lane == 0 && x) atomicAdd(&s_cnt[q], (unsigned long long)x);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_cnt[0]) atomicAdd(&st->rays, s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&st->extension, s_cnt[1]);
    if (s_cnt[2]) atomicAdd(&st->shadow, s_cnt[2]);
    if (s_cnt[3]) atomicAdd(&st->mis, s_cnt[3]);
    if (s_cnt[4]) atomicAdd(&st->traversed, s_cnt[4]);
    if (s_cnt[5]) atomicAdd(&st->samples, s_cnt[5]);
  }
}

void launch_logic(const PassParams& pp, const PathState& ps, const int* in_closest, const int* in_any,
                  const RoundCounters* rc_in, int* out_closest, int* out_any, RoundCounters* rc_out, DevStats* st,
                  int grid, cudaStream_t s) {
  k_logic<<<grid, LOGIC_TB, 0, s>>>(pp, ps, in_closest, in_any, rc_in, out_closest, out_any, rc_out, st);
}

// ---- tonemap (kernels/post-proc/tonemap.cl:14-47) ----
__global__ void k_tonemap(const float4* __restrict__ in, float4* __restrict__ out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 c = in[i];
  float y = ym::mul(0.212671f, c.x);
  y = ym::add(y, ym::mul(0.715160f, c.y));
  y = ym::add(y, ym::mul(0.072169f, c.z));
  y = ym::add(y, 0.001f);
  const float ldv = ym::div(ym::mul(y, ym::add(1.0f, ym::div(y, ym::mul(1.0f, 1.0f)))), ym::add(1.0f, y));
  const float g = ym::div(1.0f, 2.2f);
  float r[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) r[q] = ym::pow(ym::mul(ldv, ym::pow(ym::div(r[q], y), 1.0f)), g);
  out[i] = make_float4(r[0], r[1], r[2], r[3]);
}

void launch_tonemap(const float4* in, float4* out, int n, cudaStream_t s) {
  k_tonemap<<<(n + 255) / 256, 256, 0, s>>>(in, out, n);
}

}  // namespace yc
