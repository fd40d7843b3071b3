// bdpt.cu -- wavefront form of Yune's naive bidirectional path tracer
// (kernels/legacy/bdpt.cl:158-640), step (f) of the pipeline.
//
// Per sample the reference builds a light subpath (createLightPath, bdpt.cl:432-511),
// an eye subpath (createEyePath, bdpt.cl:513-560), then for every eye vertex adds its
// emission and next-event estimate and connects it to every light vertex j >= 1 with a
// shadow ray (shading, bdpt.cl:562-640). Here each path is a state machine like the
// unidirectional one (udpt.cu): the logic kernel advances it to its next ray, the extend
// and occlusion kernels trace the queues, and the subpath vertices live in HBM as one
// 64-byte record per vertex (two full 32-byte sectors: a connection reads two vertices of
// a path whose neighbours in the queue are unrelated), vertex k of path p at
// [(p * bounces + k) * 4 + field]:
//   field 0: hit point xyz, material index (int bits)
//   field 1: shading normal xyz
//   field 2: direction of the ray that reached the vertex xyz
//   field 3: contrib (the subpath throughput, float4)
// Random numbers are drawn in the reference order from the same per-pixel stream.
// One departure, shared with the CPU oracle: a camera ray that hits the light ends the
// eye path (the reference keeps extending it from a vertex with triangle_ID = -1 and
// reads scene_data[-1]; the pixel colour is fixed to white or grey either way).
#include <cuda_runtime.h>

#include "yc_bdpt.h"
#include "yc_shade.cuh"

namespace yc {

enum : int { BF_GLOSSY = 1, BF_OCCLUDED = 2 };

// The BRDF and Phong-lobe helpers of the logic kernel, inlined or called (BDPT_HELPER).
#define BDPT_HELPER __forceinline__
__device__ BDPT_HELPER f4 brdf_bk(f4 w_i, f4 w_o, f4 n, const yc_material& m, bool glossy, float rr_prob) {
  return brdf_b(w_i, w_o, n, m, glossy, rr_prob);
}
__device__ BDPT_HELPER f4 sample_phong_bk(const Vtx& v, const yc_material& m, f4 w_i, uint32_t& seed, float& pdf) {
  return sample_phong_b(v, m, w_i, seed, pdf);
}

struct BCount {
  int i, j, lp, ep;
};
__device__ __forceinline__ int pack_cnt(const BCount& c) { return c.i | (c.j << 6) | (c.lp << 12) | (c.ep << 18); }
__device__ __forceinline__ BCount unpack_cnt(int v) {
  return BCount{v & 63, (v >> 6) & 63, (v >> 12) & 63, (v >> 18) & 63};
}
__device__ __forceinline__ int pack_st(int state, int flags, int lj, int k) {
  return state | (flags << 4) | ((lj + 1) << 8) | ((k + 1) << 13);
}

struct VertexRef {
  float4* base;     // the path's first vertex
  __device__ __forceinline__ float4& at(int k, int f) const { return base[(size_t)k * 4 + f]; }
  __device__ __forceinline__ void store(int k, const Vtx& v, f4 dir, f4 contrib) const {
    at(k, 0) = make_float4(v.hp.x, v.hp.y, v.hp.z, __int_as_float(v.mat));
    at(k, 1) = make_float4(v.n.x, v.n.y, v.n.z, 0.0f);
    at(k, 2) = make_float4(dir.x, dir.y, dir.z, 0.0f);
    at(k, 3) = make_float4(contrib.x, contrib.y, contrib.z, contrib.w);
  }
  __device__ __forceinline__ Vtx vtx(int k) const {
    const float4 a = at(k, 0), b = at(k, 1);
    Vtx v;
    v.hp = ym::mk(a.x, a.y, a.z, 1.0f);
    v.n = ym::mk(b.x, b.y, b.z, 0.0f);
    v.mat = __float_as_int(a.w);
    return v;
  }
  __device__ __forceinline__ f4 dir(int k) const { const float4 d = at(k, 2); return ym::mk(d.x, d.y, d.z, 0.0f); }
  __device__ __forceinline__ f4 contrib(int k) const { return f4of(at(k, 3)); }
};

// ---- raygen: pixel prologue, eye ray, light vertex 0 and the first light ray ----
__global__ void __launch_bounds__(256) k_raygen_bdpt(PassParams pp, PathState ps, BdptBuffers bb, int* q_closest,
                                                     RoundCounters* rc, DevStats* st) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = pp.tile_w * pp.tile_h;
  int px = 0, py = 0;
  bool active = false;
  if (gid < n) {
    px = gid % pp.tile_w + pp.off_x;
    py = gid / pp.tile_w + pp.off_y;
    active = px < pp.width && py < pp.height;
  }
  const int W = pp.width, H = pp.height;
  const int pix = py * W + px;
  const int slot = pix;
  bool eye_first = false;
  if (active) {
    const DevScene& sc = pp.sc;
    uint32_t seed = (uint32_t)((py + 1) * W + (px + 1));
    seed = pp.rand_seed * seed;
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
    f4 d;
    d.x = ym::dot(ld4(pp.cam.r1), dir);
    d.y = ym::dot(ld4(pp.cam.r2), dir);
    d.z = ym::dot(ld4(pp.cam.r3), dir);
    d.w = ym::dot(ld4(pp.cam.r4), dir);
    d = ym::normalize(d);
    VertexRef ev{bb.ev + (size_t)slot * bb.bounces * 4};
    VertexRef lv{bb.lv + (size_t)slot * bb.bounces * 4};
    ev.at(0, 2) = make_float4(d.x, d.y, d.z, d.w);   // the camera ray, traced after the light subpath
    // light vertex 0 on light 0 (createLightPath, bdpt.cl:435-456)
    const yc_quad_light& L = sc.lights[0];
    seed = ym::xor_shift(seed);
    const float lr1 = (float)((double)seed / 4294967295.0);   // seed / (double)UINT_MAX
    const float lr2 = draw(seed);
    const f4 A = ld4(L.edge_l) * lr2;
    const f4 B = ld4(L.edge_w) * lr1;
    Vtx v0;
    v0.hp = (A + B) + ld4(L.pos);
    v0.n = ld4(L.normal);
    v0.mat = -1;
    const float area = ym::mul(ym::length(ld4(L.edge_l)), ym::length(ld4(L.edge_w)));
    const float fwd = ym::div(1.0f, area);
    const f4 c0 = ld4(L.ke) / fwd;
    lv.at(0, 0) = make_float4(v0.hp.x, v0.hp.y, v0.hp.z, __int_as_float(-1));
    lv.at(0, 1) = make_float4(v0.n.x, v0.n.y, v0.n.z, v0.n.w);
    lv.at(0, 3) = make_float4(c0.x, c0.y, c0.z, c0.w);
    float pdf = 1.0f;
    const f4 ldir = sample_cosine(v0, seed, pdf);
    BCount cnt{1, 0, 1, 1};
    f4 o, rdir;
    int state;
    if (pdf <= 0.0f) {
      o = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
      rdir = d;
      state = B_EYE0;
      cnt.i = 0;
      eye_first = true;
    } else {
      o = v0.hp + ldir * EPS_F;
      rdir = ldir;
      state = B_LIGHT;
    }
    float len = __int_as_float(0x7f800000);
    int k = -1;
    light_test(sc, o, rdir, len, k);
    ps.misc[slot] = make_int4((int)seed, pix, pack_st(state, 0, -1, k), pack_cnt(cnt));
    ps.ro[slot] = make_float4(o.x, o.y, o.z, len);
    ps.rd[slot] = make_float4(rdir.x, rdir.y, rdir.z, rdir.w);
    ps.direct[slot] = make_float4(1.0f, 0.0f, pdf, 0.0f);   // weight, ks, pending pdf, pending lobe prob
  }
  const unsigned m = __ballot_sync(0xffffffffu, active);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == 0 && m) base = atomicAdd(&rc->n_closest, __popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (active) q_closest[base + __popc(m & ((1u << lane) - 1))] = slot;
  const unsigned m_eye = __ballot_sync(0xffffffffu, active && eye_first);
  if (lane == 0 && m) {
    atomicAdd(&st->rays, (unsigned long long)__popc(m));
    atomicAdd(&st->traversed, (unsigned long long)__popc(m));
    if (m_eye) atomicAdd(&st->primary, (unsigned long long)__popc(m_eye));
    if (m & ~m_eye) atomicAdd(&st->extension, (unsigned long long)__popc(m & ~m_eye));
  }
}

void launch_raygen_bdpt(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, int* q_closest,
                        RoundCounters* rc, DevStats* st, cudaStream_t s) {
  const int n = pp.tile_w * pp.tile_h;
  k_raygen_bdpt<<<(n + 255) / 256, 256, 0, s>>>(pp, ps, bb, q_closest, rc, st);
}

// ---- logic: advance each path to its next ray ----
__global__ void __launch_bounds__(256) k_logic_bdpt(PassParams pp, PathState ps, BdptBuffers bb,
                                                    const int* __restrict__ in_closest, const int* __restrict__ in_any,
                                                    const RoundCounters* rc_in, int* out_closest, int* out_any,
                                                    RoundCounters* rc_out, DevStats* st, const int* __restrict__ sorted,
                                                    const SortCtl* sctl) {
  __shared__ unsigned long long s_cnt[8];   // rays, primary, extension, shadow, connection, traversed, samples
  if (threadIdx.x < 8) s_cnt[threadIdx.x] = 0;
  __syncthreads();
  const int nc = rc_in->n_closest, na = rc_in->n_any;
  const int n = nc + na;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const DevScene& sc = pp.sc;
  const float INF = __int_as_float(0x7f800000);
  const int BOUNCES = bb.bounces;
  const int RR = 4;   // RR_THRESHOLD of bdpt.cl:4
  const bool use_sorted = sctl && sctl->use;

  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int e = wbase + lane;
    int emit = 0;
    int p = -1;
    unsigned c[7] = {0, 0, 0, 0, 0, 0, 0};
    if (e < n) {
      p = use_sorted ? sorted[e] : (e < nc ? in_closest[e] : in_any[e - nc]);
      const VertexRef lv{bb.lv + (size_t)p * bb.bounces * 4};
      const VertexRef ev{bb.ev + (size_t)p * bb.bounces * 4};
      const int4 misc = ps.misc[p];
      uint32_t seed = (uint32_t)misc.x;
      const int pix = misc.y;
      int phase = misc.z & 15;
      int flags = (misc.z >> 4) & 15;
      int lj = ((misc.z >> 8) & 31) - 1;
      int k = ((misc.z >> 13) & 31) - 1;
      BCount cnt = unpack_cnt(misc.w);
      // While the subpaths are built (B_LIGHT, B_EYE0, B_EYE) the connection stage's
      // fields (colour, sub-sum, NEE direction) are dead: Q_CONNECT initialises them.
      // They are loaded in the connection states only and stored once the stage has
      // started; the ray origin is read only where a hit point is built from it.
      const bool building = phase == B_LIGHT || phase == B_EYE0 || phase == B_EYE;
      bool conn_live = !building;
      f4 color = ym::splat(0.0f), sub = ym::splat(0.0f), w_i = ym::splat(0.0f);
      float light_pdf = 0.0f;
      if (!building) {
        color = f4of(ps.thr[p]);
        sub = f4of(ps.thr_next[p]);
        const float4 nee = ps.indirect[p];
        w_i = ym::mk(nee.x, nee.y, nee.z, 0.0f);
        light_pdf = nee.w;
      }
      float4 dv = ps.direct[p];
      float weight = dv.x, ks = dv.y, pend_pdf = dv.z, pend_prob = dv.w;
      f4 ro = ym::splat(0.0f), rd = ym::splat(0.0f);
      float tmax = 0.0f;
      if (building) {
        const float4 ro4 = ps.ro[p];
        ro = ym::mk(ro4.x, ro4.y, ro4.z, 1.0f);
        tmax = ro4.w;
      }
      if (building || phase == B_CONN) {
        const float4 rd4 = ps.rd[p];
        rd = ym::mk(rd4.x, rd4.y, rd4.z, rd4.w);
      }
      const float4 hit = ps.hit[p];
      bool done = false;

      for (int guard = 0; guard < 8192 && !done; ++guard) {
        switch (phase) {
          case B_LIGHT: {   // createLightPath, bdpt.cl:458-510
            const int tri = __float_as_int(hit.w);
            if (tri < 0 || pend_pdf <= 0.0f) { phase = Q_EYE_START; break; }
            const Vtx v = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            f4 contrib;
            if (cnt.i == 1) {
              const float c1 = ym::div(ym::max(0.0f, ym::dot(lv.vtx(0).n, rd)), pend_pdf);
              contrib = ym::splat(c1) * lv.contrib(0);
            } else {
              const Vtx pv = lv.vtx(cnt.i - 1);
              contrib = brdf_bk(-lv.dir(cnt.i - 1), rd, pv.n, sc.mats[pv.mat], (flags & BF_GLOSSY) != 0, pend_prob) *
                        ym::fmax(0.0f, ym::dot(rd, pv.n));
              contrib = contrib / pend_pdf;
              contrib = contrib * lv.contrib(cnt.i - 1);
            }
            cnt.lp = cnt.i + 1;
            bool stop = false;
            if (cnt.i >= 2 && cnt.i > RR) {
              const float r = draw(seed);
              const float pr = ym::min(luminance(contrib), 0.95f);
              if (r >= pr) stop = true;
              else contrib = contrib * ym::div(1.0f, pr);
            }
            lv.store(cnt.i, v, rd, contrib);
            if (stop || cnt.i + 1 >= BOUNCES) { phase = Q_EYE_START; break; }
            cnt.i += 1;
            phase = Q_LIGHT_SAMPLE;
            break;
          }
          case Q_LIGHT_SAMPLE: {   // sample from light vertex i - 1 (bdpt.cl:473-484)
            const Vtx pv = lv.vtx(cnt.i - 1);
            const yc_material& m = sc.mats[pv.mat];
            float prob = 0.0f;
            const bool g = sample_glossy_b(m, seed, prob);
            if (prob == 0.0f) { phase = Q_EYE_START; break; }
            float pdf = 1.0f;
            const f4 nd = g ? sample_phong_bk(pv, m, -lv.dir(cnt.i - 1), seed, pdf) : sample_cosine(pv, seed, pdf);
            flags = g ? (flags | BF_GLOSSY) : (flags & ~BF_GLOSSY);
            pend_pdf = pdf;
            pend_prob = prob;
            // the reference traces before it tests the pdf (bdpt.cl:486)
            ro = pv.hp + nd * EPS_F;
            rd = nd;
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            c[0]++; c[2]++; c[5]++;
            phase = B_LIGHT;
            emit = 1;
            done = true;
            break;
          }
          case Q_EYE_START: {   // createEyePath: the camera ray (bdpt.cl:517-519)
            ro = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
            const float4 d = ev.at(0, 2);
            rd = ym::mk(d.x, d.y, d.z, d.w);
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            cnt.i = 0;
            c[0]++; c[1]++; c[5]++;
            phase = B_EYE0;
            emit = 1;
            done = true;
            break;
          }
          case B_EYE0: {
            const int tri = __float_as_int(hit.w);
            if (tri < 0) {
              if (k >= 0) {
                color = (ym::dot(rd, ld4(sc.lights[k].normal)) < 0.0f) ? ym::mk(1.0f, 1.0f, 1.0f, 1.0f)
                                                                       : ym::mk(0.1f, 0.1f, 0.1f, 1.0f);
              } else {
                color = ym::mk(0.4f, 0.4f, 0.4f, 1.0f);
              }
              phase = Q_FINISH;
              break;
            }
            const Vtx v = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            ev.store(0, v, rd, ym::mk(1.0f, 1.0f, 1.0f, 1.0f));
            cnt.ep = 1;
            cnt.i = 1;
            phase = Q_EYE_SAMPLE;
            break;
          }
          case Q_EYE_SAMPLE: {   // bdpt.cl:527-535
            if (cnt.i >= BOUNCES) { phase = Q_CONNECT; cnt.i = 0; cnt.j = 0; flags = 0; break; }
            const Vtx pv = ev.vtx(cnt.i - 1);
            const yc_material& m = sc.mats[pv.mat];
            float prob = 0.0f;
            const bool g = sample_glossy_b(m, seed, prob);
            if (prob == 0.0f) { phase = Q_CONNECT; cnt.i = 0; cnt.j = 0; flags = 0; break; }
            float pdf = 1.0f;
            const f4 nd = g ? sample_phong_bk(pv, m, -ev.dir(cnt.i - 1), seed, pdf) : sample_cosine(pv, seed, pdf);
            if (pdf <= 0.0f) { phase = Q_CONNECT; cnt.i = 0; cnt.j = 0; flags = 0; break; }
            flags = g ? (flags | BF_GLOSSY) : (flags & ~BF_GLOSSY);
            pend_pdf = pdf;
            pend_prob = prob;
            ro = pv.hp + nd * EPS_F;
            rd = nd;
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            c[0]++; c[2]++; c[5]++;
            phase = B_EYE;
            emit = 1;
            done = true;
            break;
          }
          case B_EYE: {   // bdpt.cl:537-558
            const int tri = __float_as_int(hit.w);
            if (tri < 0) { phase = Q_CONNECT; cnt.i = 0; cnt.j = 0; flags = 0; break; }
            const Vtx v = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            const Vtx pv = ev.vtx(cnt.i - 1);
            f4 contrib = brdf_bk(rd, -ev.dir(cnt.i - 1), pv.n, sc.mats[pv.mat], (flags & BF_GLOSSY) != 0, pend_prob) *
                         ym::max(0.0f, ym::dot(rd, pv.n));
            contrib = contrib / pend_pdf;
            contrib = contrib * ev.contrib(cnt.i - 1);
            cnt.ep = cnt.i + 1;
            bool stop = false;
            if (cnt.i > RR) {
              const float r = draw(seed);
              const float pr = ym::min(luminance(contrib), 0.95f);
              if (r >= pr) stop = true;
              else contrib = contrib * ym::div(1.0f, pr);
            }
            ev.store(cnt.i, v, rd, contrib);
            if (stop) { phase = Q_CONNECT; cnt.i = 0; cnt.j = 0; flags = 0; break; }
            cnt.i += 1;
            phase = Q_EYE_SAMPLE;
            break;
          }
          case Q_CONNECT: {   // shading, bdpt.cl:578-595: start eye vertex i
            if (cnt.i == 0 && cnt.j == 0 && !(flags & 8)) {
              color = ym::mk(0.0f, 0.0f, 0.0f, 1.0f);
              weight = 1.0f;
              ks = 0.0f;
              conn_live = true;
              flags = 8;   // connection stage started
            }
            if (cnt.i >= cnt.ep || weight == 0.0f) { phase = Q_FINISH; break; }
            phase = Q_VERTEX;
            break;
          }
          case Q_VERTEX: {   // emission + next-event estimate at eye vertex i (bdpt.cl:591-597, 642-660)
            const Vtx v = ev.vtx(cnt.i);
            const yc_material& m = sc.mats[v.mat];
            sub = ym::mk(0.0f, 0.0f, 0.0f, 1.0f);
            ks = ym::max(ym::max(m.ks.x, ym::max(m.ks.y, m.ks.z)), 0.1f);
            f4 wi_raw;
            lj = sample_lights(sc, v, seed, light_pdf, wi_raw);
            if (lj == -1 || light_pdf <= 0.0f) {
              // DL = emission
              color = color + (ev.contrib(cnt.i) * (ld4(m.ke) + ld4(m.ke))) * weight;
              cnt.j = cnt.lp - 1;
              phase = Q_CONNECT + 16;   // connections
              break;
            }
            float len = ym::length(wi_raw);
            len = ym::sub(len, ym::mul(EPS_F, 1.5f));
            w_i = ym::normalize(wi_raw);
            ro = v.hp + w_i * EPS_F;
            rd = w_i;
            tmax = len;
            c[0]++; c[3]++;
            int lk = -1;
            float tl = len;
            light_test(sc, ro, rd, tl, lk);
            if (lk >= 0) { flags |= BF_OCCLUDED; phase = B_NEE; break; }
            flags &= ~BF_OCCLUDED;
            c[5]++;
            phase = B_NEE;
            emit = 2;
            done = true;
            break;
          }
          case B_NEE: {   // bdpt.cl:662-671 (MIS off, as shipped)
            if (hit.x != 0.0f) flags |= BF_OCCLUDED;
            const Vtx v = ev.vtx(cnt.i);
            const yc_material& m = sc.mats[v.mat];
            const f4 em = ld4(m.ke);
            f4 dl = ym::splat(0.0f) + em;   // light_sample (0) + emission
            if (!(flags & BF_OCCLUDED)) {
              float prob = 0.0f;
              const bool g = sample_glossy_b(m, seed, prob);
              if (prob == 0.0f) {
                dl = em;
              } else {
                f4 ls = (brdf_bk(w_i, -ev.dir(cnt.i), v.n, m, g, prob) * ld4(sc.lights[lj].ke)) *
                        ym::fmax(ym::dot(w_i, v.n), 0.0f);
                ls = ls * ym::div(1.0f, light_pdf);
                dl = ls + em;
              }
            }
            flags &= ~BF_OCCLUDED;
            color = color + (ev.contrib(cnt.i) * (em + dl)) * weight;
            cnt.j = cnt.lp - 1;
            phase = Q_CONNECT + 16;
            break;
          }
          case Q_CONNECT + 16: {   // next connection j (bdpt.cl:598-615)
            if (cnt.j <= 0) {
              color = color + sub * ym::mul(weight, ym::sub(1.0f, ks));
              weight = ym::mul(weight, ks);
              cnt.i += 1;
              phase = Q_CONNECT;
              break;
            }
            const Vtx e_v = ev.vtx(cnt.i);
            const Vtx l_v = lv.vtx(cnt.j);
            const f4 dir = ym::normalize(l_v.hp - e_v.hp);
            const f4 org = e_v.hp + dir * EPS_F;
            if (ym::dot(dir, e_v.n) <= 0.0f || ym::dot(-dir, l_v.n) <= 0.0f) { cnt.j -= 1; break; }
            ro = org;
            rd = dir;
            tmax = ym::length(l_v.hp - org);
            c[0]++; c[4]++;
            int lk = -1;
            float tl = tmax;
            light_test(sc, ro, rd, tl, lk);
            if (lk >= 0) { cnt.j -= 1; break; }   // a light closes the segment: occluded
            c[5]++;
            phase = B_CONN;
            emit = 2;
            done = true;
            break;
          }
          case B_CONN: {   // bdpt.cl:616-634
            if (hit.x == 0.0f) {
              const Vtx e_v = ev.vtx(cnt.i);
              const Vtx l_v = lv.vtx(cnt.j);
              float dist = ym::length(l_v.hp - e_v.hp);
              dist = ym::mul(dist, dist);
              const f4 wi = rd;
              const f4 wo = -ev.dir(cnt.i);
              const float gf = ym::div(ym::mul(ym::max(ym::dot(wi, e_v.n), 0.0f), ym::max(ym::dot(-wi, l_v.n), 0.0f)), dist);
              float prob = 0.0f;
              bool g = sample_glossy_b(sc.mats[e_v.mat], seed, prob);
              const f4 e2l = brdf_bk(wi, wo, e_v.n, sc.mats[e_v.mat], g, prob);
              g = sample_glossy_b(sc.mats[l_v.mat], seed, prob);
              const f4 l2e = brdf_bk(-lv.dir(cnt.j), -wi, l_v.n, sc.mats[l_v.mat], g, prob);
              f4 tlp = lv.contrib(cnt.j);
              tlp = tlp * ((gf * e2l) * l2e);
              tlp = tlp * ev.contrib(cnt.i);
              sub = sub + tlp;
            }
            cnt.j -= 1;
            phase = Q_CONNECT + 16;
            break;
          }
          case Q_FINISH:
          default: {
            if (ym::any_nan(color)) color = ym::mk(0.988f, 0.0588f, 0.7529f, 1.0f);
            const float4 prev = pp.accum[pix];
            f4 cc = color;
            if (pp.reset == 1) {
              cc.w = 1.0f;
            } else {
              const int np = (int)prev.w;
              cc = cc + f4of(prev) * (float)np;
              cc = cc / (float)(np + 1);
              cc.w = (float)(np + 1);
            }
            pp.accum[pix] = make_float4(cc.x, cc.y, cc.z, cc.w);
            c[6]++;
            done = true;
            break;
          }
        }
      }
      if (emit) {
        ps.misc[p] = make_int4((int)seed, pix, pack_st(phase, flags & 15, lj, k), pack_cnt(cnt));
        if (conn_live) {
          ps.thr[p] = make_float4(color.x, color.y, color.z, color.w);
          ps.thr_next[p] = make_float4(sub.x, sub.y, sub.z, sub.w);
          ps.indirect[p] = make_float4(w_i.x, w_i.y, w_i.z, light_pdf);
        }
        ps.direct[p] = make_float4(weight, ks, pend_pdf, pend_prob);
        ps.ro[p] = make_float4(ro.x, ro.y, ro.z, tmax);
        ps.rd[p] = make_float4(rd.x, rd.y, rd.z, rd.w);
      }
    }
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
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      unsigned x = c[q];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
      if (lane == 0 && x) atomicAdd(&s_cnt[q], (unsigned long long)x);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (s_cnt[0]) atomicAdd(&st->rays, s_cnt[0]);
    if (s_cnt[1]) atomicAdd(&st->primary, s_cnt[1]);
    if (s_cnt[2]) atomicAdd(&st->extension, s_cnt[2]);
    if (s_cnt[3]) atomicAdd(&st->shadow, s_cnt[3]);
    if (s_cnt[4]) atomicAdd(&st->connection, s_cnt[4]);
    if (s_cnt[5]) atomicAdd(&st->traversed, s_cnt[5]);
    if (s_cnt[6]) atomicAdd(&st->samples, s_cnt[6]);
  }
}

void launch_logic_bdpt(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, const int* in_closest,
                       const int* in_any, const RoundCounters* rc_in, int* out_closest, int* out_any,
                       RoundCounters* rc_out, DevStats* st, int grid, cudaStream_t s, const int* sorted,
                       const SortCtl* sctl) {
  k_logic_bdpt<<<grid, 256, 0, s>>>(pp, ps, bb, in_closest, in_any, rc_in, out_closest, out_any, rc_out, st, sorted,
                                    sctl);
}

}  // namespace yc
