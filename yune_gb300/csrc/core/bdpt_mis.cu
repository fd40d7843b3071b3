// bdpt_mis.cu -- wavefront bidirectional path tracer with multiple importance sampling
// (integrator YC_BDPT_MIS).
//
// bdpt.cl stores forward and reverse densities on its vertices but never uses them; its
// connections are summed with the heuristic weight `weight * (1 - ks)` (bdpt.cl:38-39, 453,
// 465, 598-636), so it converges to another image than the unidirectional tracer. This
// integrator weights every strategy (s light vertices, t >= 2 eye vertices; no light
// tracing to the camera) with the power heuristic over the strategies that can make the
// same path. The denominators come from two partial sums per subpath vertex (the
// recursive form of Georgiev, "Implementing Vertex Connection and Merging", 2012):
// arriving at vertex v from u with solid-angle density w_f, squared distance d2 and
// cosine c_v at v,
//   r_v = (d2 / (w_f c_v))^2,   s_v = r_v (c_u / d2)^2 acc_u,
// and once v's next direction fixes its reverse density w_r, acc_v = r_v + s_v w_r^2.
// A connection of eye vertex Y to light vertex L then has the weight
//   1 / (1 + (w_{Y->L} c_L / d2)^2 (r_L + s_L w_{L,rev}^2) + (w_{L->Y} c_Y / d2)^2 (r_Y + s_Y w_{Y,rev}^2)).
// The random-number order, the material and light models and the operation order are
// those of the CPU statement the parity tests compare against; each sample is one state
// machine as in bdpt.cu (one ray in flight), with the light subpath in 64-byte vertex
// records, vertex k of path p at [(p * bounces + k) * 4 + field]:
//   field 0: hit point xyz, material index (int bits; -1 for the point on the light)
//   field 1: shading normal xyz, r
//   field 2: direction of the ray that reached the vertex xyz, s
//   field 3: subpath throughput xyz
// The eye subpath is walked vertex by vertex: next-event estimate, then the connections
// to every stored light vertex, then the next eye ray. Path slot fields:
//   thr      pixel colour              thr_next  eye throughput xyz, r of the eye vertex
//   direct   pending shadow-ray contribution xyz, s of the eye vertex
//   indirect throughput after the pending bounce xyz, its solid-angle density
//   ls       cosine toward the pending ray at its origin, acc of the origin vertex,
//            area density of the light subpath's start point
//   hp, nrm, wo   the current eye vertex: point + material, normal, arriving direction
//   wi       the camera ray, kept while the light subpath is traced
#include <cuda_runtime.h>

#include "yc_bdpt.h"
#include "yc_shade.cuh"

namespace yc {

namespace {

enum : int { M_EYE_START = 8, M_VERTEX = 9, M_CONN = 10, M_CONT = 11, M_FINISH = 12 };

struct MCount {
  int j, m, nl;   // light vertex index, eye vertex index, stored light vertices
};
__device__ __forceinline__ int pack_mc(const MCount& c) { return c.j | (c.m << 6) | (c.nl << 12); }
__device__ __forceinline__ MCount unpack_mc(int v) { return MCount{v & 63, (v >> 6) & 63, (v >> 12) & 63}; }
__device__ __forceinline__ int pack_ms(int state, int lk, int k) { return state | ((lk + 1) << 8) | ((k + 1) << 13); }

__device__ __forceinline__ float mis(float x) { return ym::mul(x, x); }
// a * b with 0 * inf = 0 (a vanishing density removes the strategy)
__device__ __forceinline__ float mul0(float a, float b) { return (a == 0.0f || b == 0.0f) ? 0.0f : ym::mul(a, b); }
__device__ __forceinline__ f4 rgb(const yc_float4& c) { return ym::mk(c.x, c.y, c.z, 0.0f); }

__device__ __forceinline__ float diffuse_prob(const yc_material& m) {
  const float sd = ym::add(ym::add(m.kd.x, m.kd.y), m.kd.z);
  const float ss = ym::add(ym::add(m.ks.x, m.ks.y), m.ks.z);
  if (ss == 0.0f) return 1.0f;
  if (sd == 0.0f) return 0.0f;
  return ym::div(sd, ym::add(sd, ss));
}

__device__ __forceinline__ f4 mirror(f4 w, f4 n) { return ym::normalize(ym::mul(2.0f, ym::dot(w, n)) * n - w); }

// BRDF at v between the direction toward the previous subpath vertex and the next one.
// f_eval and pdf_dir are called, not inlined: the logic kernel's lanes run different
// states, and one copy of each keeps the code within the instruction cache (measured
// 1024x1024: 797 against 651 Mrays/s inlined, despite the call's register spills).
__device__ __noinline__ f4 f_eval(const Vtx& v, const yc_material& m, f4 w_prev, f4 w_next, int brdf_model,
                                  const float2* on_ab) {
  const bool glossy = ym::length3(ld4(m.ks)) != 0.0f;
  f4 f;
  if (brdf_model == 1 && !glossy) f = oren_nayar(w_next, w_prev, v, m, on_ab[v.mat]);
  else f = ld4(m.kd) * INV_PI_F;
  if (glossy) {
    const float ca = ym::pow(ym::fmax(ym::dot(w_next, mirror(w_prev, v.n)), 0.0f), ym::add(m.px, m.py));
    const int pe = (int)ym::add(m.px, m.py);
    f = f + (((ld4(m.ks) * ca) * (float)(pe + 2)) * INV_PI_F) * 0.5f;
  }
  f.w = 0.0f;
  return f;
}

// solid-angle density with which sample_dir picks w_next at v after arriving from w_prev
__device__ __noinline__ float pdf_dir(const Vtx& v, const yc_material& m, f4 w_prev, f4 w_next) {
  const float cn = ym::dot(w_next, v.n);
  if (!(cn > 0.0f)) return 0.0f;
  const float pd = diffuse_prob(m);
  float p = ym::mul(pd, ym::mul(cn, INV_PI_F));
  if (pd < 1.0f) {
    const int pe = (int)ym::add(m.px, m.py);
    const float ca = ym::fmax(ym::dot(w_next, mirror(w_prev, v.n)), 0.0f);
    const float lobe = ym::mul(ym::mul(ym::mul((float)(pe + 1), 0.5f), INV_PI_F), ym::pow(ca, (float)pe));
    p = ym::add(p, ym::mul(ym::sub(1.0f, pd), lobe));
  }
  return p;
}

// lobe (1 number), then a cosine or Phong-lobe direction (2 numbers); false when the
// direction does not leave the surface
__device__ __forceinline__ bool sample_dir(const Vtx& v, const yc_material& m, f4 w_prev, uint32_t& seed,
                                           f4& w_next) {
  const float u = draw(seed);
  const float pd = diffuse_prob(m);
  float pdf = 0.0f;
  if (pd >= 1.0f || u < pd) w_next = sample_cosine(v, seed, pdf);
  else w_next = sample_phong_b(v, m, w_prev, seed, pdf);
  return ym::dot(w_next, v.n) > 0.0f;
}

__device__ __forceinline__ float light_area(const yc_quad_light& L) {
  return ym::mul(ym::length(ld4(L.edge_l)), ym::length(ld4(L.edge_w)));
}
__device__ __forceinline__ float light_weight(const yc_quad_light& L) {
  return ym::mul(ym::add(ym::add(L.ke.x, L.ke.y), L.ke.z), light_area(L));
}
__device__ __forceinline__ float light_total(const DevScene& sc) {
  float t = 0.0f;
  for (int i = 0; i < sc.n_lights; ++i) t = ym::add(t, light_weight(sc.lights[i]));
  return t;
}
// area density of the point a light sample lands on, on light i
__device__ __forceinline__ float light_point_pdf(const DevScene& sc, int i) {
  const yc_quad_light& L = sc.lights[i];
  return ym::div(ym::div(light_weight(L), light_total(sc)), light_area(L));
}
// picks a light (1 number) with probability proportional to (ke.r + ke.g + ke.b) * area
__device__ __forceinline__ int pick_light(const DevScene& sc, uint32_t& seed) {
  const float u = draw(seed);
  const float total = light_total(sc);
  if (!(total > 0.0f)) return -1;
  float cum = 0.0f;
  int last = -1;
  for (int i = 0; i < sc.n_lights; ++i) {
    const float w = light_weight(sc.lights[i]);
    if (!(w > 0.0f)) continue;
    last = i;
    const float p = ym::div(w, total);
    if (u < ym::add(cum, p)) return i;
    cum = ym::add(cum, p);
  }
  return last;
}
__device__ __forceinline__ f4 light_point(const yc_quad_light& L, uint32_t& seed) {
  const float a = draw(seed);
  const float b = draw(seed);
  return (ld4(L.pos) + ld4(L.edge_l) * a) + ld4(L.edge_w) * b;
}

struct MisRec {
  float4* base;   // the path's first light vertex
  __device__ __forceinline__ float4& at(int k, int f) const { return base[(size_t)k * 4 + f]; }
  __device__ __forceinline__ Vtx vtx(int k) const {
    const float4 a = at(k, 0), b = at(k, 1);
    Vtx v;
    v.hp = ym::mk(a.x, a.y, a.z, 1.0f);
    v.n = ym::mk(b.x, b.y, b.z, 0.0f);
    v.mat = __float_as_int(a.w);
    return v;
  }
};

__device__ __forceinline__ void count_ray(unsigned* c, int kind) {
  c[0]++;
  c[kind]++;
}

}  // namespace

// ---- raygen: pixel prologue, camera ray kept, light point and the first light ray ----
__global__ void __launch_bounds__(256) k_raygen_bdpt_mis(PassParams pp, PathState ps, BdptBuffers bb, int* q_closest,
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
    ps.wi[slot] = make_float4(d.x, d.y, d.z, d.w);
    const MisRec lv{bb.lv + (size_t)slot * bb.bounces * 4};
    const int lk = pick_light(sc, seed);
    f4 o = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w), rdir = d;
    int state = B_EYE0;
    MCount cnt{0, 0, 0};
    float p0 = 0.0f, c0 = 0.0f;
    if (lk >= 0) {
      const yc_quad_light& L = sc.lights[lk];
      p0 = light_point_pdf(sc, lk);
      Vtx v0;
      v0.hp = light_point(L, seed);
      v0.n = ld4(L.normal);
      v0.mat = -1;
      lv.at(0, 0) = make_float4(v0.hp.x, v0.hp.y, v0.hp.z, __int_as_float(-1));
      lv.at(0, 1) = make_float4(v0.n.x, v0.n.y, v0.n.z, 0.0f);
      float pdf = 0.0f;
      const f4 ldir = sample_cosine(v0, seed, pdf);
      c0 = ym::dot(ldir, v0.n);
      if (c0 > 0.0f) {
        o = v0.hp + ldir * EPS_F;
        rdir = ldir;
        state = B_LIGHT;
        cnt.j = 1;
      }
    }
    eye_first = state == B_EYE0;
    float len = __int_as_float(0x7f800000);
    int k = -1;
    light_test(sc, o, rdir, len, k);
    ps.misc[slot] = make_int4((int)seed, pix, pack_ms(state, lk, k), pack_mc(cnt));
    ps.ro[slot] = make_float4(o.x, o.y, o.z, len);
    ps.rd[slot] = make_float4(rdir.x, rdir.y, rdir.z, rdir.w);
    ps.indirect[slot] = make_float4(1.0f, 1.0f, 1.0f, ym::mul(c0, INV_PI_F));
    ps.ls[slot] = make_float4(c0, lk >= 0 ? ym::div(1.0f, mis(p0)) : 0.0f, p0, 0.0f);
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

void launch_raygen_bdpt_mis(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, int* q_closest,
                            RoundCounters* rc, DevStats* st, cudaStream_t s) {
  const int n = pp.tile_w * pp.tile_h;
  k_raygen_bdpt_mis<<<(n + 255) / 256, 256, 0, s>>>(pp, ps, bb, q_closest, rc, st);
}

// ---- logic: advance each path to its next ray ----
__global__ void __launch_bounds__(256) k_logic_bdpt_mis(PassParams pp, PathState ps, BdptBuffers bb,
                                                        const int* __restrict__ in_closest,
                                                        const int* __restrict__ in_any, const RoundCounters* rc_in,
                                                        int* out_closest, int* out_any, RoundCounters* rc_out,
                                                        DevStats* st, const int* __restrict__ sorted,
                                                        const SortCtl* sctl) {
  // per-warp counts of rays, primary, extension, shadow, connection, traversed, samples,
  // added to the device counters when the warp leaves (no block barrier: warps finish at
  // different times)
  unsigned w_cnt[7] = {0, 0, 0, 0, 0, 0, 0};
  const int nc = rc_in->n_closest, na = rc_in->n_any;
  const int n = nc + na;
  const int lane = threadIdx.x & 31;
  const int warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int warps_total = (gridDim.x * blockDim.x) >> 5;
  const DevScene& sc = pp.sc;
  const float INF = __int_as_float(0x7f800000);
  const int KMAX = bb.bounces;
  const int RR = pp.rr_threshold;
  const bool use_sorted = sctl && sctl->use;

  for (int wbase = warp_global * 32; wbase < n; wbase += warps_total * 32) {
    const int e = wbase + lane;
    int emit = 0;
    int p = -1;
    unsigned c[7] = {0, 0, 0, 0, 0, 0, 0};
    if (e < n) {
      p = use_sorted ? sorted[e] : (e < nc ? in_closest[e] : in_any[e - nc]);
      const MisRec lv{bb.lv + (size_t)p * bb.bounces * 4};
      const int4 misc = ps.misc[p];
      uint32_t seed = (uint32_t)misc.x;
      const int pix = misc.y;
      int phase = misc.z & 15;
      const int lk = ((misc.z >> 8) & 31) - 1;
      int k = ((misc.z >> 13) & 31) - 1;
      MCount cnt = unpack_mc(misc.w);
      // only the fields the state reads are loaded, and only the changed ones are
      // written back: the eye vertex and colour exist from B_EYE on, the pending
      // bounce (throughput, density, cosine, acc) is read when its ray returns, and a
      // shadow ray's own origin and direction are not needed after it is traced
      const bool eye_state = phase >= B_EYE;
      const bool pending = phase == B_LIGHT || phase == B_EYE;
      const bool shadow = phase == B_NEE || phase == B_CONN;
      const float4 l4 = ps.ls[p];
      float c_out = l4.x, acc = l4.y;
      const float p0 = l4.z;
      f4 color = ym::splat(0.0f), beta = ym::splat(0.0f), pend = ym::splat(0.0f), bnext = ym::splat(0.0f);
      float r_y = 0.0f, s_y = 0.0f, w_f = 0.0f;
      Vtx y;
      y.hp = ym::splat(0.0f);
      y.n = ym::splat(0.0f);
      y.mat = 0;
      f4 wp = ym::splat(0.0f);
      if (eye_state) {
        color = f4of(ps.thr[p]);
        const float4 tn = ps.thr_next[p], dc = ps.direct[p];
        beta = ym::mk(tn.x, tn.y, tn.z, 0.0f);
        r_y = tn.w;
        s_y = dc.w;
        pend = ym::mk(dc.x, dc.y, dc.z, 0.0f);
        const float4 a = ps.hp[p], b = ps.nrm[p], w = ps.wo[p];
        y.hp = ym::mk(a.x, a.y, a.z, 1.0f);
        y.n = ym::mk(b.x, b.y, b.z, 0.0f);
        y.mat = __float_as_int(a.w);
        wp = ym::mk(-w.x, -w.y, -w.z, -0.0f);
      }
      if (pending) {
        const float4 ind = ps.indirect[p];
        bnext = ym::mk(ind.x, ind.y, ind.z, 0.0f);
        w_f = ind.w;
      }
      f4 ro = ym::splat(0.0f), rd = ym::splat(0.0f);
      float tmax = 0.0f;
      if (!shadow) {
        const float4 ro4 = ps.ro[p], rd4 = ps.rd[p];
        ro = ym::mk(ro4.x, ro4.y, ro4.z, 1.0f);
        rd = ym::mk(rd4.x, rd4.y, rd4.z, rd4.w);
        tmax = ro4.w;
      }
      const float4 hit = ps.hit[p];
      bool moved = false;    // the eye vertex changed
      bool w_color = false, w_eye = false, w_pend = false, w_bounce = false;   // fields to write back
      bool done = false;

      for (int guard = 0; guard < 8192 && !done; ++guard) {
        switch (phase) {
          case B_LIGHT: {   // light vertex j reached (or the light subpath ends)
            const int tri = __float_as_int(hit.w);
            if (tri < 0) { phase = M_EYE_START; break; }
            const Vtx v = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            const float cv = -ym::dot(rd, v.n);
            if (!(cv > 0.0f)) { phase = M_EYE_START; break; }
            const int j = cnt.j;
            const Vtx pv = lv.vtx(j - 1);
            const f4 dv = v.hp - pv.hp;
            const float d2 = ym::dot(dv, dv);
            const float r = mis(ym::div(d2, ym::mul(w_f, cv)));
            const float s = mul0(ym::mul(r, mis(ym::div(c_out, d2))), acc);
            lv.at(j, 0) = make_float4(v.hp.x, v.hp.y, v.hp.z, __int_as_float(v.mat));
            lv.at(j, 1) = make_float4(v.n.x, v.n.y, v.n.z, r);
            lv.at(j, 2) = make_float4(rd.x, rd.y, rd.z, s);
            lv.at(j, 3) = make_float4(bnext.x, bnext.y, bnext.z, 0.0f);
            cnt.nl = j;
            if (j + 1 > KMAX - 2) { phase = M_EYE_START; break; }
            const yc_material& m = sc.mats[v.mat];
            f4 cont = bnext;
            if (j > RR) {
              const float q = ym::min(luminance(bnext), 0.95f);
              if (!(draw(seed) < q)) { phase = M_EYE_START; break; }
              cont = bnext / q;
            }
            const f4 lp = -rd;
            f4 wn;
            if (!sample_dir(v, m, lp, seed, wn)) { phase = M_EYE_START; break; }
            w_f = pdf_dir(v, m, lp, wn);
            if (!(w_f > 0.0f)) { phase = M_EYE_START; break; }
            const float w_r = pdf_dir(v, m, wn, lp);
            c_out = ym::dot(wn, v.n);
            acc = ym::add(r, mul0(s, mis(w_r)));
            bnext = ((cont * f_eval(v, m, lp, wn, pp.brdf_model, sc.on_ab)) * c_out) / w_f;
            w_bounce = true;
            ro = v.hp + wn * EPS_F;
            rd = wn;
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            cnt.j = j + 1;
            count_ray(c, 2);
            c[5]++;
            emit = 1;
            done = true;
            break;
          }
          case M_EYE_START: {   // the camera ray
            ro = ym::mk(pp.cam.r1.w, pp.cam.r2.w, pp.cam.r3.w, pp.cam.r4.w);
            const float4 d = ps.wi[p];
            rd = ym::mk(d.x, d.y, d.z, d.w);
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            cnt.m = 0;
            count_ray(c, 1);
            c[5]++;
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
              phase = M_FINISH;
              break;
            }
            color = ym::mk(0.0f, 0.0f, 0.0f, 1.0f);
            w_color = true;
            y = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            wp = -rd;
            if (!(ym::dot(wp, y.n) > 0.0f)) { phase = M_FINISH; break; }
            beta = ym::mk(1.0f, 1.0f, 1.0f, 0.0f);
            r_y = 0.0f;
            s_y = 0.0f;
            cnt.m = 1;
            moved = w_eye = w_pend = true;
            phase = M_VERTEX;
            break;
          }
          case M_VERTEX: {   // emission, then the next-event estimate at eye vertex m
            const yc_material& m = sc.mats[y.mat];
            color = color + beta * rgb(m.ke);
            w_color = true;
            if (cnt.m + 1 > KMAX) { phase = M_FINISH; break; }
            if (lk < 0) { phase = M_CONT; break; }
            cnt.j = 1;
            phase = M_CONN;
            const int kl = pick_light(sc, seed);
            if (kl < 0) break;
            const yc_quad_light& L = sc.lights[kl];
            const float pk = light_point_pdf(sc, kl);
            const f4 x = light_point(L, seed);
            const f4 v = x - y.hp;
            const float d2 = ym::dot(v, v);
            const float dist = ym::sqrt(d2);
            const f4 dir = v * ym::div(1.0f, dist);
            const float cy = ym::dot(dir, y.n);
            const float cl = -ym::dot(dir, ld4(L.normal));
            if (!(cy > 0.0f) || !(cl > 0.0f)) break;
            const float wf = pdf_dir(y, m, wp, dir);
            const float wr = pdf_dir(y, m, dir, wp);
            const float ls = mis(ym::div(ym::mul(wf, cl), ym::mul(d2, pk)));
            const float es = mul0(mis(ym::div(ym::mul(ym::mul(cl, INV_PI_F), cy), d2)), ym::add(r_y, mul0(s_y, mis(wr))));
            const float w = ym::div(1.0f, ym::add(ym::add(1.0f, ls), es));
            const float g = ym::div(ym::mul(cy, cl), ym::mul(d2, pk));
            pend = ((beta * f_eval(y, m, wp, dir, pp.brdf_model, sc.on_ab)) * rgb(L.ke)) * ym::mul(g, w);
            w_pend = true;
            ro = y.hp + dir * EPS_F;
            rd = dir;
            tmax = ym::sub(dist, ym::mul(EPS_F, 1.5f));
            count_ray(c, 3);
            int lh = -1;
            float tl = tmax;
            light_test(sc, ro, rd, tl, lh);
            if (lh >= 0) break;   // a light closes the segment: occluded
            c[5]++;
            phase = B_NEE;
            emit = 2;
            done = true;
            break;
          }
          case B_NEE: {
            if (hit.x == 0.0f) {
              color = color + pend;
              w_color = true;
            }
            phase = M_CONN;
            break;
          }
          case M_CONN: {   // connection of eye vertex m to light vertex j
            const int j = cnt.j;
            if (j > cnt.nl || cnt.m + j + 1 > KMAX) { phase = M_CONT; break; }
            cnt.j = j + 1;
            const Vtx lvx = lv.vtx(j);
            const f4 v = lvx.hp - y.hp;
            const float d2 = ym::dot(v, v);
            const float dist = ym::sqrt(d2);
            const f4 dir = v * ym::div(1.0f, dist);
            const float cy = ym::dot(dir, y.n);
            const float cl = -ym::dot(dir, lvx.n);
            if (!(cy > 0.0f) || !(cl > 0.0f)) break;
            const float4 f2 = lv.at(j, 2), f3 = lv.at(j, 3);
            const float lr = lv.at(j, 1).w, lsv = f2.w;
            const f4 lp = ym::mk(-f2.x, -f2.y, -f2.z, -0.0f);
            const f4 wl = -dir;
            const yc_material& my = sc.mats[y.mat];
            const yc_material& ml = sc.mats[lvx.mat];
            const float wy_f = pdf_dir(y, my, wp, dir);
            const float wy_r = pdf_dir(y, my, dir, wp);
            const float wl_f = pdf_dir(lvx, ml, lp, wl);
            const float wl_r = pdf_dir(lvx, ml, wl, lp);
            const float ls = mul0(mis(ym::div(ym::mul(wy_f, cl), d2)), ym::add(lr, mul0(lsv, mis(wl_r))));
            const float es = mul0(mis(ym::div(ym::mul(wl_f, cy), d2)), ym::add(r_y, mul0(s_y, mis(wy_r))));
            const float w = ym::div(1.0f, ym::add(ym::add(1.0f, ls), es));
            const float g = ym::div(ym::mul(cy, cl), d2);
            const f4 le = rgb(sc.lights[lk].ke) * ym::div(PI_F, p0);
            pend = ((((beta * f_eval(y, my, wp, dir, pp.brdf_model, sc.on_ab)) * f_eval(lvx, ml, lp, wl, pp.brdf_model, sc.on_ab)) *
                     ym::mk(f3.x, f3.y, f3.z, 0.0f)) * le) * ym::mul(g, w);
            w_pend = true;
            ro = y.hp + dir * EPS_F;
            rd = dir;
            tmax = ym::sub(dist, ym::mul(EPS_F, 2.0f));
            count_ray(c, 4);
            int lh = -1;
            float tl = tmax;
            light_test(sc, ro, rd, tl, lh);
            if (lh >= 0) break;
            c[5]++;
            phase = B_CONN;
            emit = 2;
            done = true;
            break;
          }
          case B_CONN: {
            if (hit.x == 0.0f) {
              color = color + pend;
              w_color = true;
            }
            phase = M_CONN;
            break;
          }
          case M_CONT: {   // the next eye ray from vertex m
            const yc_material& m = sc.mats[y.mat];
            f4 cont = beta;
            if (cnt.m > RR) {
              const float q = ym::min(luminance(beta), 0.95f);
              if (!(draw(seed) < q)) { phase = M_FINISH; break; }
              cont = beta / q;
            }
            f4 wn;
            if (!sample_dir(y, m, wp, seed, wn)) { phase = M_FINISH; break; }
            w_f = pdf_dir(y, m, wp, wn);
            if (!(w_f > 0.0f)) { phase = M_FINISH; break; }
            const float w_r = pdf_dir(y, m, wn, wp);
            c_out = ym::dot(wn, y.n);
            acc = ym::add(r_y, mul0(s_y, mis(w_r)));
            bnext = ((cont * f_eval(y, m, wp, wn, pp.brdf_model, sc.on_ab)) * c_out) / w_f;
            w_bounce = true;
            ro = y.hp + wn * EPS_F;
            rd = wn;
            tmax = INF;
            k = -1;
            light_test(sc, ro, rd, tmax, k);
            count_ray(c, 2);
            c[5]++;
            phase = B_EYE;
            emit = 1;
            done = true;
            break;
          }
          case B_EYE: {   // eye vertex m + 1 reached, or a light (strategy s = 0)
            const int tri = __float_as_int(hit.w);
            if (tri < 0) {
              if (k >= 0) {
                const yc_quad_light& L = sc.lights[k];
                const float cl = -ym::dot(rd, ld4(L.normal));
                if (cl > 0.0f) {
                  const f4 z = ro + rd * tmax;
                  const f4 dv = z - y.hp;
                  const float d2 = ym::dot(dv, dv);
                  const float r2 = mis(ym::div(d2, ym::mul(w_f, cl)));
                  const float s2 = mul0(ym::mul(r2, mis(ym::div(c_out, d2))), acc);
                  const float es = ym::mul(mis(light_point_pdf(sc, k)), ym::add(r2, mul0(s2, mis(ym::mul(cl, INV_PI_F)))));
                  const float w = ym::div(1.0f, ym::add(1.0f, es));
                  color = color + (bnext * rgb(L.ke)) * w;
                }
              }
              phase = M_FINISH;
              break;
            }
            const Vtx v = tri_vertex(sc, ro, rd, hit.x, hit.y, hit.z, tri);
            const float cv = -ym::dot(rd, v.n);
            if (!(cv > 0.0f)) { phase = M_FINISH; break; }
            const f4 dv = v.hp - y.hp;
            const float d2 = ym::dot(dv, dv);
            r_y = mis(ym::div(d2, ym::mul(w_f, cv)));
            s_y = mul0(ym::mul(r_y, mis(ym::div(c_out, d2))), acc);
            beta = bnext;
            y = v;
            wp = -rd;
            cnt.m += 1;
            moved = w_eye = w_pend = true;
            phase = M_VERTEX;
            break;
          }
          case M_FINISH:
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
        ps.misc[p] = make_int4((int)seed, pix, pack_ms(phase, lk, k), pack_mc(cnt));
        if (w_color) ps.thr[p] = make_float4(color.x, color.y, color.z, color.w);
        if (w_eye) ps.thr_next[p] = make_float4(beta.x, beta.y, beta.z, r_y);
        if (w_pend) ps.direct[p] = make_float4(pend.x, pend.y, pend.z, s_y);
        if (w_bounce) {
          ps.indirect[p] = make_float4(bnext.x, bnext.y, bnext.z, w_f);
          ps.ls[p] = make_float4(c_out, acc, p0, 0.0f);
        }
        if (moved) {
          ps.hp[p] = make_float4(y.hp.x, y.hp.y, y.hp.z, __int_as_float(y.mat));
          ps.nrm[p] = make_float4(y.n.x, y.n.y, y.n.z, 0.0f);
          ps.wo[p] = make_float4(-wp.x, -wp.y, -wp.z, 0.0f);
        }
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
    for (int q = 0; q < 7; ++q) w_cnt[q] += c[q];
  }
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    unsigned x = w_cnt[q];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    w_cnt[q] = x;
  }
  if (lane == 0) {
    if (w_cnt[0]) atomicAdd(&st->rays, (unsigned long long)w_cnt[0]);
    if (w_cnt[1]) atomicAdd(&st->primary, (unsigned long long)w_cnt[1]);
    if (w_cnt[2]) atomicAdd(&st->extension, (unsigned long long)w_cnt[2]);
    if (w_cnt[3]) atomicAdd(&st->shadow, (unsigned long long)w_cnt[3]);
    if (w_cnt[4]) atomicAdd(&st->connection, (unsigned long long)w_cnt[4]);
    if (w_cnt[5]) atomicAdd(&st->traversed, (unsigned long long)w_cnt[5]);
    if (w_cnt[6]) atomicAdd(&st->samples, (unsigned long long)w_cnt[6]);
  }
}

void launch_logic_bdpt_mis(const PassParams& pp, const PathState& ps, const BdptBuffers& bb, const int* in_closest,
                           const int* in_any, const RoundCounters* rc_in, int* out_closest, int* out_any,
                           RoundCounters* rc_out, DevStats* st, int grid, cudaStream_t s, const int* sorted,
                           const SortCtl* sctl) {
  k_logic_bdpt_mis<<<grid, 256, 0, s>>>(pp, ps, bb, in_closest, in_any, rc_in, out_closest, out_any, rc_out, st,
                                        sorted, sctl);
}

}  // namespace yc
