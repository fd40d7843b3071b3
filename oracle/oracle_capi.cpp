// oracle_capi.cpp -- C entry points of the CPU oracle (liboracle.so).
//
// TEST INFRASTRUCTURE: called by tests, the smoke check and the benchmark's
// CPU-baseline leg only. The float entry points reproduce kernels/legacy/udpt.cl and
// kernels/post-proc/tonemap.cl bit for bit; or_render_f64 is the FP64 accuracy oracle.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "bdpt_mis_oracle.hpp"
#include "bdpt_oracle.hpp"
#include "udpt_oracle.hpp"

extern "C" {

typedef struct or_cfg {
  int mis, rr_threshold, max_depth, brdf_model, mis_lobe_fix, heap_size, gi_check;
} or_cfg;

typedef struct or_counters {
  uint64_t rays, primary, extension, shadow, mis, heap_overflow;
} or_counters;

}  // extern "C"

namespace {

orc::Config to_cfg(const or_cfg* c) {
  orc::Config k;
  if (c) {
    k.mis = c->mis;
    k.rr_threshold = c->rr_threshold;
    k.max_depth = c->max_depth;
    k.brdf_model = c->brdf_model;
    k.mis_lobe_fix = c->mis_lobe_fix;
    k.heap_size = c->heap_size > 0 ? c->heap_size : 1500;
    k.gi_check = c->gi_check;
  }
  return k;
}

template <class R>
orc::Scene<R> mk_scene(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b,
                       int nb, const yc_quad_light* l, int nl) {
  orc::Scene<R> s;
  s.tris = t; s.n_tri = nt; s.mats = m; s.n_mat = nm; s.nodes = b; s.n_node = nb; s.lights = l; s.n_light = nl;
  return s;
}

void add(or_counters* o, const orc::Counters& c) {
  if (!o) return;
  o->rays += c.rays; o->primary += c.primary; o->extension += c.extension;
  o->shadow += c.shadow; o->mis += c.mis; o->heap_overflow += c.heap_overflow;
}

template <class R, class Acc>
int render(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
           const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, Acc* accum, uint32_t rand_,
           int reset, const or_cfg* cfg, int threads, int row0, int row1, or_counters* out, int bdpt_bounces = 0,
           int bdpt_mis = 0) {
  if (!cam || !accum || W <= 0 || H <= 0 || nl < 0 || nl > 16) return -1;
  if (row1 <= row0) { row0 = 0; row1 = H; }
  const orc::Scene<R> sc = mk_scene<R>(t, nt, m, nm, b, nb, l, nl);
  const orc::Config k = to_cfg(cfg);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next(row0);
  std::vector<orc::Counters> cnts(threads);
  auto work = [&](int tid) {
    orc::BdptMisTracer<R> tr(sc, k, cnts[tid], bdpt_bounces > 0 ? bdpt_bounces : 20);
    tr.bounces = bdpt_bounces > 0 ? bdpt_bounces : 20;
    for (;;) {
      const int y = next.fetch_add(1);
      if (y >= row1) break;
      for (int x = 0; x < W; ++x) {
        const orc::V4<R> c = bdpt_mis ? orc::pixel_sample_bdpt_mis<R>(tr, *cam, x, y, W, H, rand_)
                             : bdpt_bounces > 0 ? orc::pixel_sample_bdpt<R>(tr, *cam, x, y, W, H, rand_)
                                                : orc::pixel_sample<R>(tr, *cam, x, y, W, H, rand_);
        Acc* p = accum + 4 * ((size_t)y * W + x);
        const orc::V4<R> prev{(R)p[0], (R)p[1], (R)p[2], (R)p[3]};
        const orc::V4<R> o = orc::accumulate<R>(c, prev, reset);
        p[0] = (Acc)o.x; p[1] = (Acc)o.y; p[2] = (Acc)o.z; p[3] = (Acc)o.w;
      }
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(work, i);
  work(0);
  for (auto& th : pool) th.join();
  for (auto& c : cnts) add(out, c);
  return 0;
}

}  // namespace

extern "C" {

// traceRay on n explicit rays (origin xyzw, dir xyzw, length), udpt.cl:240-286.
// Writes the hit triangle (-1 none), the hit light (-1 none), the final ray length
// and whether the breadth-first queue overflowed.
int or_trace(const yc_triangle* t, int nt, const yc_bvh_node* b, int nb, const yc_quad_light* l, int nl,
             const float* rays, int n, int is_shadow, int heap_size, int* tri_out, int* light_out,
             float* t_out, int* overflow_out) {
  if (n < 0 || (n > 0 && (!rays || !tri_out || !t_out))) return -1;
  const orc::Scene<float> sc = mk_scene<float>(t, nt, nullptr, 0, b, nb, l, nl);
  orc::Config k;
  k.heap_size = heap_size > 0 ? heap_size : 1500;
  orc::Counters cnt;
  orc::Tracer<float> tr(sc, k, cnt);
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 9 * (size_t)i;
    orc::Ray<float> ray{{r[0], r[1], r[2], r[3]}, {r[4], r[5], r[6], r[7]}, r[8], is_shadow != 0};
    orc::Hit<float> hit;
    const uint64_t ov0 = cnt.heap_overflow;
    const bool h = tr.trace(ray, hit);
    tri_out[i] = h ? hit.tri : -1;
    if (light_out) light_out[i] = h ? hit.light : -1;
    t_out[i] = ray.length;
    if (overflow_out) overflow_out[i] = cnt.heap_overflow != ov0;
  }
  return 0;
}

// The rays one pass of pathtracer (udpt.cl:158-211) walks a BVH with over rows
// [row0, row1), in order (the Tracer::rec format, 8 floats per ray). Writes at most cap
// rays and their number to *n_out (the full count, which may exceed cap).
int or_record_rays(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                   const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, uint32_t rand_, const or_cfg* cfg,
                   int row0, int row1, float* out, int64_t cap, int64_t* n_out) {
  if (!cam || !out || !n_out || W <= 0 || H <= 0 || nl < 0 || nl > 16) return -1;
  if (row1 <= row0) { row0 = 0; row1 = H; }
  const orc::Scene<float> sc = mk_scene<float>(t, nt, m, nm, b, nb, l, nl);
  const orc::Config k = to_cfg(cfg);
  orc::Counters cnt;
  orc::Tracer<float> tr(sc, k, cnt);
  std::vector<float> rec;
  tr.rec = &rec;
  for (int y = row0; y < row1; ++y)
    for (int x = 0; x < W; ++x) orc::pixel_sample<float>(tr, *cam, x, y, W, H, rand_);
  const int64_t n = (int64_t)(rec.size() / 8);
  *n_out = n;
  std::memcpy(out, rec.data(), (size_t)std::min(n, cap) * 8 * sizeof(float));
  return 0;
}

// One pass of pathtracer (udpt.cl:158-211) over rows [row0, row1) of a W x H RGBA32F
// accumulator updated in place (row1 <= row0 means the whole image).
int or_render(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
              const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, float* accum, uint32_t rand_,
              int reset, const or_cfg* cfg, int threads, int row0, int row1, or_counters* out) {
  return render<float, float>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads, row0,
                              row1, out);
}

// One pass of the BDPT `pathtracer` (kernels/legacy/bdpt.cl:158-210) with
// BDPT_BOUNCES = bounces (<= 32).
int or_render_bdpt(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                   const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, float* accum, uint32_t rand_,
                   int reset, const or_cfg* cfg, int bounces, int threads, int row0, int row1, or_counters* out) {
  if (bounces < 2 || bounces > 32) return -1;
  return render<float, float>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads, row0, row1,
                              out, bounces);
}

int or_render_bdpt_f64(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                       const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, double* accum,
                       uint32_t rand_, int reset, const or_cfg* cfg, int bounces, int threads, int row0, int row1,
                       or_counters* out) {
  if (bounces < 2 || bounces > 32) return -1;
  return render<double, double>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads, row0,
                                row1, out, bounces);
}

// One pass of the bidirectional tracer with multiple importance sampling
// (bdpt_mis_oracle.hpp), paths of at most kmax segments (3 <= kmax <= 32).
int or_render_bdpt_mis(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                       const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, float* accum, uint32_t rand_,
                       int reset, const or_cfg* cfg, int kmax, int threads, int row0, int row1, or_counters* out) {
  if (kmax < 3 || kmax > 32) return -1;
  return render<float, float>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads, row0, row1,
                              out, kmax, 1);
}

int or_render_bdpt_mis_f64(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                           const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, double* accum,
                           uint32_t rand_, int reset, const or_cfg* cfg, int kmax, int threads, int row0, int row1,
                           or_counters* out) {
  if (kmax < 3 || kmax > 32) return -1;
  return render<double, double>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads, row0,
                                row1, out, kmax, 1);
}

// The same pass evaluated in double precision into a double accumulator.
int or_render_f64(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                  const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, double* accum,
                  uint32_t rand_, int reset, const or_cfg* cfg, int threads, int row0, int row1,
                  or_counters* out) {
  return render<double, double>(t, nt, m, nm, b, nb, l, nl, cam, W, H, accum, rand_, reset, cfg, threads,
                                row0, row1, out);
}

// Converged-image reference: n_pass passes (seeds[k]) of the FP64 restatement over an
// explicit pixel list, accumulated as a running mean into out (n x 4 doubles). Used for
// the RMSE of a configuration against a high-spp double-precision image.
int or_render_pixels_f64(const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b, int nb,
                         const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, const int* xs,
                         const int* ys, int n, const uint32_t* seeds, int n_pass, const or_cfg* cfg, int bdpt_bounces,
                         int threads, double* out, int bdpt_mis) {
  if (!cam || !xs || !ys || !seeds || !out || n < 0 || n_pass <= 0) return -1;
  const orc::Scene<double> sc = mk_scene<double>(t, nt, m, nm, b, nb, l, nl);
  const orc::Config k = to_cfg(cfg);
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next(0);
  auto work = [&]() {
    orc::Counters cnt;
    orc::BdptMisTracer<double> tr(sc, k, cnt, bdpt_bounces > 0 ? bdpt_bounces : 20);
    tr.bounces = bdpt_bounces > 0 ? bdpt_bounces : 20;
    for (;;) {
      const int i = next.fetch_add(1);
      if (i >= n) break;
      orc::V4<double> acc{0, 0, 0, 0};
      for (int p = 0; p < n_pass; ++p) {
        const orc::V4<double> c = bdpt_mis ? orc::pixel_sample_bdpt_mis<double>(tr, *cam, xs[i], ys[i], W, H, seeds[p])
                                  : bdpt_bounces > 0 ? orc::pixel_sample_bdpt<double>(tr, *cam, xs[i], ys[i], W, H, seeds[p])
                                                   : orc::pixel_sample<double>(tr, *cam, xs[i], ys[i], W, H, seeds[p]);
        acc = orc::accumulate<double>(c, acc, p == 0 ? 1 : 0);
      }
      out[4 * (size_t)i + 0] = acc.x;
      out[4 * (size_t)i + 1] = acc.y;
      out[4 * (size_t)i + 2] = acc.z;
      out[4 * (size_t)i + 3] = acc.w;
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(work);
  work();
  for (auto& th : pool) th.join();
  return 0;
}

// tonemap, kernels/post-proc/tonemap.cl:14-47: Reinhard with L_white = 1 on Y + 0.001,
// then pow(., 1/2.2); the clamp result is discarded as in tonemap.cl:32.
int or_tonemap(const float* in, int W, int H, float* out) {
  if (!in || !out || W <= 0 || H <= 0) return -1;
  const size_t n = (size_t)W * H;
  const float inv_gamma = ym::div(1.0f, 2.2f);
  for (size_t i = 0; i < n; ++i) {
    const float* c = in + 4 * i;
    float y = ym::mul(0.212671f, c[0]);
    y = ym::add(y, ym::mul(0.715160f, c[1]));
    y = ym::add(y, ym::mul(0.072169f, c[2]));
    y = ym::add(y, 0.001f);
    const float ld = ym::div(ym::mul(y, ym::add(1.0f, ym::div(y, ym::mul(1.0f, 1.0f)))), ym::add(1.0f, y));
    for (int k = 0; k < 4; ++k) {
      const float s = ym::mul(ld, ym::pow(ym::div(c[k], y), 1.0f));
      out[4 * i + k] = ym::pow(s, inv_gamma);
    }
  }
  return 0;
}

// Per-function probes used by the known-answer tests.
int or_ym_eval(int fn, const float* a, const float* b, float* out, int n) {
  for (int i = 0; i < n; ++i) {
    switch (fn) {
      case 0: out[i] = ym::sin(a[i]); break;
      case 1: out[i] = ym::cos(a[i]); break;
      case 2: out[i] = ym::pow(a[i], b[i]); break;
      case 3: out[i] = ym::exp2(a[i]); break;
      case 4: out[i] = a[i] > 0 ? ym::log2_pos(a[i]) : 0.0f; break;
      default: return -1;
    }
  }
  return 0;
}

uint32_t or_wang_hash(uint32_t s) { return ym::wang_hash(s); }
uint32_t or_xor_shift(uint32_t s) { return ym::xor_shift(s); }

// evaluateBRDF (udpt.cl:611-630, Oren-Nayar of udpt-primitives.cl:696-725 when
// brdf_model = 1) for one triangle hit, used to pin the BRDF terms one by one.
int or_brdf(const yc_triangle* t, int nt, const yc_material* m, int nm, int tri, const float* hit_point,
            const float* normal, const float* w_i, const float* w_o, int glossy, float rr_prob, int brdf_model,
            float* out) {
  const orc::Scene<float> sc = mk_scene<float>(t, nt, m, nm, nullptr, 0, nullptr, 0);
  orc::Config k;
  k.brdf_model = brdf_model;
  orc::Counters cnt;
  orc::Tracer<float> tr(sc, k, cnt);
  orc::Hit<float> h;
  h.tri = tri;
  h.hit_point = {hit_point[0], hit_point[1], hit_point[2], hit_point[3]};
  h.normal = {normal[0], normal[1], normal[2], normal[3]};
  const orc::V4<float> c = tr.brdf({w_i[0], w_i[1], w_i[2], w_i[3]}, {w_o[0], w_o[1], w_o[2], w_o[3]}, h,
                                   glossy != 0, rr_prob);
  out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
  return 0;
}

}  // extern "C"
