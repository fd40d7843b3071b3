// ref_harness.cpp -- drives Yune's own kernel code, compiled as C++ on the CPU.
//
// TEST INFRASTRUCTURE: built into oracle/_ref/libyune_ref.so by oracle/build_oracle.py
// from the reference files where they lie (kernels/legacy/udpt.cl, bdpt.cl,
// udpt-primitives.cl, kernels/post-proc/tonemap.cl after the syntax-only transform of
// transform.py, plus src/BVH.cpp, src/TriangleCPU.cpp, src/BVHNodeCPU.cpp unchanged).
// Each variant of a kernel is the same text included under different #defines:
//   udpt_a      udpt.cl as shipped (no MIS, RR_THRESHOLD 6, LIGHT_SIZE 1)
//   udpt_mis    udpt.cl with -DMIS
//   udpt_mis4   udpt.cl with -DMIS and LIGHT_SIZE 4
//   udpt_mis_on udpt.cl with -DMIS and the Oren-Nayar diffuse rule of udpt-primitives.cl
//               (udpt_on.inc, transform.graft_oren_nayar): the configurations' variant B
//   bdpt8/20    bdpt.cl with BDPT_BOUNCES 8 / 20 (shipped: 20), LIGHT_SIZE 1
//   bdpt8_l4    bdpt.cl with BDPT_BOUNCES 8 and LIGHT_SIZE 4
// RR_THRESHOLD (udpt.cl) and the GI-loop bound are read at run time.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "cl_shim.hpp"

namespace yref {

#define YREF_MAX_DEPTH (yref_max_depth)

namespace udpt_a {
#define RR_THRESHOLD (yref_rr_threshold)
#include "udpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace udpt_a

namespace udpt_mis {
#define MIS
#define RR_THRESHOLD (yref_rr_threshold)
#include "udpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef MIS
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace udpt_mis

namespace udpt_mis4 {
#define MIS
#define LIGHT_SIZE 4
#define RR_THRESHOLD (yref_rr_threshold)
#include "udpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef LIGHT_SIZE
#undef MIS
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace udpt_mis4

namespace udpt_mis_on {
#define MIS
#define RR_THRESHOLD (yref_rr_threshold)
#include "udpt_on.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef MIS
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace udpt_mis_on

namespace bdpt20 {
#include "bdpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef LIGHT_SIZE
#undef HEAP_SIZE
#undef BDPT_BOUNCES
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace bdpt20

namespace bdpt8 {
#define BDPT_BOUNCES 8
#include "bdpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef LIGHT_SIZE
#undef HEAP_SIZE
#undef BDPT_BOUNCES
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace bdpt8

namespace bdpt8_l4 {
#define BDPT_BOUNCES 8
#define LIGHT_SIZE 4
#include "bdpt.inc"
constexpr int kLights = LIGHT_SIZE;
#undef RR_THRESHOLD
#undef LIGHT_SIZE
#undef HEAP_SIZE
#undef BDPT_BOUNCES
#undef PI
#undef INV_PI
#undef EPSILON
}  // namespace bdpt8_l4

namespace tonemap_k {
#include "tonemap.inc"
#undef EPSILON
}  // namespace tonemap_k

namespace prim {
#include "primitives.inc"
#undef RR_THRESHOLD
#undef LIGHT_SIZE
}  // namespace prim

}  // namespace yref

#include "../../include/yune_types.h"

namespace {

template <class K>
void set_lights(K* dst, int cap, const yc_quad_light* l, int n) {
  for (int i = 0; i < cap; ++i) {
    const yc_quad_light& s = l[i < n ? i : n - 1];
    auto f = [](const yc_float4& v) { return yref::float4(v.x, v.y, v.z, v.w); };
    dst[i].pos = f(s.pos);
    dst[i].ke = f(s.ke);
    dst[i].kd = f(s.kd);
    dst[i].ks = f(s.ks);
    dst[i].edge_l = f(s.edge_l);
    dst[i].edge_w = f(s.edge_w);
    dst[i].phong_exponent = s.phong_exponent;
  }
}
template <class K> void set_normal_udpt(K* dst, int cap, const yc_quad_light* l, int n) {
  for (int i = 0; i < cap; ++i) { const yc_float4& v = l[i < n ? i : n - 1].normal; dst[i].normal = yref::float4(v.x, v.y, v.z, v.w); }
}
template <class K> void set_normal_bdpt(K* dst, int cap, const yc_quad_light* l, int n) {
  for (int i = 0; i < cap; ++i) { const yc_float4& v = l[i < n ? i : n - 1].normal; dst[i].norm = yref::float4(v.x, v.y, v.z, v.w); }
}

template <class Fn>
void parallel_rows(int row0, int H, int threads, Fn fn) {
  if (threads <= 0) threads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int> next(row0);
  auto work = [&]() {
    for (;;) {
      const int y = next.fetch_add(1);
      if (y >= H) break;
      fn(y);
    }
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < threads; ++i) pool.emplace_back(work);
  work();
  for (auto& t : pool) t.join();
}

}  // namespace

static_assert(sizeof(yref::udpt_a::Triangle) == sizeof(yc_triangle), "Triangle");
static_assert(sizeof(yref::udpt_a::Material) == sizeof(yc_material), "Material");
static_assert(sizeof(yref::udpt_a::BVHNodeGPU) == sizeof(yc_bvh_node), "BVHNodeGPU");
static_assert(sizeof(yref::udpt_a::Camera) == sizeof(yc_cam), "Camera");

#define YREF_RENDER(NS, SETN)                                                                         \
  do {                                                                                                \
    using namespace yref::NS;                                                                         \
    if (nl < 1 || nl > kLights) return -2;                                                            \
    set_lights(light_sources, kLights, l, nl);                                                        \
    SETN(light_sources, kLights, l, nl);                                                              \
    yref::image2d_t img{reinterpret_cast<yref::float4*>(accum), W, H};                                \
    parallel_rows(row0, row1, threads, [&](int y) {                                                            \
      for (int x = 0; x < W; ++x) {                                                                   \
        yref::tl_gid[0] = (size_t)x;                                                                  \
        yref::tl_gid[1] = (size_t)y;                                                                  \
        pathtracer(img, img, (Camera*)(cam), nt, (Triangle*)(t), (Material*)(m), \
                   nb, (BVHNodeGPU*)(b), gi_check, reset, rand_, 0, 1, 1);                             \
      }                                                                                               \
    });                                                                                               \
  } while (0)

extern "C" {

// One pass of the reference `pathtracer` kernel over rows [row0, row1) of a W x H
// RGBA32F accumulator, updated in place (row1 <= row0: the whole image). variant: 0 udpt_a, 1 udpt_mis, 2 udpt_mis4, 3 udpt_mis_on, 10 bdpt20, 11 bdpt8,
// 12 bdpt8_l4.
int ref_render(int variant, const yc_triangle* t, int nt, const yc_material* m, int nm, const yc_bvh_node* b,
               int nb, const yc_quad_light* l, int nl, const yc_cam* cam, int W, int H, float* accum,
               uint32_t rand_, int reset, int gi_check, int rr_threshold, int max_depth, int threads, int row0,
               int row1) {
  (void)nm;
  if (!cam || !accum || W <= 0 || H <= 0 || !l) return -1;
  if (row1 <= row0) { row0 = 0; row1 = H; }
  // bdpt.cl keeps extending the eye path after the camera ray hits the light, from a
  // vertex whose triangle_ID is -1, so it reads scene_data[-1]; give it a valid record
  // there (material 0). The pixel colour does not depend on it.
  std::vector<yc_triangle> padded;
  if (variant >= 10) {
    padded.resize((size_t)nt + 1);
    std::memset(padded.data(), 0, sizeof(yc_triangle));
    if (nt > 0) std::memcpy(padded.data() + 1, t, (size_t)nt * sizeof(yc_triangle));
    t = padded.data() + 1;
  }
  yref::yref_rr_threshold = rr_threshold;
  yref::yref_max_depth = max_depth;
  switch (variant) {
    case 0: YREF_RENDER(udpt_a, set_normal_udpt); break;
    case 1: YREF_RENDER(udpt_mis, set_normal_udpt); break;
    case 2: YREF_RENDER(udpt_mis4, set_normal_udpt); break;
    case 3: YREF_RENDER(udpt_mis_on, set_normal_udpt); break;
    case 10: YREF_RENDER(bdpt20, set_normal_bdpt); break;
    case 11: YREF_RENDER(bdpt8, set_normal_bdpt); break;
    case 12: YREF_RENDER(bdpt8_l4, set_normal_bdpt); break;
    default: return -1;
  }
  return 0;
}

// The reference traceRay (udpt.cl:240-286) on explicit rays: origin xyzw, dir xyzw,
// length, 9 floats per ray.
int ref_trace(const yc_triangle* t, int nt, const yc_bvh_node* b, int nb, const yc_quad_light* l, int nl,
              const float* rays, int n, int is_shadow, int* tri_out, int* light_out, float* t_out) {
  using namespace yref::udpt_a;
  if (nl != 1 || !l) return -2;
  set_lights(light_sources, kLights, l, nl);
  set_normal_udpt(light_sources, kLights, l, nl);
  for (int i = 0; i < n; ++i) {
    const float* r = rays + 9 * (size_t)i;
    Ray ray;
    ray.origin = yref::float4(r[0], r[1], r[2], r[3]);
    ray.dir = yref::float4(r[4], r[5], r[6], r[7]);
    ray.length = r[8];
    ray.is_shadow_ray = is_shadow != 0;
    HitInfo hit = {-1, -1, yref::float4(0, 0, 0, 1), yref::float4(0, 0, 0, 0)};
    const bool h = traceRay(&ray, &hit, nb, (BVHNodeGPU*)b, nt, (Triangle*)t);
    tri_out[i] = h ? hit.triangle_ID : -1;
    if (light_out) light_out[i] = h ? hit.light_ID : -1;
    t_out[i] = ray.length;
  }
  return 0;
}

// The reference tonemap kernel (tonemap.cl:14-35) over a W x H image.
int ref_tonemap(const float* in, int W, int H, float* out) {
  using namespace yref::tonemap_k;
  std::vector<yref::float4> cur((size_t)W * H);
  std::memcpy(cur.data(), in, cur.size() * sizeof(yref::float4));
  yref::image2d_t a{cur.data(), W, H};
  yref::image2d_t o{reinterpret_cast<yref::float4*>(out), W, H};
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      yref::tl_gid[0] = (size_t)x;
      yref::tl_gid[1] = (size_t)y;
      tonemap(a, a, o, 0);
    }
  return 0;
}

// OrenNayarBRDF of udpt-primitives.cl:696-725 for one material and shading frame.
int ref_oren_nayar(const yc_material* mat, const float* hit_point, const float* normal, const float* w_i,
                   const float* w_o, float* out) {
  using namespace yref::prim;
  std::memcpy((void*)&materials[0], mat, sizeof(yc_material));
  walls[0].matID = 0;
  HitInfo h;
  h.sphereID = -1; h.quadID = 0; h.lightID = -1;
  h.hit_point = yref::float4(hit_point[0], hit_point[1], hit_point[2], hit_point[3]);
  h.normal = yref::float4(normal[0], normal[1], normal[2], normal[3]);
  const yref::float4 c = OrenNayarBRDF(yref::float4(w_i[0], w_i[1], w_i[2], w_i[3]),
                                       yref::float4(w_o[0], w_o[1], w_o[2], w_o[3]), h);
  out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
  return 0;
}

}  // extern "C"

#ifndef YREF_NO_HOST
// The reference BVH builder (src/BVH.cpp) over the triangles, with the root box computed
// as Scene::loadModel does (src/Scene.cpp:350-356).
#define private public
#include "BVH.h"
#undef private

extern "C" int ref_bvh_build(const yc_triangle* t, int nt, int bins, int leaf, yc_bvh_node* out, int cap,
                             int* n_out) {
  std::vector<yune::TriangleCPU> list(nt);
  AABB root;
  const float inf = std::numeric_limits<float>::max();
  root.p_min = {inf, inf, inf, 1.0};
  root.p_max = {-inf, -inf, -inf, 1.0};
  for (int i = 0; i < nt; ++i) {
    std::memcpy(&list[i].props, &t[i], sizeof(yc_triangle));
    list[i].computeCentroid();
    for (int k = 0; k < 3; ++k) {
      root.p_min.s[k] = std::min(root.p_min.s[k], list[i].aabb.p_min.s[k]);
      root.p_max.s[k] = std::max(root.p_max.s[k], list[i].aabb.p_max.s[k]);
    }
  }
  yune::BVH bvh;
  bvh.leaf_primitives = leaf;
  bvh.createBVH(root, list, bins);
  *n_out = (int)bvh.gpu_node_list.size();
  if ((int)bvh.gpu_node_list.size() > cap) return -3;
  std::memcpy(out, bvh.gpu_node_list.data(), bvh.gpu_node_list.size() * sizeof(yc_bvh_node));
  return 0;
}

// The reference OBJ/MTL loader (Scene::loadModel, src/Scene.cpp:133-383, compiled
// unchanged against glm stand-ins). Its Camera member is never used by the loader; the
// two Camera members the Scene object needs are defined here as no-ops (the camera code
// needs the full glm).
#define private public
#include "Scene.h"
#undef private
namespace yune {
Camera::Camera() {}
Camera::~Camera() {}
}  // namespace yune

extern "C" int ref_load_obj(const char* path, const char* filename, yc_triangle* tris, int cap_t, int* nt,
                            yc_material* mats, int cap_m, int* nm, yc_bvh_node* nodes, int cap_n, int* nn) {
  yune::Scene s;
  try {
    s.loadModel(path, filename);
  } catch (...) {
    return -1;
  }
  *nt = (int)s.vert_data.size();
  *nm = (int)s.mat_data.size();
  *nn = (int)s.bvh.gpu_node_list.size();
  if (*nt > cap_t || *nm > cap_m || *nn > cap_n) return -3;
  for (int i = 0; i < *nt; ++i) std::memcpy(&tris[i], &s.vert_data[i], sizeof(yc_triangle));
  for (int i = 0; i < *nm; ++i) std::memcpy(&mats[i], &s.mat_data[i], sizeof(yc_material));
  if (*nn) std::memcpy(nodes, s.bvh.gpu_node_list.data(), (size_t)*nn * sizeof(yc_bvh_node));
  return 0;
}
#endif
