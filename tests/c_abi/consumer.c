/* consumer.c -- a plain C11 caller of include/yune_cuda.h and include/yune_host.h.
 *
 * Checks that the headers and libyune_gb300.so form a C ABI a non-C++ host can bind
 * (plain structs, pointers and sizes; no C++ or torch types): it builds a scene with the
 * host producers, its BVH (BVH::createBVH), its device layout and a camera, refits the
 * BVH on the unmoved triangles (must not change a byte), writes and reads back a scene
 * cache file, writes a PNG, checks the request server's admission rules (host only) and
 * opens a core context. Without a CUDA device yc_create must fail cleanly with
 * a negative code and a message; with one the context is created and destroyed.
 * Usage: consumer <scratch directory>. Prints "ok" and exits 0 when every check holds.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "yune_cuda.h"
#include "yune_host.h"

static int failures = 0;

#define CHECK(cond, what)                                   \
  do {                                                      \
    if (!(cond)) {                                          \
      fprintf(stderr, "check failed: %s (%s)\n", what, #cond); \
      ++failures;                                           \
    }                                                       \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <scratch directory>\n", argv[0]);
    return 2;
  }
  char path[4096];

  /* a Cornell box with a diffuse icosphere */
  yh_scene* sc = NULL;
  CHECK(yh_scene_new(&sc) == YH_OK && sc, "yh_scene_new");
  CHECK(yh_scene_add_cornell(sc, 7u, 0.09f, 50.0f, 15.0f, 1) == YH_OK, "yh_scene_add_cornell");
  yc_material m;
  memset(&m, 0, sizeof m);
  m.kd.x = m.kd.y = m.kd.z = 0.5f;
  m.kd.w = m.ke.w = m.ks.w = 1.0f;
  m.n = m.k = m.px = m.py = 1.0f;
  m.alpha_x = m.alpha_y = 100.0f;
  int mat_id = -1;
  CHECK(yh_scene_add_material(sc, &m, &mat_id) == YH_OK && mat_id >= 0, "yh_scene_add_material");
  const float centre[3] = {0.1f, -0.1f, 0.0f};
  CHECK(yh_scene_add_icosphere(sc, centre, 0.25f, 3, 0.02f, 11u, mat_id) == YH_OK, "yh_scene_add_icosphere");
  int n_tri = 0, n_mat = 0, n_light = 0;
  CHECK(yh_scene_counts(sc, &n_tri, &n_mat, &n_light) == YH_OK, "yh_scene_counts");
  CHECK(n_tri == 34 + 20 * 64 && n_light == 1, "triangle and light counts");
  yc_triangle* tris = (yc_triangle*)malloc(sizeof(yc_triangle) * (size_t)n_tri);
  yc_material* mats = (yc_material*)malloc(sizeof(yc_material) * (size_t)n_mat);
  yc_quad_light* lights = (yc_quad_light*)malloc(sizeof(yc_quad_light) * (size_t)n_light);
  CHECK(tris && mats && lights, "malloc");
  CHECK(yh_scene_copy(sc, tris, mats, lights) == YH_OK, "yh_scene_copy");
  yh_scene_free(sc);

  /* BVH::createBVH: 20 bins, leaves of up to 10 triangles */
  yh_bvh* bvh = NULL;
  CHECK(yh_bvh_build(tris, n_tri, 20, 10, &bvh) == YH_OK && bvh, "yh_bvh_build");
  const int n_node = yh_bvh_node_count(bvh);
  CHECK(n_node > 1, "node count");
  yc_bvh_node* nodes = (yc_bvh_node*)malloc(sizeof(yc_bvh_node) * (size_t)n_node);
  yc_bvh_node* refit = (yc_bvh_node*)malloc(sizeof(yc_bvh_node) * (size_t)n_node);
  CHECK(nodes && refit, "malloc nodes");
  CHECK(yh_bvh_copy_nodes(bvh, nodes, n_node) == YH_OK, "yh_bvh_copy_nodes");
  CHECK(yh_bvh_copy_nodes(bvh, nodes, n_node - 1) == YH_E_RANGE, "copy into too small an array");
  const int depth = yh_bvh_depth(bvh);
  CHECK(depth > 0, "depth");
  yh_bvh_free(bvh);
  memcpy(refit, nodes, sizeof(yc_bvh_node) * (size_t)n_node);
  CHECK(yh_bvh_refit(tris, n_tri, refit, n_node) == YH_OK, "yh_bvh_refit");
  CHECK(memcmp(refit, nodes, sizeof(yc_bvh_node) * (size_t)n_node) == 0, "refit of unmoved triangles");

  /* the device layout of the upload, computed on the host */
  yc_scene_layout_info lay;
  CHECK(yc_scene_layout(tris, n_tri, n_mat, nodes, n_node, 1, &lay) == YC_OK, "yc_scene_layout");
  CHECK(lay.stream_bytes == 48u * (uint64_t)n_tri && lay.shade_bytes == 64u * (uint64_t)n_tri &&
        lay.device_bytes > lay.node_bytes + lay.stream_bytes + lay.shade_bytes && lay.depth > 0,
        "layout sizes");
  CHECK(yc_scene_layout(tris, n_tri, 0, nodes, n_node, 1, &lay) == YC_E_INVALID && yc_last_error()[0],
        "layout refuses triangles without materials");

  /* Camera::setBuffer */
  const float eye[3] = {0, 0, 1.4f}, side[3] = {1, 0, 0}, up[3] = {0, 1, 0}, look[3] = {0, 0, -1};
  yc_cam cam;
  CHECK(yh_camera_look(eye, side, up, look, 60.0f, &cam) == YH_OK, "yh_camera_look");

  /* scene cache round trip */
  snprintf(path, sizeof path, "%s/scene.ysc", argv[1]);
  const char meta[] = "{\"width\": 32, \"height\": 32}";
  CHECK(yh_cache_save(path, 42u, tris, n_tri, mats, n_mat, lights, n_light, nodes, n_node, depth, &cam, meta,
                      (int)sizeof meta) == YH_OK, "yh_cache_save");
  yh_cache_info info;
  CHECK(yh_cache_query(path, &info) == YH_OK, "yh_cache_query");
  CHECK(info.key == 42u && info.n_tri == n_tri && info.n_node == n_node && info.depth == depth &&
        info.has_cam == 1 && info.meta_bytes == (int)sizeof meta, "cache header");
  yc_triangle* t2 = (yc_triangle*)malloc(sizeof(yc_triangle) * (size_t)n_tri);
  yc_material* m2 = (yc_material*)malloc(sizeof(yc_material) * (size_t)n_mat);
  yc_quad_light* l2 = (yc_quad_light*)malloc(sizeof(yc_quad_light) * (size_t)n_light);
  yc_bvh_node* nd2 = (yc_bvh_node*)malloc(sizeof(yc_bvh_node) * (size_t)n_node);
  yc_cam cam2;
  char meta2[64];
  CHECK(t2 && m2 && l2 && nd2, "malloc cache arrays");
  CHECK(yh_cache_load(path, 43u, t2, n_tri, m2, n_mat, l2, n_light, nd2, n_node, &cam2, meta2,
                      (int)sizeof meta2) == YH_E_STALE, "stale key");
  CHECK(yh_cache_load(path, 42u, t2, n_tri, m2, n_mat, l2, n_light, nd2, n_node, &cam2, meta2,
                      (int)sizeof meta2) == YH_OK, "yh_cache_load");
  CHECK(memcmp(t2, tris, sizeof(yc_triangle) * (size_t)n_tri) == 0 &&
        memcmp(m2, mats, sizeof(yc_material) * (size_t)n_mat) == 0 &&
        memcmp(l2, lights, sizeof(yc_quad_light) * (size_t)n_light) == 0 &&
        memcmp(nd2, nodes, sizeof(yc_bvh_node) * (size_t)n_node) == 0 && memcmp(&cam2, &cam, sizeof cam) == 0 &&
        memcmp(meta2, meta, sizeof meta) == 0, "cache contents");

  /* image output: a 16 x 8 gradient */
  float rgba[16 * 8 * 4];
  for (int i = 0; i < 16 * 8; ++i) {
    rgba[4 * i + 0] = (float)(i % 16) / 15.0f;
    rgba[4 * i + 1] = (float)(i / 16) / 7.0f;
    rgba[4 * i + 2] = 0.5f;
    rgba[4 * i + 3] = 1.0f;
  }
  snprintf(path, sizeof path, "%s/gradient.png", argv[1]);
  CHECK(yh_write_png(path, 16, 8, rgba) == YH_OK, "yh_write_png");
  FILE* f = fopen(path, "rb");
  unsigned char sig[8] = {0};
  CHECK(f && fread(sig, 1, 8, f) == 8 && sig[1] == 'P' && sig[2] == 'N' && sig[3] == 'G', "PNG signature");
  if (f) fclose(f);

  /* the core: a context where a device exists, a clean error where none does */
  yc_ctx* ctx = NULL;
  const int rc = yc_create(0, &ctx);
  if (rc == YC_OK) {
    CHECK(ctx != NULL, "context");
    CHECK(yc_destroy(ctx) == YC_OK, "yc_destroy");
    printf("device: context created\n");
  } else {
    const char* msg = yc_last_error();
    CHECK(rc < 0 && msg && msg[0], "yc_create error code and message");
    printf("device: none (%d: %s)\n", rc, msg ? msg : "");
  }
  CHECK(yc_upload_scene(NULL, tris, n_tri, mats, n_mat, nodes, n_node, lights, n_light, NULL) == YC_E_INVALID,
        "yc_upload_scene without a context");

  /* the server's admission rules, host only: a budget for two 16 x 16 requests of two
   * passes, one waiting place */
  {
    const uint64_t req = 16u * 16u * 16u + 8u;
    yc_admission* adm = NULL;
    CHECK(yc_admission_create(2 * req, 1, &adm) == YC_OK && adm, "yc_admission_create");
    int64_t t[5];
    int32_t st[5];
    for (int i = 0; i < 4; ++i) CHECK(yc_admission_submit(adm, req, &t[i], &st[i]) == YC_OK, "submit");
    CHECK(yc_admission_submit(adm, 64u * 64u * 16u + 8u, &t[4], &st[4]) == YC_OK, "submit large");
    CHECK(st[0] == YC_REQ_RUNNING && st[1] == YC_REQ_RUNNING && st[2] == YC_REQ_WAITING &&
              st[3] == YC_REQ_REJECTED_QUEUE && st[4] == YC_REQ_REJECTED_BUDGET,
          "admission states");
    int64_t next = 0;
    CHECK(yc_admission_next(adm, &next) == YC_OK && next == -1, "nothing fits yet");
    int32_t s = -1;
    CHECK(yc_admission_cancel(adm, t[0], &s) == YC_OK && s == YC_REQ_CANCELLING, "cancel a running request");
    CHECK(yc_admission_finish(adm, t[0], &s) == YC_OK && s == YC_REQ_CANCELLED, "its work drained");
    CHECK(yc_admission_next(adm, &next) == YC_OK && next == t[2], "the waiting request is admitted");
    uint64_t bytes = 0;
    int32_t waiting = -1, running = -1;
    CHECK(yc_admission_usage(adm, &bytes, &waiting, &running) == YC_OK && bytes == 2 * req && waiting == 0 &&
              running == 2,
          "bytes in use");
    CHECK(yc_admission_finish(adm, t[3], &s) == YC_E_INVALID, "a rejected request holds nothing");
    CHECK(yc_admission_destroy(adm) == YC_OK, "yc_admission_destroy");
  }

  free(tris); free(mats); free(lights); free(nodes); free(refit);
  free(t2); free(m2); free(l2); free(nd2);
  if (failures) {
    printf("%d checks failed\n", failures);
    return 1;
  }
  printf("ok\n");
  return 0;
}
