/* yune_host.h -- host-side producers of the buffers the CUDA core consumes.
 *
 * In Yune these buffers come from Scene/BVH/Camera, which stay on the caller's side
 * of the boundary. This library restates those producers so that a headless caller
 * (tests, the benchmark, a batch or serving front end) can build the same
 * TriangleGPU / BVHNodeGPU / Cam arrays without the GUI application:
 *   yh_bvh_build      <- BVH::createBVH          src/BVH.cpp:56-173 (node array
 *                        identical to the reference builder's for the same input)
 *   yh_triangle_aabb  <- TriangleCPU::computeAABB src/TriangleCPU.cpp:51-71
 *   yh_camera_look    <- Camera::setViewMatrix + Camera::setBuffer
 *                        src/Camera.cpp:66-82,105-117
 *   yh_scene_*        procedural scenes (Cornell box, seeded boxes, subdivided and
 *                     displaced icospheres, sphere grids), and OBJ/MTL files
 *                     (yh_scene_load_obj <- Scene::loadModel src/Scene.cpp:133-383)
 *   yh_cache_*        binary scene cache (new: Yune re-reads its OBJ file and rebuilds
 *                     the BVH on every start)
 * Every function returns 0 on success and a negative YH_E* code on failure.
 */
#ifndef YUNE_HOST_H
#define YUNE_HOST_H

#include "yune_types.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  YH_OK = 0,
  YH_E_INVALID = -1,      /* bad argument */
  YH_E_NOMEM = -2,        /* host allocation failed */
  YH_E_RANGE = -3,        /* index or size out of range */
  YH_E_IO = -4,           /* a file cannot be opened, read or written */
  YH_E_FORMAT = -5,       /* not a scene cache of this format, truncated, or corrupt */
  YH_E_STALE = -6         /* a scene cache made for another key */
};

/* ---- host threads ----
 * The host producers (yh_bvh_build, yh_cache_*) and the scene repack inside
 * yc_upload_scene run on every core the host reports unless a limit is set here
 * (process-wide; n = 0 lifts it). Their outputs do not depend on the thread count. No
 * reference counterpart: Yune builds its BVH on one thread.
 * yh_get_host_threads: the count in effect. */
int yh_set_host_threads(int n);
int yh_get_host_threads(void);

/* ---- BVH (src/BVH.cpp) ---- */
typedef struct yh_bvh yh_bvh;
/* Builds the breadth-first binned BVH of BVH::createBVH over tris[0..n_tri).
 * YH_E_RANGE: the tree would pass 1024 levels, which happens when more than leaf_max
 * triangles share one centroid (the reference builder does not terminate there).
 * bins: BVH::bins (20 by default; <= 2 selects median splits only).
 * leaf_max: BVH::leaf_primitives (10 in the reference; 1..10).
 * The root box is the union of the padded triangle boxes, as Scene::loadModel
 * computes it (src/Scene.cpp:350-356). */
int yh_bvh_build(const yc_triangle* tris, int n_tri, int bins, int leaf_max, yh_bvh** out);
int yh_bvh_node_count(const yh_bvh* b);
int yh_bvh_copy_nodes(const yh_bvh* b, yc_bvh_node* out, int capacity);
/* Longest root-to-leaf path (edges); the traversal stack needs depth + 1 slots. */
int yh_bvh_depth(const yh_bvh* b);
void yh_bvh_free(yh_bvh* b);

/* Refits nodes[0..n_node) in place after the triangles moved (same count, same
 * indices): the bottom-up pass BVH::createBVH ends with (BVH::resizeBvh,
 * src/BVH.cpp:218-247) run on the new positions. A leaf's box becomes the union of its
 * triangles' padded boxes (TriangleCPU::computeAABB), an interior node's the union of its
 * two children, an empty node keeps its box. Which triangles share a leaf does not
 * change: traversal stays exact, and slows down as the geometry departs from the one the
 * tree was built for (rebuild then). On unmoved triangles the array is unchanged, bit
 * for bit. Upload the refitted array with yc_upload_scene as any other. YH_E_RANGE: a
 * leaf entry outside [0, n_tri), a vert_len above 10, or a child index that does not
 * come after its parent (the reference's breadth-first order). No reference counterpart
 * as an entry point: Yune rebuilds the whole tree when a scene changes. */
int yh_bvh_refit(const yc_triangle* tris, int n_tri, yc_bvh_node* nodes, int n_node);

/* TriangleCPU::computeCentroid / computeAABB for one triangle. */
int yh_triangle_aabb(const yc_triangle* t, yc_aabb* aabb, yc_float4* centroid);

/* ---- camera (src/Camera.cpp) ---- */
/* Writes the Cam rows of mat4(side, up, -look, eye) with y_fov in degrees. The
 * vectors are normalised as Camera::setViewMatrix does. */
int yh_camera_look(const float eye[3], const float side[3], const float up[3],
                   const float look[3], float y_fov_deg, yc_cam* out);

/* ---- procedural scenes ---- */
typedef struct yh_scene yh_scene;
int yh_scene_new(yh_scene** out);
void yh_scene_free(yh_scene* s);
/* Appends a material, returns its index in *mat_id. */
int yh_scene_add_material(yh_scene* s, const yc_material* m, int* mat_id);
/* Unit-cube Cornell box: 5 walls (10 triangles, x,y,z in [-0.5,0.5], open at +z),
 * a quad light under the ceiling and two boxes with seeded yaw (24 triangles).
 * Materials: walls Oren-Nayar sigma^2 = on_sigma2 (white, red, green), box 0 modified
 * Phong with exponent phong_exp, box 1 Oren-Nayar white. light_emission sets the
 * quad's ke. */
int yh_scene_add_cornell(yh_scene* s, uint64_t seed, float on_sigma2, float phong_exp,
                         float light_emission, int with_boxes);
/* Icosphere subdivided `level` times (20*4^level triangles), radius r, centre c,
 * each vertex moved radially by r*U(-disp, disp) from a seeded stream; vertex
 * normals are the area-weighted face normals (the unit position when disp == 0). */
int yh_scene_add_icosphere(yh_scene* s, const float c[3], float r, int level,
                           float disp, uint64_t seed, int mat_id);
int yh_scene_add_light(yh_scene* s, const yc_quad_light* l);
/* Loads an OBJ file and its material file (named by the OBJ's first `mtllib` line, read
 * from the OBJ's directory) the way Scene::loadModel does (src/Scene.cpp:133-383,
 * :385-410): its triangles are appended with material indices offset by the materials
 * already in the scene, so loading into an empty scene gives Scene::vert_data and
 * Scene::mat_data. Quirks kept: `px` sets the py field and `py` the px field; a face
 * reads its first three vertices; an unknown `usemtl` name is material 0; without an
 * `mtllib` line the scene gets the default material (nothing is written to disk). A
 * face without normal indices gets zero normals. *n_tri_loaded (may be NULL) receives the
 * triangles added. YH_E_INVALID: a file cannot be read or has no material; YH_E_RANGE: a
 * face index outside the vertices read so far. */
int yh_scene_load_obj(yh_scene* s, const char* obj_path, int* n_tri_loaded);
int yh_scene_counts(const yh_scene* s, int* n_tri, int* n_mat, int* n_light);
int yh_scene_copy(const yh_scene* s, yc_triangle* tris, yc_material* mats, yc_quad_light* lights);

/* ---- binary scene cache ----
 * One file holds the arrays one scene hands to the core (yc_upload_scene, yc_set_lights,
 * yc_set_camera): triangles, materials, quad lights, the BVH node array with its depth,
 * an optional camera, and up to INT_MAX opaque caller bytes (render settings, say).
 * Reading it back replaces generating the scene and building its BVH (a 10M-triangle
 * scene: about 5 s on 8 cores, against 0.2 s to read its 1.8 GB). `key` is the caller's
 * identity for the contents (a hash of a generator's name and parameters, for
 * instance); a load with another key fails with YH_E_STALE, so a cache never stands in
 * for a scene it was not made from. The file is little-endian with 64-byte aligned
 * sections; a header hash and a payload hash reject truncated or corrupt files
 * (YH_E_FORMAT), and so do record sizes other than this library's. A file is written
 * under a temporary name beside `path` and renamed into place.
 *
 * yh_cache_save: depth is the value yh_bvh_depth reports (-1 when unknown); cam and meta
 * may be NULL (no camera, no caller bytes). YH_E_IO: the file cannot be written.
 * yh_cache_query: the counts, key, depth and camera flag from the header (the payload
 * is not read). YH_E_IO: the file cannot be opened.
 * yh_cache_load: reads every section into the caller's arrays, size them from
 * yh_cache_query; YH_E_RANGE when one is smaller than its section (a NULL cam counts as
 * room for none), YH_E_STALE on a key mismatch, YH_E_FORMAT when the payload does not
 * match its hash (the arrays then hold undefined contents). */
typedef struct yh_cache_info {
  uint64_t key;
  int n_tri, n_mat, n_light, n_node;
  int depth;
  int has_cam;
  int meta_bytes;
} yh_cache_info;
int yh_cache_save(const char* path, uint64_t key, const yc_triangle* tris, int n_tri, const yc_material* mats,
                  int n_mat, const yc_quad_light* lights, int n_light, const yc_bvh_node* nodes, int n_node,
                  int depth, const yc_cam* cam, const void* meta, int meta_bytes);
int yh_cache_query(const char* path, yh_cache_info* info);
int yh_cache_load(const char* path, uint64_t key, yc_triangle* tris, int cap_tri, yc_material* mats, int cap_mat,
                  yc_quad_light* lights, int cap_light, yc_bvh_node* nodes, int cap_node, yc_cam* cam, void* meta,
                  int cap_meta);

/* ---- image output (RendererCore::saveImage, src/RendererCore.cpp:608-646) ----
 * rgba: width*height float4 pixels, row y at rgba + y*width*4 (the layout of yc_tonemap
 * and yc_read_accum). As the reference writes them, the file's first row is the frame's
 * last row. yh_write_png: 8-bit RGB of the tonemapped frame, each channel
 * round(clamp(c, 0, 1) * 255) as GL converts it for glReadPixels (uncompressed deflate).
 * yh_write_hdr: Radiance RGBE of linear radiance (flat scanlines). JPEG is not written. */
int yh_write_png(const char* path, int width, int height, const float* rgba);
int yh_write_hdr(const char* path, int width, int height, const float* rgba);

#ifdef __cplusplus
}
#endif

#endif /* YUNE_HOST_H */
