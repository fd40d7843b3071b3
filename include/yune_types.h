/* yune_types.h -- buffer layouts shared by the host producers and the CUDA core.
 *
 * Every struct here is byte-for-byte the layout Yune's host already produces, so a
 * caller hands over its own std::vector data without conversion:
 *   yc_float4    <- cl_float4 (16 B, 16-byte aligned)
 *   yc_cam       <- Cam         include/CL_headers.h:57-65   (80 B)
 *   yc_triangle  <- TriangleGPU include/CL_headers.h:67-77   (112 B)
 *   yc_aabb      <- AABB        include/CL_headers.h:79-84   (32 B)
 *   yc_bvh_node  <- BVHNodeGPU  include/CL_headers.h:86-92   (80 B)
 *   yc_material  <- Material    include/CL_headers.h:94-107  (80 B)
 *   yc_quad_light <- the kernel-side Quad of kernels/legacy/udpt.cl:34-45, padded
 *                   to 128 B. The reference compiles its lights into the kernel as a
 *                   __constant array (udpt.cl:97-106); here they are a per-scene
 *                   buffer.
 * Points carry w = 1 and directions w = 0, as src/Scene.cpp:328-344 writes them.
 */
#ifndef YUNE_TYPES_H
#define YUNE_TYPES_H

#include <stdint.h>

#if defined(__cplusplus)
#define YC_ALIGN16 alignas(16)
#else
#define YC_ALIGN16 _Alignas(16)
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct yc_float4 { YC_ALIGN16 float x; float y, z, w; } yc_float4;

typedef struct yc_cam {
  yc_float4 r1, r2, r3, r4;    /* rows of the view-to-world matrix */
  float view_plane_dist;       /* 1/tan(yFOV*3.14/360), src/Camera.cpp:62 */
  float pad[3];
} yc_cam;

typedef struct yc_triangle {
  yc_float4 v1, v2, v3;        /* positions, w = 1 */
  yc_float4 vn1, vn2, vn3;     /* vertex normals, w = 0 */
  int32_t matID;
  float pad[3];
} yc_triangle;

typedef struct yc_aabb { yc_float4 p_min, p_max; } yc_aabb;

typedef struct yc_bvh_node {
  yc_aabb aabb;
  int32_t vert_list[10];       /* triangle indices of a leaf */
  int32_t child_idx;           /* first of two contiguous children; -1 leaf; -2 empty */
  int32_t vert_len;            /* triangles in a leaf; -1 interior or empty */
} yc_bvh_node;

typedef struct yc_material {
  yc_float4 ke, kd, ks;
  float n, k, px, py, alpha_x, alpha_y;
  int32_t is_specular, is_transmissive;
} yc_material;

typedef struct yc_quad_light {
  yc_float4 pos, normal, ke, kd, ks, edge_l, edge_w;
  float phong_exponent;
  float pad[3];
} yc_quad_light;

#ifdef __cplusplus
}  /* extern "C" */
static_assert(sizeof(yc_float4) == 16, "cl_float4");
static_assert(sizeof(yc_cam) == 80, "Cam is 80 B");
static_assert(sizeof(yc_triangle) == 112, "TriangleGPU is 112 B");
static_assert(sizeof(yc_aabb) == 32, "AABB is 32 B");
static_assert(sizeof(yc_bvh_node) == 80, "BVHNodeGPU is 80 B");
static_assert(sizeof(yc_material) == 80, "Material is 80 B");
static_assert(sizeof(yc_quad_light) == 128, "Quad padded to 128 B");
#endif

#endif /* YUNE_TYPES_H */
