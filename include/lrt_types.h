/*
 * Plain-old-data types crossing the lrt C ABI.  Each mirrors, field for field,
 * the reference struct it replaces so that a caller holding the reference's
 * views can pass them straight through:
 *
 *   lrt_sbs_node    <- SdfSBSNode        (sdfScene/sdf_scene.h:136-142)
 *   lrt_sbs_header  <- SdfSBSHeader      (sdfScene/sdf_scene.h:155-161)
 *   lrt_svs_node    <- SdfSVSNode        (sdfScene/sdf_scene.h:127-132)
 *   lrt_preset      <- MultiRenderPreset (render_settings.h:86-95)
 *   lrt_hit         <- CRT_Hit           (CrossRT; fields as used in BVH/BVH2Common.cpp:594-601)
 *   lrt_bvh_node    <- BVHNode           (BVH/cbvh.h:21-27), lrt_bvh_pair <- BVHNodePair (:29-33)
 */
#ifndef LRT_TYPES_H
#define LRT_TYPES_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { uint32_t pos_xy, pos_z_lod_size, data_offset, _pad; } lrt_sbs_node;
typedef struct { uint32_t brick_size, brick_pad, bytes_per_value, aux_data; } lrt_sbs_header;
typedef struct { uint32_t pos_xy, pos_z_lod_size, values[2]; } lrt_svs_node;

typedef struct {
  uint32_t render_mode;         /* MULTI_RENDER_MODE_*   */
  uint32_t sdf_node_intersect;  /* SDF_OCTREE_NODE_INTERSECT_* */
  uint32_t normal_mode;         /* NORMAL_MODE_*         */
  uint32_t ray_gen_mode;        /* RAY_GEN_MODE_*        */
  uint32_t interpolation_mode;  /* INTERPOLATION_MODE_*  */
  uint32_t representation_mode; /* REPRESENTATION_MODE_* */
  uint32_t spp;                 /* samples per pixel     */
} lrt_preset;

typedef struct {
  float t;
  uint32_t primId, instId, geomId;   /* geomId = geometry | (type << 24); miss: primId == 0xFFFFFFFF */
  float coords[4];                   /* [0..1] barycentrics or packed colour, [2..3] octahedral normal */
} lrt_hit;

/* Compact per-pixel record written by the batched renderer: t, primId and the
 * octahedral normal (coords[2..3]).  16 bytes, one per ray. */
typedef struct { float t; uint32_t primId; float nx, ny; } lrt_hit16;

typedef struct { float boxMin[3]; uint32_t leftOffset; float boxMax[3]; uint32_t escapeIndex; } lrt_bvh_node;
typedef struct { lrt_bvh_node left, right; } lrt_bvh_pair;

/* One camera view of a batched render: image size and the two matrices the
 * reference's MultiRenderer::Render takes (Renderer/eye_ray_host.cpp:563-573).
 * Matrices are row-major float[16]. */
typedef struct {
  uint32_t width, height;
  float world_view[16];
  float proj[16];
} lrt_view;

/* Analytic SDF used to build sparse brick / voxel sets: a smooth union
 * (polynomial smooth minimum with parameter k, k <= 0 -> min) of spheres
 * {cx,cy,cz,r} and rounded boxes {cx,cy,cz, hx,hy,hz, rounding, R[9]} where R is
 * the row-major world->local rotation. */
typedef struct {
  uint32_t n_spheres; const float *spheres;
  uint32_t n_boxes;   const float *boxes;
  float k;
} lrt_sdf_desc;

/* reference enums used by the hot path (render_settings.h) */
enum {
  LRT_TYPE_MESH_TRIANGLE = 0, LRT_TYPE_SDF_SVS = 5, LRT_TYPE_SDF_SBS = 6,
  LRT_TYPE_SDF_SBS_TEX = 10, LRT_TYPE_SDF_SBS_COL = 11
};
enum {
  LRT_RENDER_MODE_MASK = 0, LRT_RENDER_MODE_LAMBERT_NO_TEX = 1, LRT_RENDER_MODE_DEPTH = 2,
  LRT_RENDER_MODE_LINEAR_DEPTH = 3, LRT_RENDER_MODE_INVERSE_LINEAR_DEPTH = 4,
  LRT_RENDER_MODE_PRIMITIVE = 5, LRT_RENDER_MODE_TYPE = 6, LRT_RENDER_MODE_GEOM = 7,
  LRT_RENDER_MODE_NORMAL = 8, LRT_RENDER_MODE_BARYCENTRIC = 9, LRT_RENDER_MODE_ST_ITERATIONS = 10,
  LRT_RENDER_MODE_PHONG_NO_TEX = 12, LRT_RENDER_MODE_DIFFUSE = 16, LRT_RENDER_MODE_LAMBERT = 17,
  LRT_RENDER_MODE_PHONG = 18, LRT_RENDER_MODE_HSV_DEPTH = 19
};
enum {
  LRT_INTERSECT_ST = 0, LRT_INTERSECT_ANALYTIC = 1, LRT_INTERSECT_NEWTON = 2,
  LRT_INTERSECT_BBOX = 3, LRT_INTERSECT_IT = 4
};
enum {
  LRT_SBS_LAYOUT_UNDEFINED = 0u << 24, LRT_SBS_LAYOUT_DX = 1u << 24, LRT_SBS_LAYOUT_DX_UV16 = 2u << 24,
  LRT_SBS_LAYOUT_DX_RGB8 = 3u << 24, LRT_SBS_LAYOUT_ID32F_IRGB32F = 4u << 24,
  LRT_SBS_LAYOUT_ID32F_IRGB32F_IN = 5u << 24
};

#ifdef __cplusplus
}
#endif
#endif
