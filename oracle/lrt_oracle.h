/*
 * CPU oracle for the LiteRT ray-query hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm (iMacsimus/LiteRT),
 * each function citing the reference file:line it follows.  It exists to check
 * the GPU engine (tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
 * reference arm) and is never linked into, loaded by or called from the product
 * library.  Nothing in litert_gb300/ may import it.
 *
 * Pinning: the restatement is checked bit-for-bit against the reference's own
 * translation units compiled in place (oracle/build_ref.py -> oracle/_ref/,
 * built only where the reference tree is present) on the same scenes and rays.
 * Where the reference depends on the missing LiteMath library (vector ops,
 * sign(), normalize(), matrix conventions) the conventions are restated here
 * and in the shim identically; those conventions themselves are unpinned.
 */
#ifndef LRT_ORACLE_H
#define LRT_ORACLE_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- reference data layouts (sdfScene/sdf_scene.h:127-161, BVH/cbvh.h:21-33) ---- */
typedef struct { uint32_t pos_xy, pos_z_lod_size, data_offset, pad; } orc_sbs_node;
typedef struct { uint32_t brick_size, brick_pad, bytes_per_value, aux_data; } orc_sbs_header;
typedef struct { uint32_t pos_xy, pos_z_lod_size, values[2]; } orc_svs_node;
typedef struct { float bmin[3]; uint32_t left_offset; float bmax[3]; uint32_t escape; } orc_bvh_node;
typedef struct { orc_bvh_node l, r; } orc_bvh_pair;
/* CRT_Hit as used by BVH/BVH2Common.cpp:594-601 */
typedef struct { float t; uint32_t prim_id, inst_id, geom_id; float coords[4]; } orc_hit;
/* MultiRenderPreset, render_settings.h:86-95 */
typedef struct {
  uint32_t render_mode, sdf_node_intersect, normal_mode, ray_gen_mode,
           interpolation_mode, representation_mode, spp;
} orc_preset;

enum {
  ORC_TYPE_MESH_TRIANGLE = 0, ORC_TYPE_SDF_SVS = 5, ORC_TYPE_SDF_SBS = 6,
  ORC_TYPE_SDF_SBS_COL = 11
};

/* One geometry + one instance, the state BVHRT holds for the hot path
 * (BVH/BVH2Common.h:324-481). */
typedef struct {
  uint32_t type;                    /* ORC_TYPE_* */
  /* SBS */
  orc_sbs_header sbs_hdr;
  const orc_sbs_node *sbs_nodes; uint32_t n_sbs_nodes;
  const uint32_t *sbs_values; const float *sbs_values_f;
  /* SVS */
  const orc_svs_node *svs_nodes; uint32_t n_svs_nodes;
  /* triangles, already reordered by the BVH leaves (BVH/BVH2Common_host.cpp:185-199) */
  const float *vert_pos4;           /* float4 per vertex */
  const uint32_t *tri_indices;      /* 3 per reordered triangle */
  const uint32_t *prim_indices;     /* reordered triangle -> original triangle id */
  const uint32_t *leaf_start_count; /* per BVH leaf: PackOffsetAndSize(start, count) */
  /* BVH2 fat pairs (root pair at index 0) */
  const orc_bvh_pair *pairs; uint32_t n_pairs;
  const uint32_t *tri_indices_orig; /* original index buffer (shading, Renderer/eye_ray.cpp:191-207) */
  /* single instance: TLAS leaf box (BVH/BVH2Common_host.cpp:1450-1487) and matrices */
  float inst_bmin[3], inst_bmax[3];
  float inst_inv[16], inst_inv_t[16];
  orc_preset preset;
  int closest_hit;                  /* 0: reference first-hit early-out; 1: true closest hit */
  uint32_t seed;                    /* MultiRenderer::m_seed (RAY_GEN_MODE_RANDOM) */
} orc_scene;

/* rand3 / rand2 of MultiRenderer, Renderer/eye_ray.cpp:53-80 */
void orc_rand2(uint32_t x, uint32_t y, uint32_t iter, uint32_t seed, float *rx, float *ry);

typedef struct { uint64_t n_fat, n_leaf, n_vox, n_vox_loaded, n_finder, n_tri; } orc_counters;

/* Step bound of a voxel walk over a brick segment of t-length `extent` (the
 * reference's loops have none; this covers every walk they finish).  The
 * engine's walk_step_bound computes the same number. */
static inline uint32_t orc_walk_step_bound(uint32_t brick_size, float extent) {
  const float e = extent > 0.0f ? extent : 0.0f;
  return 8u * brick_size + 16u + (uint32_t)(e < 2.6f ? e * 1.5e6f : 3.9e6f);
}

/* ---- BVH2 (oracle's own simple median-split builder, left/right fat pairs) ---- */
/* boxes: n x 6 floats (min xyz, max xyz).  prims_in_leaf >= 1.  Returns number of
 * pairs written to *out_pairs (malloc'd; free with orc_free).  For prims_in_leaf>1
 * the leaf payload indexes *out_leaf_start_count and *out_order holds the
 * reordered primitive ids; for prims_in_leaf==1 the leaf payload is the box id
 * (BVH/cbvh.cpp:628-637). */
uint32_t orc_bvh2_build(const float *boxes, uint32_t n, uint32_t prims_in_leaf,
                        orc_bvh_pair **out_pairs, uint32_t **out_leaf_start_count,
                        uint32_t **out_order, uint32_t *out_n_leaves);
void orc_free(void *p);

/* ---- ray queries ---- */
orc_hit orc_ray_query_nearest(const orc_scene *s, const float pos_near[4], const float dir_far[4],
                              orc_counters *cnt);

/* Batch of arbitrary rays (float4 pos+tNear, float4 dir+tFar each), OpenMP. */
void orc_query_rays(const orc_scene *s, const float *pos_near, const float *dir_far, uint32_t n, orc_hit *out,
                    int threads);

/* Eye rays of the pixels pix[0..n) of a w x h view (sub-pixel offset dx, dy). */
void orc_eye_rays(uint32_t w, uint32_t h, const float proj_inv[16], const float wv_inv[16], const uint32_t *pix,
                  uint32_t n, float dx, float dy, float *pos_near, float *dir_far);

/* Eye ray (Renderer/eye_ray.cpp:146-160, render_common.h:25-55). */
void orc_eye_ray(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float dx, float dy,
                 const float proj_inv[16], const float world_view_inv[16],
                 float pos_near[4], float dir_far[4]);

/* Shading of one hit (Renderer/eye_ray.cpp:162-489, subset: MASK, LAMBERT_NO_TEX,
 * DEPTH, LINEAR_DEPTH, INVERSE_LINEAR_DEPTH, NORMAL). */
void orc_shade(const orc_scene *s, const orc_hit *hit, const float pos_near[4],
               const float dir_far[4], float out_rgba[4]);

/* Render a W x H view: one regular ray per pixel (spp=1 centre, or spp samples),
 * writes hits (row-major, may be NULL) and float colours (may be NULL).
 * threads<=0 uses all OpenMP threads.  Returns total counters. */
orc_counters orc_render(const orc_scene *s, uint32_t w, uint32_t h,
                        const float proj_inv[16], const float world_view_inv[16],
                        orc_hit *hits, float *rgba, int threads);

/* Render an explicit pixel subset (for bounded CPU baseline samples). */
orc_counters orc_render_pixels(const orc_scene *s, uint32_t w, uint32_t h,
                               const float proj_inv[16], const float world_view_inv[16],
                               const uint32_t *pix, uint32_t n_pix, orc_hit *hits, int threads);

/* ---- SDF scenes and SBS/SVS construction (utils/sparse_octree_builder.cpp) ---- */
/* Primitive set: smooth union (polynomial smin, parameter k; k<=0 -> plain min)
 * of spheres {cx,cy,cz,r} and rounded boxes {cx,cy,cz, hx,hy,hz, round, R[9] row-major
 * world->local rotation}. */
typedef struct {
  uint32_t n_spheres; const float *spheres;   /* 4 floats each */
  uint32_t n_boxes;   const float *boxes;     /* 16 floats each */
  float k;
} orc_sdf;

float orc_sdf_eval(const orc_sdf *f, float x, float y, float z);

/* create_sdf_SBS (utils/sdf_converter.cpp:162-181).  Writes malloc'd nodes/values;
 * brick order is canonical (depth-first octree order).  Returns brick count. */
uint32_t orc_build_sbs(const orc_sdf *f, uint32_t depth, orc_sbs_header hdr,
                       orc_sbs_node **out_nodes, uint32_t **out_values, uint32_t *out_n_values);
/* create_sdf_SVS (utils/sdf_converter.cpp:118-134). */
uint32_t orc_build_svs(const orc_sdf *f, uint32_t depth, orc_svs_node **out_nodes);

/* ---- small matrix helpers (LiteMath conventions, restated) ---- */
void orc_perspective(float fov_deg, float aspect, float znear, float zfar, float out[16]);
void orc_look_at(const float eye[3], const float center[3], const float up[3], float out[16]);
void orc_inverse4x4(const float m[16], float out[16]);

#ifdef __cplusplus
}
#endif
#endif
