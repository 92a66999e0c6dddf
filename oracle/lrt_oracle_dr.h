/*
 * CPU oracle for the differentiable SDF render (MultiRendererDR) — TEST
 * INFRASTRUCTURE ONLY.  Plain-C restatement of diff_render/BVH2DR.cpp (the
 * per-ray gradient core, pinned bit-for-bit against that file compiled in
 * place, oracle/build_ref.py) and of the pixel-level glue of
 * diff_render/MultiRendererDR.cpp (RenderDR, CastRayWithGrad, border pixels,
 * CastBorderRay, getBaseGradientMult, OptimizeStepAdam) and
 * diff_render/DR_common.cpp:47-146 (create_grid_sbs) with
 * utils/sparse_octree_builder.cpp:2761-2850 (neighbour table).  The glue cannot
 * be compiled in place (it needs the absent LiteImage/LiteScene/Hydra
 * libraries), so it is restated line by line and pinned through the core.
 * Only tests/ and bench.py's CPU legs load this library.
 */
#ifndef LRT_ORACLE_DR_H
#define LRT_ORACLE_DR_H
#include "lrt_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  ORC_DR_RAY_FLAG_DDIFFUSE_DCOLOR = 1u << 0, ORC_DR_RAY_FLAG_DDIFFUSE_DPOS = 1u << 1,
  ORC_DR_RAY_FLAG_DNORM_DPOS = 1u << 2, ORC_DR_RAY_FLAG_BORDER = 1u << 3, ORC_DR_RAY_FLAG_DDIST_DPOS = 1u << 4
};
enum { ORC_DR_RENDER_DIFFUSE = 0, ORC_DR_RENDER_LAMBERT = 1, ORC_DR_RENDER_MASK = 2,
       ORC_DR_RENDER_LINEAR_DEPTH = 3, ORC_DR_RENDER_NORMAL = 4 };
enum { ORC_DR_RECON_COLOR = 1, ORC_DR_RECON_GEOMETRY = 2 };
#define ORC_SBS_LAYOUT_ID32F_IRGB32F (4u << 24)
#define ORC_SBS_LAYOUT_ID32F_IRGB32F_IN (5u << 24)
#define ORC_INVALID_IDX (1u << 31)      /* sdfScene/sdf_scene.h:42 */
#define ORC_DR_STACK 80                 /* STACK_SIZE, raytrace_common.h:36 */

/* An indexed SBS with its BVH2 (BVHDR state for one geometry, one instance). */
typedef struct {
  orc_sbs_header hdr;
  const orc_sbs_node *nodes; uint32_t n_nodes;
  const uint32_t *values; uint32_t n_values;
  uint32_t n_params;
  const orc_bvh_pair *pairs; uint32_t n_pairs;
  float inst_bmin[3], inst_bmax[3];
  float inst_inv[16];
  int need_normal;                      /* BVHRT::need_normal() of the DR render mode */
} orc_dr_scene;

/* Light, Renderer/eye_ray.h:48-74: type 0 direct (dir normalised), 2 ambient. */
typedef struct { uint32_t type; float dir[3]; float color[3]; } orc_dr_light;

/* The MultiRendererDRPreset fields on the path (diff_render/DR_common.h:134-196). */
typedef struct {
  uint32_t render_mode, reconstruction_flags, input_type, loss_function;
  uint32_t spp, border_spp;
  float border_relax_eps;
  uint32_t seed;                        /* MultiRenderer::m_seed */
  uint32_t n_lights;
  orc_dr_light lights[4];
  float lr, beta1, beta2, eps;          /* Adam */
  uint32_t accumulate_batch;            /* 0: the reference's per-image zeroing; 1: sum over the batch */
  uint32_t reg_function;                /* DR_REG_FUNCTION_NONE = 0, else Regularization runs */
  float reg_lambda, reg_power;
  uint32_t redistancing_enable, redistancing_interval;
  uint32_t border_sampling;             /* DR_BORDER_SAMPLING_RANDOM 0 / _SVM 1 (DR_common.h:123-124) */
  uint32_t raycasting_mask;             /* DR_RAYCASTING_MASK_OFF 0 / _ON 1 (DR_common.h:86-87) */
} orc_dr_preset;

typedef struct {
  uint32_t width, height;
  float proj_inv[16], wv_inv[16];
  float proj[16], world_view[16];
  uint8_t *cast_mask;                   /* W x H ray-casting mask of the view (masks[image]), read and
                                           rewritten by a render when raycasting_mask is on; may be NULL */
} orc_dr_view;

/* One RayQuery_NearestHitWithGrad per ray; 576-word records (oracle/ref_driver.cpp layout). */
void orc_dr_query(const orc_dr_scene *s, const float *params, uint32_t flags, const float *pos_near,
                  const float *dir_far, uint32_t n, uint32_t *out);

/* RenderDR for one view (diff_render/MultiRendererDR.cpp:578-750).  image_ref and
 * out_image are float4 W x H, out_depth float W x H (.w of out_image_depth).
 * Writes grad (n_params, already scaled by getBaseGradientMult and summed over
 * the per-thread slices in thread order) and border_mask (W x H bytes, may be
 * NULL).  threads <= 0 uses all OpenMP threads.  Returns the loss (mean over pixels). */
double orc_dr_render(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, const orc_dr_view *v,
                     const float *image_ref, float *out_image, float *out_depth, float *grad,
                     uint8_t *border_mask, int threads);

/* The interior loss of one view in double precision (forward only, no
 * derivatives), for central finite differences.  hit_count (W x H, may be NULL)
 * receives the per-pixel hit counts. */
double orc_dr_loss_f64(const orc_dr_scene *s, const double *params, const orc_dr_preset *p,
                       const orc_dr_view *v, const float *image_ref, uint8_t *hit_count);

/* One OptimizeFixedStructure iteration over images 0..n-1 in order (:390-486):
 * render each (per-image zeroing unless accumulate_batch), divide by n, Adam.
 * adam_state holds V then S (2*n_params). losses (n) and grad_out (n_params) may be NULL. */
void orc_dr_step(const orc_dr_scene *s, float *params, const orc_dr_preset *p, const orc_dr_view *views,
                 const float *images, uint32_t n_images, uint32_t iter, float *adam_state, float *grad_out,
                 double *losses, float *images_out, int threads);

/* SVM_fit (diff_render/MultiRendererDR.cpp:1518-1546) on n rows (x, y, 1) * label
 * (3 floats per row, scaled in place by etha as the reference does): W = (a, b, c,
 * error rate) of the line a x + b y + c = 0. */
void orc_dr_svm_fit(float *rows, uint32_t n, float W[4]);
/* CohenSutherlandLineClip (:1580-1649) against [0,1]^2; returns 1 when accepted. */
int orc_dr_line_clip(float *x0, float *y0, float *x1, float *y1);
/* The SVM stage of CastBorderRaySVM (:1651-1816) for pixel (x, y) of a view:
 * count border samples (0: the pixel is skipped) on the stripe p0 + u r + v radius n
 * (force: uniformly over the pixel), each weighted by pdf; svm_spp rays were spent. */
typedef struct {
  uint32_t count, force, svm_spp, pad;
  float p0[2], r[2], n[2], radius, pdf;
} orc_dr_svm_line_t;
void orc_dr_svm_line(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, const orc_dr_view *v,
                     uint32_t x, uint32_t y, orc_dr_svm_line_t *L);
/* Sub-pixel position of border sample j of a line (sample index svm_spp + j). */
void orc_dr_svm_sample(const orc_dr_svm_line_t *L, uint32_t x, uint32_t y, uint32_t seed, uint32_t j, float d[2]);

/* Regularization (diff_render/MultiRendererDR.cpp:1933-2055): for every brick
 * value and each of its 6 neighbours inside the brick (brick_size + 1 values per
 * axis), adds reg_lambda * reg_power * sign(d) * |d|^(reg_power - 1) to grad at the
 * value's parameter index, d = own value - neighbour value. */
void orc_dr_regularize(const orc_dr_scene *s, const float *params, const orc_dr_preset *p, float *grad);

/* Redistance (:2122-2330) with SolveEikonal (:2058-2120): n_iters Jacobi updates of
 * the dense n^3 distance grid dist (in place), grid spacing h; nodes next to a sign
 * change or on the surface keep their values. */
void orc_dr_redistance(float *dist, uint32_t n, float h, uint32_t n_iters);

/* OptimizeStepAdam (:828-853). */
void orc_dr_adam(uint32_t iter, const float *g, float *x, float *state, uint32_t n, float lr, float b1, float b2,
                 float eps);

/* create_grid_sbs (diff_render/DR_common.cpp:47-146) + SBS_ind_to_SBS_ind_with_neighbors
 * (utils/sparse_octree_builder.cpp:2761-2850).  Distances from the primitive set f,
 * colours either constant (color3) or, when color3 is NULL, the position colour
 * 0.5 + 0.5 p.  Returns node count; arrays malloc'd (orc_free). */
uint32_t orc_dr_grid_sbs(uint32_t brick_count, uint32_t brick_size, const orc_sdf *f, const float *color3,
                         orc_sbs_header *hdr, orc_sbs_node **nodes, uint32_t **values, uint32_t *n_values,
                         float **params, uint32_t *n_params);

/* The parameters (values_f) of create_grid_sbs(gs, bs, ...) as OptimizeGrid builds
 * them (diff_render/MultiRendererDR.cpp:228-276): gradient_color colours; distances
 * circle_sdf((0,-0.15,0), 0.7) for old_params NULL, else grid_sampler over the dense
 * distances of old_params (gs bricks of old_bs).  out: (gs bs + 1)^3 + 3 (gs + 1)^3 floats. */
void orc_dr_grid_resample(uint32_t gs, uint32_t bs, const float *old_params, uint32_t old_bs, float *out);

#ifdef __cplusplus
}
#endif
#endif
