/*
 * lrt — differentiable SDF render (MultiRendererDR), C ABI.
 *
 * Replaces dr::MultiRendererDR (diff_render/MultiRendererDR.h:71-155) for
 * indexed sparse-brick sets (SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F and _IN): the
 * parameters are the SBS's float array (values_f: distances, then RGB colours)
 * and every call works on the context's device.  Conventions as lrt_gpu.h:
 * plain pointers and sizes, an lrt_status per call, lrt_last_error(ctx) for a
 * message.  The gradient, images and parameters stay in device memory between
 * calls; lrt_dr_get copies them out.
 */
#ifndef LRT_DR_H
#define LRT_DR_H
#include "lrt_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* DR_RENDER_MODE_*, diff_render/DR_common.h:83-88 */
enum { LRT_DR_RENDER_DIFFUSE = 0, LRT_DR_RENDER_LAMBERT = 1, LRT_DR_RENDER_MASK = 2,
       LRT_DR_RENDER_LINEAR_DEPTH = 3, LRT_DR_RENDER_NORMAL = 4 };
/* DR_RECONSTRUCTION_FLAG_*, diff_render/DR_common.h:112-113 */
enum { LRT_DR_RECON_COLOR = 1, LRT_DR_RECON_GEOMETRY = 2 };
/* light types, Renderer/eye_ray.h:44-46 (point lights are not supported by the reference DR) */
enum { LRT_DR_LIGHT_DIRECT = 0, LRT_DR_LIGHT_AMBIENT = 2 };

/* Light (create_direct_light / create_ambient_light, Renderer/eye_ray.h:60-74):
 * dir is used as given (the reference normalises it on creation). */
typedef struct { uint32_t type; float dir[3]; float color[3]; } lrt_dr_light;

/* The MultiRendererDRPreset fields this path reads (diff_render/DR_common.h:134-196),
 * the renderer's seed and lights, and the Adam settings.  The finder is NEWTON,
 * ray generation RANDOM and normals SDF_SMOOTHED, as OptimizeFixedStructure
 * forces (diff_render/MultiRendererDR.cpp:324-326). */
typedef struct {
  uint32_t render_mode;          /* LRT_DR_RENDER_* */
  uint32_t reconstruction_flags; /* LRT_DR_RECON_* */
  uint32_t input_type;           /* 0 colour images, 1 linear depth */
  uint32_t loss_function;        /* 0 MSE, 1 MAE */
  uint32_t spp;                  /* 1..64 */
  uint32_t border_spp;           /* rays per border pixel (0 = no border integral) */
  float border_relax_eps;
  uint32_t seed;                 /* MultiRenderer::setSeed */
  uint32_t n_lights;             /* 0..4 */
  lrt_dr_light lights[4];
  float opt_lr, opt_beta_1, opt_beta_2, opt_eps;
  /* 0: the reference's batch behaviour (its per-thread gradient buffer is
   * refilled for every image of a batch, so only the last image's gradient
   * reaches Adam, divided by the batch size); 1: the batch's gradients are summed */
  uint32_t accumulate_batch;
  /* 1: warp-aggregated gradient atomics (default), 0: one atomic per contribution */
  uint32_t warp_aggregate;
  /* Regularization (diff_render/MultiRendererDR.cpp:1933-2055): reg_function != 0
   * adds reg_lambda * reg_power * sign(d) * |d|^(reg_power-1) per brick value and
   * in-brick neighbour to the batch gradient (defaults 0, 0.25, 2) */
  uint32_t reg_function;
  float reg_lambda, reg_power;
  /* Redistance (:2122-2330) of the dense distance grid every redistancing_interval
   * iterations when enabled (defaults off, 1); needs a cubic create_grid_sbs set */
  uint32_t redistancing_enable, redistancing_interval;
  /* dr_border_sampling (DR_common.h:123-124): 0 random (CastBorderRay), 1 SVM
   * (CastBorderRaySVM, :1651-1931: a quarter of border_spp classifies the pixel's
   * sub-samples by depth, a linear SVM fits the silhouette line and the rest
   * sample a stripe around it; border_spp <= 1024).  The reference draws the
   * stripe points from the process-wide rand(); here they come from the same
   * per-sample hash as the other samples, so results are reproducible. */
  uint32_t border_sampling;
  /* dr_raycasting_mask (DR_common.h:86-87): 1 casts a view's interior rays only
   * where its previous render hit (:1097-1100, :443-448); the masks start full
   * at lrt_dr_set_reference, lrt_dr_set_scene and lrt_dr_set_preset. */
  uint32_t raycasting_mask;
} lrt_dr_preset;

/* getDefaultPresetDR (diff_render/MultiRendererDR.h:12-66) with the colour+geometry
 * Lambert reconstruction and MultiRenderer's default lights (Renderer/eye_ray_host.cpp:40). */
void lrt_dr_default_preset(lrt_dr_preset *p);

/* MultiRendererDR::SetScene for OptimizeFixedStructure (diff_render/MultiRendererDR.cpp:353-355):
 * the indexed SBS (copied to the device) and its BVH2, built by the project's
 * builder unless `pairs` is given (n_pairs fat pairs, root at 0). */
lrt_status lrt_dr_set_scene(lrt_ctx *ctx, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes, uint32_t n_nodes,
                            const uint32_t *values, uint64_t n_values, const float *params, uint32_t n_params,
                            const lrt_bvh_pair *pairs, uint32_t n_pairs);
/* The BVH2 in use (host copy owned by ctx). */
lrt_status lrt_dr_get_bvh2(lrt_ctx *ctx, const lrt_bvh_pair **pairs, uint32_t *n_pairs);

/* MultiRendererDR::SetReference (diff_render/MultiRendererDR.cpp:147-160): target
 * images (float RGBA, row-major, view after view) and their cameras.  Resets the
 * optimiser state. */
lrt_status lrt_dr_set_reference(lrt_ctx *ctx, uint32_t n_views, const lrt_view *views, const float *images);

lrt_status lrt_dr_set_preset(lrt_ctx *ctx, const lrt_dr_preset *preset);

/* Replaces the parameters (values_f) and resets the optimiser state. */
lrt_status lrt_dr_set_params(lrt_ctx *ctx, const float *params, uint32_t n_params);

/* MultiRendererDR::RenderDR for one view (diff_render/MultiRendererDR.cpp:578-750):
 * renders it, computes dLoss/dparams (interior + border integral, scaled by
 * getBaseGradientMult) into the gradient buffer (overwritten) and returns the
 * mean pixel loss.  Asynchronous on the context's stream except for *loss. */
lrt_status lrt_dr_render_grad(lrt_ctx *ctx, uint32_t view, double *loss);

/* One iteration of OptimizeFixedStructure (diff_render/MultiRendererDR.cpp:390-486):
 * every view renders with gradients (batch = all views, in order), the batch
 * gradient is divided by the batch size and OptimizeStepAdam updates the
 * parameters.  losses (n_views) may be NULL; when given the call waits for them. */
lrt_status lrt_dr_step(lrt_ctx *ctx, uint32_t iter, double *losses);

/* OptimizeFixedStructure: `iterations` steps from iteration `first_iter` (Adam's
 * bias correction uses the iteration number); the parameters stay on the device. */
lrt_status lrt_dr_optimize(lrt_ctx *ctx, uint32_t first_iter, uint32_t iterations, double *last_losses);

/* Copies out device state.  what: LRT_DR_PARAMS (n_params floats),
 * LRT_DR_GRAD (n_params floats, the last gradient before Adam's batch division),
 * LRT_DR_IMAGE (view's W*H float4 = getLastImage), LRT_DR_DEPTH (W*H floats,
 * depth-discontinuity thresholds), LRT_DR_BORDER (W*H bytes, border-pixel mask),
 * LRT_DR_ADAM (2*n_params floats: first then second moments).  bytes must match. */
enum { LRT_DR_PARAMS = 0, LRT_DR_GRAD = 1, LRT_DR_IMAGE = 2, LRT_DR_DEPTH = 3, LRT_DR_BORDER = 4, LRT_DR_ADAM = 5,
       LRT_DR_CAST_MASK = 6 /* view's W*H bytes of ray-casting mask (raycasting_mask on) */ };
lrt_status lrt_dr_get(lrt_ctx *ctx, uint32_t what, uint32_t view, void *out, uint64_t bytes);

/* dr::BVHDR::RayQuery_NearestHitWithGrad (diff_render/BVH2DR.cpp:12-102) on n rays
 * (float4 pos+tNear, float4 dir+tFar, host memory) with DR_RAY_FLAG_* bits
 * (1 dDiffuse/dColour, 2 dDiffuse/dPos, 4 dNorm/dPos, 8 border, 16 dDist/dPos)
 * and the render mode of the current preset.  Bit 32 (no reference counterpart)
 * runs the border integral's walk instead of the border walk: voxels whose
 * corner values all exceed the preset's border_relax_eps are skipped from the
 * start, and a ray is walked again in full where that could change its record;
 * for every ray whose relaxation SDF ends below border_relax_eps the record is
 * the border walk's, bit for bit (the others contribute nothing to the border
 * integral; their relaxation fields may differ).  Writes 32 words per ray: hit t,
 * primId, colour[3], normal[3]; the border relaxation point missed_hit t, sdf,
 * colour[3], normal[3]; missed_indices[8]; missed_dSDF_dtheta[8]. */
lrt_status lrt_dr_query_rays(lrt_ctx *ctx, uint32_t flags, const float *pos_near, const float *dir_far, uint32_t n,
                             uint32_t *out);

/* Number of kernel launches of the last lrt_dr_render_grad / lrt_dr_step call. */
uint32_t lrt_dr_last_launch_count(const lrt_ctx *ctx);

/* create_grid_sbs (diff_render/DR_common.cpp:47-146) followed by
 * SBS_ind_to_SBS_ind_with_neighbors (utils/sparse_octree_builder.cpp:2761-2850):
 * a dense brick_count^3 grid of brick_size^3 bricks over [-1,1]^3 in the
 * ID32F_IRGB32F_IN layout, distances from `sdf`, colours constant (color3) or,
 * with color3 NULL, 0.5 + 0.5 p.  Host only; arrays malloc'd, free with lrt_free. */
lrt_status lrt_dr_grid_sbs(uint32_t brick_count, uint32_t brick_size, const lrt_sdf_desc *sdf, const float *color3,
                           lrt_sbs_header *hdr, lrt_sbs_node **nodes, uint32_t *n_nodes, uint32_t **values,
                           uint64_t *n_values, float **params, uint32_t *n_params);

/* create_grid_sbs as MultiRendererDR::OptimizeGrid calls it (diff_render/
 * MultiRendererDR.cpp:228-276): brick_count^3 bricks of brick_size, colours
 * gradient_color (diff_render/DR_common.cpp:25-35); distances circle_sdf((0,-0.15,0),
 * 0.7) when old_params is NULL (the starting grid), else grid_sampler (:242-262):
 * trilinear in the dense distances of old_params, a grid of the same brick count
 * with bricks of old_brick_size.  Layout ID32F_IRGB32F_IN; host only; arrays
 * malloc'd, free with lrt_free. */
lrt_status lrt_dr_grid_resample(uint32_t brick_count, uint32_t brick_size, const float *old_params,
                                uint32_t old_brick_size, lrt_sbs_header *hdr, lrt_sbs_node **nodes, uint32_t *n_nodes,
                                uint32_t **values, uint64_t *n_values, float **params, uint32_t *n_params);
/* PreprocessRefImages (diff_render/MultiRendererDR.cpp:169-226) on the host: each
 * view's image resampled to width x height, ceil(W/width) x ceil(H/height)
 * bilinear samples a pixel, alpha from the mask "colour differs from black"
 * (CreateRefImageMasks).  Bilinear: texel centres at (i + 0.5)/size, clamped at
 * the edges (the reference's image-library sampler is not in its tree).
 * out_views: the views with the new size; out_images: n_views x width x height float4. */
lrt_status lrt_dr_preprocess_reference(uint32_t n_views, const lrt_view *views, const float *images, uint32_t width,
                                       uint32_t height, lrt_view *out_views, float *out_images);
/* MultiRendererDR::OptimizeGrid (:228-276) on the reference images given to
 * lrt_dr_set_reference: from the starting grid (start_grid_size bricks of size 1)
 * each stage i renders the reference resampled to render_sizes[2i] x
 * render_sizes[2i+1] (0 x 0 or render_sizes NULL: as given; the preset's
 * render_width/height), sets the grid as the scene (BVH from the builder
 * lrt_set_tuning "bvh_builder" selects), applies presets[i] and runs iterations[i]
 * optimisation steps (the preset's opt_iterations), then resamples the optimised
 * distances into bricks twice as large (the same size after the last stage when
 * no_last_step_resize).  Returns the final grid (malloc'd, free with lrt_free) and
 * the last step's per-view losses (n_views, may be NULL). */
lrt_status lrt_dr_optimize_grid(lrt_ctx *ctx, uint32_t start_grid_size, uint32_t no_last_step_resize,
                                const lrt_dr_preset *presets, const uint32_t *iterations,
                                const uint32_t *render_sizes, uint32_t n_stages, lrt_sbs_header *hdr,
                                lrt_sbs_node **nodes, uint32_t *n_nodes, uint32_t **values, uint64_t *n_values,
                                float **params, uint32_t *n_params, double *last_losses);
#ifdef __cplusplus
}
#endif
#endif
