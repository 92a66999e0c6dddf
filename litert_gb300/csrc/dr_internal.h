// Device-side state of the differentiable SDF render (MultiRendererDR path):
// shared between the CUDA kernels (dr.cu) and the host driver (dr_api.cpp).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace lrt {
namespace drk {

constexpr uint32_t kInvalidIdx = 1u << 31;   // empty neighbour slot, sdfScene/sdf_scene.h:42
constexpr uint32_t kNoIndex = 0xFFFFFFFFu;   // unset PD index, diff_render/DR_common.h:24
constexpr int kStack = 80;                   // STACK_SIZE, raytrace_common.h:36
constexpr uint32_t kMaxSpp = 64;             // samples per pixel kept for the depth threshold

// status bits written by the kernels (read back by the host after a step)
constexpr uint32_t kStatusStackOverflow = 1u;
constexpr uint32_t kStatusTraversalBound = 2u;   // more node visits than the BVH has pairs (a cycle)

// Indexed SBS (ID32F_IRGB32F or _IN) with its BVH2, one identity-or-given instance.
struct DevScene {
  const uint4 *nodes;        // SdfSBSNode: pos_xy, pos_z_lod_size, data_offset, unused
  const uint32_t *values;    // per node: v^3 distance indices, 8 colour indices, [27 neighbours]
  const float *P;            // parameters (values_f): distances then RGB colours
  float *grad;               // dLoss/dP
  const float4 *pairs;       // BVH2 fat pairs: 4 float4 each (left min|offset, left max|escape, right ...)
  uint32_t n_pairs;
  const float2 *brick_bounds; // per brick: min distance value, max |distance value|
  const float *bvals;         // per brick: its v^3 distance values gathered from P
  const float2 *vbounds;      // per voxel (brick-major, x-major in the brick): min and max |.| of its 8 corners
  uint32_t brick_size, v_size, layout_in, need_normal;
  float inst_bmin[3], inst_bmax[3];
  float inst_inv[12];        // rows 0..2 of the instance's inverse transform
  uint32_t *status;
};

struct DevPreset {
  uint32_t render_mode, recon, input_type, loss_fn;
  uint32_t spp, border_spp, seed, n_lights;
  float relax_eps, g_mult;
  uint32_t light_type[4];
  float light_dir[4][3], light_col[4][3];
  uint32_t agg;              // 1: warp-aggregated gradient atomics, 0: one atomic per contribution
  uint32_t flags;            // DR_RAY_FLAG_* of CastRayWithGrad for this preset
  uint32_t svm;              // border sampling: 0 random (CastBorderRay), 1 SVM (CastBorderRaySVM)
  uint32_t svm_spp, svm_sqrt;   // the SVM stage's ray count (a square) and its side
};

// Sampling line of one border pixel from the SVM stage of CastBorderRaySVM
// (diff_render/MultiRendererDR.cpp:1651-1816): count border samples (0: none)
// at p0 + u r + v radius n (force: anywhere in the pixel), each weighted by pdf.
struct SvmLine {
  uint32_t count, force, pad0, pad1;
  float p0x, p0y, rx, ry, nx, ny, radius, pdf;
};
constexpr uint32_t kMaxSvm = 256;   // SVM-stage rays per border pixel (border_spp <= 1024)

struct DevView {
  uint32_t width, height;
  float proj_inv[16], wv_inv[16], pv[16];
  const float4 *ref;         // target image
  float4 *img;               // rendered image (rgb, hit fraction)
  float *depth;              // depth-discontinuity threshold (out_image_depth .w)
  uint8_t *border_mask;
  uint32_t *border_list;
  uint32_t *border_count;
  double *loss;              // sum of pixel losses
  uint8_t *cast_mask;        // ray-casting mask (masks[image]), null when off
  SvmLine *svm;              // per border-list entry (SVM border sampling)
  float up[3];               // row 1 of the world-view matrix
};

void launch_pixels(const DevScene &s, const DevPreset &p, const DevView &v, cudaStream_t st);
void launch_border_detect(const DevPreset &p, const DevView &v, cudaStream_t st);
void launch_border(const DevScene &s, const DevPreset &p, const DevView &v, uint32_t max_pixels, int n_sm,
                   cudaStream_t st);
// the SVM stage of CastBorderRaySVM for every border pixel, into v.svm
void launch_svm_lines(const DevScene &s, const DevPreset &p, const DevView &v, uint32_t max_pixels, int n_sm,
                      cudaStream_t st);
// Regularization (diff_render/MultiRendererDR.cpp:1933-2055) into s.grad
void launch_regularize(const DevScene &s, uint32_t n_nodes, float lambda, float power, cudaStream_t st);
// Redistance (:2122-2330) of the dense n^3 grid at the start of dist, in place
cudaError_t launch_redistance(float *dist, uint32_t n, float h, uint32_t n_iters, cudaStream_t st);
void launch_adam(float *x, float *V, float *S, const float *g, uint32_t n, float inv_batch, float lr, float b1,
                 float b2, float eps, double c1, double c2, cudaStream_t st);
void launch_scale(float *g, uint32_t n, float s, cudaStream_t st);
void launch_brick_bounds(const DevScene &s, uint32_t n_nodes, float2 *out, cudaStream_t st);
void launch_query(const DevScene &s, uint32_t flags, float relax_eps, const float4 *pos, const float4 *dir, uint32_t n,
                  uint32_t *out, cudaStream_t st);

}  // namespace drk
}  // namespace lrt
