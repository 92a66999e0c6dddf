// C ABI of the differentiable SDF render (dr::MultiRendererDR replacement):
// scene / reference / preset staging, per-view gradient rendering, the
// OptimizeFixedStructure iteration with Adam, and the create_grid_sbs fixture.
// Host code only; kernels live in dr.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <new>
#include <vector>

#include "ctx_internal.h"
#include "dr_internal.h"
#include "lrt_dr.h"

namespace lrt {

struct DrState {
  lrt_sbs_header hdr{};
  uint32_t n_nodes = 0, n_params = 0;
  uint64_t n_values = 0;
  std::vector<lrt_bvh_pair> pairs;
  DevBuf<uint4> d_nodes;
  DevBuf<uint32_t> d_values;
  DevBuf<float> d_params, d_grad, d_adam;
  DevBuf<float4> d_pairs;
  DevBuf<float2> d_bounds;     // per-brick distance bounds for the exact skips
  DevBuf<float> d_bvals;       // per-brick gathered distance values
  DevBuf<float2> d_vbounds;    // per-voxel corner bounds (the walks' skip test)
  // views
  std::vector<lrt_view> views;
  std::vector<lrt_view> orig_views;   // the reference as lrt_dr_set_reference received it
  std::vector<float> orig_images;
  std::vector<size_t> off;     // pixel offset of each view
  size_t n_pix = 0, max_view_pix = 0;
  DevBuf<float4> d_ref, d_img;
  DevBuf<float> d_depth;
  DevBuf<uint8_t> d_border_mask;
  DevBuf<uint8_t> d_cast_mask;  // ray-casting masks of all views (raycasting_mask)
  DevBuf<drk::SvmLine> d_svm;   // SVM sampling lines of all views' border lists
  DevBuf<uint32_t> d_border_list, d_border_count, d_status;
  DevBuf<double> d_loss;
  lrt_dr_preset preset{};
  bool has_scene = false, has_ref = false;
  uint32_t last_launches = 0;
  // summed batches: views run concurrently on side streams forked from and joined
  // back into the caller's stream, so one view's tail overlaps the next one's work
  static constexpr int kSide = 4;
  cudaStream_t side[kSide] = {};
  cudaEvent_t fork = nullptr, join[kSide] = {};
};

void dr_state_free(DrState *st) {
  if (!st) return;
  for (auto *b : {&st->d_params, &st->d_grad, &st->d_adam}) b->release();
  st->d_nodes.release();
  st->d_values.release();
  st->d_pairs.release();
  st->d_bounds.release();
  st->d_bvals.release();
  st->d_vbounds.release();
  st->d_ref.release();
  st->d_img.release();
  st->d_depth.release();
  st->d_border_mask.release();
  st->d_cast_mask.release();
  st->d_svm.release();
  st->d_border_list.release();
  st->d_border_count.release();
  st->d_status.release();
  for (int k = 0; k < DrState::kSide; k++) {
    if (st->side[k]) cudaStreamDestroy(st->side[k]);
    if (st->join[k]) cudaEventDestroy(st->join[k]);
  }
  if (st->fork) cudaEventDestroy(st->fork);
  st->d_loss.release();
  delete st;
}

}  // namespace lrt

namespace {

lrt_status ensure_state(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!ctx->dr) {
    ctx->dr = new (std::nothrow) DrState();
    if (!ctx->dr) return fail(ctx, LRT_ERR_OOM, "DR state allocation failed");
    lrt_dr_default_preset(&ctx->dr->preset);
  }
  return LRT_OK;
}

template <typename T>
cudaError_t upload(DevBuf<T> &b, const T *h, size_t n) {
  cudaError_t e = b.ensure(n);
  if (e != cudaSuccess) return e;
  return cudaMemcpy(b.p, h, n * sizeof(T), cudaMemcpyHostToDevice);
}

// m_proj * m_worldView (TransformWorldToScreenSpace, diff_render/MultiRendererDR.cpp:1296-1301)
void mat4_mul(const float *a, const float *b, float *r) {
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      r[i * 4 + j] = a[i * 4 + 0] * b[0 * 4 + j] + a[i * 4 + 1] * b[1 * 4 + j] + a[i * 4 + 2] * b[2 * 4 + j] +
                     a[i * 4 + 3] * b[3 * 4 + j];
}

// ray flags of CastRayWithGrad (diff_render/MultiRendererDR.cpp:1113-1140)
uint32_t pixel_flags(const lrt_dr_preset &p) {
  if (p.input_type == 1) return 16u;
  uint32_t f = 0;
  if (p.reconstruction_flags & LRT_DR_RECON_COLOR) f |= 1u;
  if (p.reconstruction_flags & LRT_DR_RECON_GEOMETRY) {
    if (p.render_mode == LRT_DR_RENDER_DIFFUSE) f |= 2u;
    else if (p.render_mode == LRT_DR_RENDER_LAMBERT) f |= 2u | 4u;
    else if (p.render_mode == LRT_DR_RENDER_NORMAL) f |= 4u;
  }
  return f;
}

// BVHRT::need_normal of the MultiRenderer mode the DR mode maps to
// (diff_render/MultiRendererDR.cpp:98-116, BVH/BVH2Common.cpp:20-27)
bool dr_need_normal(uint32_t render_mode) {
  return render_mode == LRT_DR_RENDER_LAMBERT || render_mode == LRT_DR_RENDER_NORMAL;
}

drk::DevScene dev_scene(lrt_ctx *ctx) {
  DrState &st = *ctx->dr;
  drk::DevScene s{};
  s.nodes = st.d_nodes.p;
  s.values = st.d_values.p;
  s.P = st.d_params.p;
  s.grad = st.d_grad.p;
  s.pairs = st.d_pairs.p;
  s.n_pairs = uint32_t(st.pairs.size());
  s.brick_bounds = st.d_bounds.p;
  s.bvals = st.d_bvals.p;
  s.vbounds = st.d_vbounds.p;
  s.brick_size = st.hdr.brick_size;
  s.v_size = st.hdr.brick_size + 2 * st.hdr.brick_pad + 1;
  s.layout_in = (st.hdr.aux_data & 0xFF000000u) == (5u << 24) ? 1u : 0u;
  s.need_normal = dr_need_normal(st.preset.render_mode) ? 1u : 0u;
  for (int k = 0; k < 3; k++) { s.inst_bmin[k] = -1.0f; s.inst_bmax[k] = 1.0f; }
  const float id[12] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0};
  std::memcpy(s.inst_inv, id, sizeof(id));
  s.status = st.d_status.p;
  return s;
}

drk::DevPreset dev_preset(const DrState &st) {
  const lrt_dr_preset &p = st.preset;
  drk::DevPreset d{};
  d.render_mode = p.render_mode;
  d.recon = p.reconstruction_flags;
  d.input_type = p.input_type;
  d.loss_fn = p.loss_function;
  d.spp = p.spp;
  d.border_spp = p.border_spp;
  d.seed = p.seed;
  d.n_lights = p.n_lights;
  d.relax_eps = p.border_relax_eps;
  for (uint32_t i = 0; i < 4; i++) {
    d.light_type[i] = p.lights[i].type;
    for (int k = 0; k < 3; k++) { d.light_dir[i][k] = p.lights[i].dir[k]; d.light_col[i][k] = p.lights[i].color[k]; }
  }
  d.agg = p.warp_aggregate;
  d.flags = pixel_flags(p);
  d.svm = p.border_sampling;
  if (d.svm) {   // svm_spp = max(1, 0.25 border_spp) rounded down to a square (:1675-1678)
    uint32_t n = (uint32_t)(0.25f * float(p.border_spp));
    if (n < 1u) n = 1u;
    d.svm_sqrt = (uint32_t)std::sqrt(double(n));
    d.svm_spp = d.svm_sqrt * d.svm_sqrt;
  }
  return d;
}

drk::DevView dev_view(DrState &st, uint32_t v) {
  const lrt_view &lv = st.views[v];
  drk::DevView d{};
  d.width = lv.width;
  d.height = lv.height;
  lrt_inverse4x4(lv.proj, d.proj_inv);
  lrt_inverse4x4(lv.world_view, d.wv_inv);
  mat4_mul(lv.proj, lv.world_view, d.pv);
  d.ref = st.d_ref.p + st.off[v];
  d.img = st.d_img.p + st.off[v];
  d.depth = st.d_depth.p + st.off[v];
  d.border_mask = st.d_border_mask.p + st.off[v];
  d.border_list = st.d_border_list.p + st.off[v];
  d.border_count = st.d_border_count.p + v;
  d.loss = st.d_loss.p + v;
  d.cast_mask = st.preset.raycasting_mask ? st.d_cast_mask.p + st.off[v] : nullptr;
  d.svm = st.preset.border_sampling ? st.d_svm.p + st.off[v] : nullptr;
  for (int k = 0; k < 3; k++) d.up[k] = lv.world_view[4 + k];
  return d;
}

// RenderDR for view v, gradients added into d_grad (:578-750)
lrt_status render_view(lrt_ctx *ctx, uint32_t v, cudaStream_t stream) {
  DrState &st = *ctx->dr;
  const drk::DevScene s = dev_scene(ctx);
  drk::DevPreset p = dev_preset(st);
  const drk::DevView dv = dev_view(st, v);
  const uint32_t W = dv.width, H = dv.height;
  p.g_mult = float(std::pow(st.n_params + 1.0, 2.0 / 3.0) / (double(W) * double(H)));   // getBaseGradientMult :140-145
  LRT_CUDA(ctx, cudaMemsetAsync(dv.loss, 0, sizeof(double), stream));
  LRT_CUDA(ctx, cudaMemsetAsync(dv.border_count, 0, sizeof(uint32_t), stream));
  drk::launch_pixels(s, p, dv, stream);
  drk::launch_border_detect(p, dv, stream);
  st.last_launches += 2;
  if ((st.preset.reconstruction_flags & LRT_DR_RECON_GEOMETRY) && st.preset.border_spp > 0) {
    if (p.svm) {
      drk::launch_svm_lines(s, p, dv, W * H, ctx->num_sms, stream);
      st.last_launches += 1;
    }
    drk::launch_border(s, p, dv, W * H, ctx->num_sms, stream);
    st.last_launches += 1;
  }
  LRT_CUDA(ctx, cudaGetLastError());
  return LRT_OK;
}

// Buffers of the optional DR features for the current views; the ray-casting
// masks restart full (OptimizeFixedStructure :369-383).
lrt_status prepare_extras(lrt_ctx *ctx) {
  DrState &st = *ctx->dr;
  if (!st.has_ref || st.n_pix == 0) return LRT_OK;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  if (st.preset.raycasting_mask) {
    LRT_CUDA(ctx, st.d_cast_mask.ensure(st.n_pix));
    LRT_CUDA(ctx, cudaMemset(st.d_cast_mask.p, 1, st.n_pix));
  }
  if (st.preset.border_sampling) LRT_CUDA(ctx, st.d_svm.ensure(st.n_pix));
  return LRT_OK;
}

lrt_status check_ready(lrt_ctx *ctx) {
  if (!ctx || !ctx->dr || !ctx->dr->has_scene) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_scene first");
  if (!ctx->dr->has_ref) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_reference first");
  return LRT_OK;
}

lrt_status read_status(lrt_ctx *ctx) {
  uint32_t status = 0;
  LRT_CUDA(ctx, cudaMemcpy(&status, ctx->dr->d_status.p, 4, cudaMemcpyDeviceToHost));
  if (status & drk::kStatusStackOverflow)
    return fail(ctx, LRT_ERR_BOUNDS, "BVH traversal stack (80 entries, the reference's STACK_SIZE) overflowed");
  if (status & drk::kStatusTraversalBound)
    return fail(ctx, LRT_ERR_BOUNDS, "BVH traversal visited more nodes than the tree holds (malformed BVH)");
  return LRT_OK;
}

}  // namespace

extern "C" void lrt_dr_default_preset(lrt_dr_preset *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->render_mode = LRT_DR_RENDER_LAMBERT;
  p->reconstruction_flags = LRT_DR_RECON_COLOR | LRT_DR_RECON_GEOMETRY;
  p->input_type = 0;
  p->loss_function = 0;
  p->spp = 1;
  p->border_spp = 256;
  p->border_relax_eps = 1e-3f;
  p->seed = 1;
  p->n_lights = 2;
  const float inv = 1.0f / std::sqrt(3.0f);
  p->lights[0] = lrt_dr_light{LRT_DR_LIGHT_DIRECT, {inv, inv, inv}, {2.0f / 3.0f, 2.0f / 3.0f, 2.0f / 3.0f}};
  p->lights[1] = lrt_dr_light{LRT_DR_LIGHT_AMBIENT, {0, 0, 0}, {0.25f, 0.25f, 0.25f}};
  p->opt_lr = 0.01f;
  p->opt_beta_1 = 0.9f;
  p->opt_beta_2 = 0.999f;
  p->opt_eps = 1e-8f;
  p->accumulate_batch = 0;
  p->warp_aggregate = 1;
  p->reg_function = 0;            // getDefaultPresetDR, diff_render/MultiRendererDR.h:42-47
  p->reg_lambda = 0.25f;
  p->reg_power = 2.0f;
  p->redistancing_enable = 0;
  p->redistancing_interval = 1;
}

extern "C" lrt_status lrt_dr_set_scene(lrt_ctx *ctx, const lrt_sbs_header *hdr, const lrt_sbs_node *nodes,
                                       uint32_t n_nodes, const uint32_t *values, uint64_t n_values,
                                       const float *params, uint32_t n_params, const lrt_bvh_pair *pairs,
                                       uint32_t n_pairs) {
  lrt_status s = ensure_state(ctx);
  if (s != LRT_OK) return s;
  if (!hdr || !nodes || !values || !params || n_nodes == 0 || n_values == 0 || n_params == 0)
    return fail(ctx, LRT_ERR_INVALID, "lrt_dr_set_scene: empty scene");
  const uint32_t layout = hdr->aux_data & 0xFF000000u;
  if (layout != (4u << 24) && layout != (5u << 24))
    return fail(ctx, LRT_ERR_UNSUPPORTED, "DR needs the ID32F_IRGB32F or ID32F_IRGB32F_IN layout");
  if (n_nodes > 0x00FFFFFFu) return fail(ctx, LRT_ERR_UNSUPPORTED, "more bricks than a BVH leaf can address");
  const uint64_t v3 = uint64_t(hdr->brick_size + 2 * hdr->brick_pad + 1) * (hdr->brick_size + 2 * hdr->brick_pad + 1) *
                      (hdr->brick_size + 2 * hdr->brick_pad + 1);
  const uint64_t per = v3 + 8 + (layout == (5u << 24) ? 27 : 0);
  // host-side bounds: every index the kernels follow must stay inside the arrays
  for (uint32_t i = 0; i < n_nodes; i++) {
    if (uint64_t(nodes[i].data_offset) + per > n_values)
      return fail(ctx, LRT_ERR_BOUNDS, "node data_offset beyond the values array");
    const uint32_t *b = values + nodes[i].data_offset;
    for (uint64_t k = 0; k < v3; k++)
      if (b[k] >= n_params) return fail(ctx, LRT_ERR_BOUNDS, "distance index beyond the parameters");
    for (int k = 0; k < 8; k++)
      if (uint64_t(b[v3 + k]) + 3 > n_params) return fail(ctx, LRT_ERR_BOUNDS, "colour index beyond the parameters");
    if (layout == (5u << 24))
      for (int k = 0; k < 27; k++)
        if (b[v3 + 8 + k] != drk::kInvalidIdx && b[v3 + 8 + k] >= n_nodes)
          return fail(ctx, LRT_ERR_BOUNDS, "neighbour index beyond the nodes");
  }
  DrState &st = *ctx->dr;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  st.hdr = *hdr;
  st.n_nodes = n_nodes;
  st.n_values = n_values;
  st.n_params = n_params;
  if (pairs && n_pairs) {
    st.pairs.assign(pairs, pairs + n_pairs);
  } else {
    std::vector<float> boxes(6 * size_t(n_nodes));
    for (uint32_t i = 0; i < n_nodes; i++) {   // AddGeom_SdfSBS boxes, BVH/BVH2Common_host.cpp:640-653
      const float px = float(nodes[i].pos_xy >> 16), py = float(nodes[i].pos_xy & 0xFFFF);
      const float pz = float(nodes[i].pos_z_lod_size >> 16), sz = float(nodes[i].pos_z_lod_size & 0xFFFF);
      const float lo[3] = {-1 + 2.0f * px / sz, -1 + 2.0f * py / sz, -1 + 2.0f * pz / sz};
      for (int k = 0; k < 3; k++) {
        boxes[6 * i + k] = lo[k];
        boxes[6 * i + 3 + k] = lo[k] + 2.0f * 1 / sz;
      }
    }
    bool built = false;
    if (ctx->bvh_builder != 0) {   // device build (lrt_set_tuning "bvh_builder"), pairs fetched back
      const uint32_t n_int = n_nodes > 1 ? n_nodes - 1 : 1;
      DevBuf<float> d_boxes;
      DevBuf<WNode4> d_wide;
      DevBuf<lrt_bvh_pair> d_pairs;
      cudaError_t e = upload(d_boxes, boxes.data(), boxes.size());
      if (e == cudaSuccess) e = d_wide.ensure(n_int);
      if (e == cudaSuccess) e = d_pairs.ensure(n_int);
      GpuBvhInfo info;
      if (e == cudaSuccess)
        e = build_bvh_gpu(d_boxes.p, n_nodes, true, ctx->bvh_builder == 1, d_wide.p, nullptr, d_pairs.p, nullptr,
                          info, 0);
      if (e == cudaSuccess) {
        st.pairs.resize(info.n_pairs);
        e = cudaMemcpy(st.pairs.data(), d_pairs.p, size_t(info.n_pairs) * sizeof(lrt_bvh_pair),
                       cudaMemcpyDeviceToHost);
        built = e == cudaSuccess;
      }
      d_boxes.release();
      d_wide.release();
      d_pairs.release();
      if (e == cudaErrorNotSupported) (void)cudaGetLastError();   // the host builder makes the same tree
      else if (e != cudaSuccess) return cuda_fail(ctx, e, "lrt_dr_set_scene: device BVH build");
    }
    if (!built) {
      BvhData b;
      s = build_bvh(boxes.data(), n_nodes, true, b);
      if (s != LRT_OK) return fail(ctx, s, "BVH build failed");
      st.pairs.assign(reinterpret_cast<const lrt_bvh_pair *>(b.pairs.data()),
                      reinterpret_cast<const lrt_bvh_pair *>(b.pairs.data()) + b.pairs.size());
    }
  }
  // every child reference of the BVH2 must be a pair index or a leaf of a valid brick
  for (const lrt_bvh_pair &p : st.pairs)
    for (const lrt_bvh_node *c : {&p.left, &p.right}) {
      const uint32_t o = c->leftOffset;
      if (o == 0xFFFFFFFFu) continue;
      if (o & 0x80000000u) {
        if ((o & 0x00FFFFFFu) >= n_nodes) return fail(ctx, LRT_ERR_BOUNDS, "BVH leaf beyond the nodes");
      } else if (o >= st.pairs.size()) {
        return fail(ctx, LRT_ERR_BOUNDS, "BVH child beyond the pairs");
      }
    }
  cudaError_t e;
  if ((e = upload(st.d_nodes, reinterpret_cast<const uint4 *>(nodes), n_nodes)) != cudaSuccess)
    return cuda_fail(ctx, e, "upload nodes");
  if ((e = upload(st.d_values, values, size_t(n_values))) != cudaSuccess) return cuda_fail(ctx, e, "upload values");
  if ((e = upload(st.d_params, params, n_params)) != cudaSuccess) return cuda_fail(ctx, e, "upload params");
  if ((e = upload(st.d_pairs, reinterpret_cast<const float4 *>(st.pairs.data()), st.pairs.size() * 4)) != cudaSuccess)
    return cuda_fail(ctx, e, "upload BVH");
  LRT_CUDA(ctx, st.d_grad.ensure(n_params));
  LRT_CUDA(ctx, st.d_adam.ensure(2 * size_t(n_params)));
  LRT_CUDA(ctx, cudaMemset(st.d_grad.p, 0, sizeof(float) * n_params));
  LRT_CUDA(ctx, cudaMemset(st.d_adam.p, 0, sizeof(float) * 2 * size_t(n_params)));
  LRT_CUDA(ctx, st.d_status.ensure(1));
  LRT_CUDA(ctx, cudaMemset(st.d_status.p, 0, 4));
  LRT_CUDA(ctx, st.d_bounds.ensure(n_nodes));
  LRT_CUDA(ctx, st.d_bvals.ensure(size_t(n_nodes) * v3));
  LRT_CUDA(ctx, st.d_vbounds.ensure(size_t(n_nodes) * hdr->brick_size * hdr->brick_size * hdr->brick_size));
  st.has_scene = true;
  return prepare_extras(ctx);
}

extern "C" lrt_status lrt_dr_get_bvh2(lrt_ctx *ctx, const lrt_bvh_pair **pairs, uint32_t *n_pairs) {
  if (!ctx || !ctx->dr || !ctx->dr->has_scene || !pairs || !n_pairs) return LRT_ERR_INVALID;
  *pairs = ctx->dr->pairs.data();
  *n_pairs = uint32_t(ctx->dr->pairs.size());
  return LRT_OK;
}

// the device side of SetReference: views, target images and per-view buffers
static lrt_status upload_reference(lrt_ctx *ctx, uint32_t n_views, const lrt_view *views, const float *images) {
  DrState &st = *ctx->dr;
  st.views.assign(views, views + n_views);
  st.off.assign(n_views, 0);
  size_t n = 0, mx = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    if (views[v].width == 0 || views[v].height == 0 || views[v].width > 16384 || views[v].height > 16384)
      return fail(ctx, LRT_ERR_INVALID, "view size out of range");
    st.off[v] = n;
    const size_t px = size_t(views[v].width) * views[v].height;
    n += px;
    mx = std::max(mx, px);
  }
  st.n_pix = n;
  st.max_view_pix = mx;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  cudaError_t e;
  if ((e = upload(st.d_ref, reinterpret_cast<const float4 *>(images), n)) != cudaSuccess)
    return cuda_fail(ctx, e, "upload reference images");
  LRT_CUDA(ctx, st.d_img.ensure(n));
  LRT_CUDA(ctx, st.d_depth.ensure(n));
  LRT_CUDA(ctx, st.d_border_mask.ensure(n));
  LRT_CUDA(ctx, st.d_border_list.ensure(n));   // one region per view: views may run concurrently
  LRT_CUDA(ctx, st.d_border_count.ensure(n_views));
  LRT_CUDA(ctx, st.d_loss.ensure(n_views));
  LRT_CUDA(ctx, cudaMemset(st.d_img.p, 0, n * sizeof(float4)));
  LRT_CUDA(ctx, cudaMemset(st.d_border_count.p, 0, n_views * 4));
  LRT_CUDA(ctx, cudaMemset(st.d_loss.p, 0, n_views * sizeof(double)));
  if (st.d_adam.p) LRT_CUDA(ctx, cudaMemset(st.d_adam.p, 0, sizeof(float) * 2 * size_t(st.n_params)));
  st.has_ref = true;
  return prepare_extras(ctx);
}

extern "C" lrt_status lrt_dr_set_reference(lrt_ctx *ctx, uint32_t n_views, const lrt_view *views, const float *images) {
  lrt_status s = ensure_state(ctx);
  if (s != LRT_OK) return s;
  if (n_views == 0 || !views || !images) return fail(ctx, LRT_ERR_INVALID, "lrt_dr_set_reference: no views");
  if ((s = upload_reference(ctx, n_views, views, images)) != LRT_OK) return s;
  DrState &st = *ctx->dr;
  st.orig_views.assign(views, views + n_views);
  st.orig_images.assign(images, images + 4 * st.n_pix);
  return LRT_OK;
}

// Bilinear lookup of a float RGBA image at uv in [0,1]^2: texel centres at
// (i + 0.5) / size, clamped at the edges.  (The reference samples through its
// image library's LINEAR sampler, which is not part of the reference tree; this
// is the usual definition of that filter.)
static void sample_bilinear(const float *img, uint32_t w, uint32_t h, float u, float v, float out[4]) {
  const float fx = u * float(w) - 0.5f, fy = v * float(h) - 0.5f;
  const float x0f = std::floor(fx), y0f = std::floor(fy);
  const float tx = fx - x0f, ty = fy - y0f;
  const int x0 = int(x0f), y0 = int(y0f);
  auto cx = [w](int x) { return uint32_t(std::min(std::max(x, 0), int(w) - 1)); };
  auto cy = [h](int y) { return uint32_t(std::min(std::max(y, 0), int(h) - 1)); };
  const uint32_t xa = cx(x0), xb = cx(x0 + 1), ya = cy(y0), yb = cy(y0 + 1);
  for (int c = 0; c < 4; c++) {
    const float a = img[4 * (size_t(ya) * w + xa) + c], b = img[4 * (size_t(ya) * w + xb) + c];
    const float d = img[4 * (size_t(yb) * w + xa) + c], e = img[4 * (size_t(yb) * w + xb) + c];
    out[c] = (1 - ty) * ((1 - tx) * a + tx * b) + ty * ((1 - tx) * d + tx * e);
  }
}

extern "C" lrt_status lrt_dr_preprocess_reference(uint32_t n_views, const lrt_view *views, const float *images,
                                                  uint32_t width, uint32_t height, lrt_view *out_views,
                                                  float *out_images) {
  if (n_views == 0 || !views || !images || !out_views || !out_images || width == 0 || height == 0 || width > 16384 ||
      height > 16384)
    return LRT_ERR_INVALID;
  size_t in_off = 0, out_off = 0;
  for (uint32_t n = 0; n < n_views; n++) {
    const uint32_t w0 = views[n].width, h0 = views[n].height;
    if (w0 == 0 || h0 == 0) return LRT_ERR_INVALID;
    const float *src = images + 4 * in_off;
    // CreateRefImageMasks (:169-185): 1 where the colour differs from the black background
    std::vector<float> mask(4 * size_t(w0) * h0);
    for (size_t i = 0; i < size_t(w0) * h0; i++) {
      const float r = src[4 * i], g = src[4 * i + 1], b = src[4 * i + 2];
      const float m = std::sqrt(r * r + g * g + b * b) < 0.001f ? 0.0f : 1.0f;
      for (int c = 0; c < 4; c++) mask[4 * i + c] = m;
    }
    // PreprocessRefImages (:187-226): spp_x x spp_y samples a pixel, colour from the
    // image, alpha from the mask, averaged
    const uint32_t spp_x = uint32_t(std::ceil(float(w0) / width)), spp_y = uint32_t(std::ceil(float(h0) / height));
    float *dst = out_images + 4 * out_off;
    for (uint32_t y = 0; y < height; y++)
      for (uint32_t x = 0; x < width; x++) {
        float acc[4] = {0, 0, 0, 0};
        for (uint32_t dx = 0; dx < spp_x; dx++)
          for (uint32_t dy = 0; dy < spp_y; dy++) {
            const float u = (float(spp_x * x + dx) + 0.5f) / float(spp_x * width);
            const float v = (float(spp_y * y + dy) + 0.5f) / float(spp_y * height);
            float col[4], msk[4];
            sample_bilinear(src, w0, h0, u, v, col);
            sample_bilinear(mask.data(), w0, h0, u, v, msk);
            col[3] = msk[3];
            const float k = float(spp_x * spp_y);
            for (int c = 0; c < 4; c++) acc[c] += col[c] / k;
          }
        for (int c = 0; c < 4; c++) dst[4 * (size_t(y) * width + x) + c] = acc[c];
      }
    out_views[n] = views[n];
    out_views[n].width = width;
    out_views[n].height = height;
    in_off += size_t(w0) * h0;
    out_off += size_t(width) * height;
  }
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_set_preset(lrt_ctx *ctx, const lrt_dr_preset *preset) {
  lrt_status s = ensure_state(ctx);
  if (s != LRT_OK) return s;
  if (!preset) return fail(ctx, LRT_ERR_INVALID, "null preset");
  if (preset->spp == 0 || preset->spp > drk::kMaxSpp) return fail(ctx, LRT_ERR_INVALID, "spp must be 1..64");
  if (preset->n_lights > 4) return fail(ctx, LRT_ERR_INVALID, "at most 4 lights");
  if (preset->render_mode > LRT_DR_RENDER_NORMAL || preset->loss_function > 1 || preset->input_type > 1)
    return fail(ctx, LRT_ERR_INVALID, "unknown render mode, loss or input type");
  for (uint32_t i = 0; i < preset->n_lights; i++)
    if (preset->lights[i].type != LRT_DR_LIGHT_DIRECT && preset->lights[i].type != LRT_DR_LIGHT_AMBIENT)
      return fail(ctx, LRT_ERR_UNSUPPORTED, "only direct and ambient lights");
  if (!(preset->border_relax_eps > 0.0f)) return fail(ctx, LRT_ERR_INVALID, "border_relax_eps must be > 0");
  if (preset->border_sampling > 1 || preset->raycasting_mask > 1)
    return fail(ctx, LRT_ERR_INVALID, "border_sampling and raycasting_mask are 0 or 1");
  if (preset->border_sampling == 1 && preset->border_spp > 4 * drk::kMaxSvm)
    return fail(ctx, LRT_ERR_UNSUPPORTED, "SVM border sampling takes border_spp <= 1024");
  ctx->dr->preset = *preset;
  return prepare_extras(ctx);
}

extern "C" lrt_status lrt_dr_set_params(lrt_ctx *ctx, const float *params, uint32_t n_params) {
  if (!ctx || !ctx->dr || !ctx->dr->has_scene) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_scene first");
  DrState &st = *ctx->dr;
  if (!params || n_params != st.n_params) return fail(ctx, LRT_ERR_INVALID, "parameter count differs from the scene");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemcpy(st.d_params.p, params, sizeof(float) * n_params, cudaMemcpyHostToDevice));
  LRT_CUDA(ctx, cudaMemset(st.d_adam.p, 0, sizeof(float) * 2 * size_t(n_params)));
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_render_grad(lrt_ctx *ctx, uint32_t view, double *loss) {
  lrt_status s = check_ready(ctx);
  if (s != LRT_OK) return s;
  DrState &st = *ctx->dr;
  if (view >= st.views.size()) return fail(ctx, LRT_ERR_INVALID, "view index out of range");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  st.last_launches = 0;
  LRT_CUDA(ctx, cudaMemsetAsync(st.d_grad.p, 0, sizeof(float) * st.n_params, 0));
  drk::launch_brick_bounds(dev_scene(ctx), st.n_nodes, st.d_bounds.p, 0);
  st.last_launches += 1;
  if ((s = render_view(ctx, view, 0)) != LRT_OK) return s;
  if (loss) {
    double l = 0;
    LRT_CUDA(ctx, cudaMemcpy(&l, st.d_loss.p + view, sizeof(double), cudaMemcpyDeviceToHost));
    *loss = l / double(size_t(st.views[view].width) * st.views[view].height);
    if ((s = read_status(ctx)) != LRT_OK) return s;
  }
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_step(lrt_ctx *ctx, uint32_t iter, double *losses) {
  lrt_status s = check_ready(ctx);
  if (s != LRT_OK) return s;
  DrState &st = *ctx->dr;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  st.last_launches = 0;
  const uint32_t nv = uint32_t(st.views.size());
  if (st.preset.accumulate_batch) LRT_CUDA(ctx, cudaMemsetAsync(st.d_grad.p, 0, sizeof(float) * st.n_params, 0));
  drk::launch_brick_bounds(dev_scene(ctx), st.n_nodes, st.d_bounds.p, 0);
  st.last_launches += 1;
  if (st.preset.accumulate_batch && nv > 1) {
    // summed batch: the views are independent until Adam; fork them over side streams
    if (!st.fork) {
      LRT_CUDA(ctx, cudaEventCreateWithFlags(&st.fork, cudaEventDisableTiming));
      for (int k = 0; k < DrState::kSide; k++) {
        LRT_CUDA(ctx, cudaStreamCreateWithFlags(&st.side[k], cudaStreamNonBlocking));
        LRT_CUDA(ctx, cudaEventCreateWithFlags(&st.join[k], cudaEventDisableTiming));
      }
    }
    LRT_CUDA(ctx, cudaEventRecord(st.fork, 0));
    const int used = int(std::min<uint32_t>(nv, DrState::kSide));
    for (int k = 0; k < used; k++) LRT_CUDA(ctx, cudaStreamWaitEvent(st.side[k], st.fork, 0));
    for (uint32_t v = 0; v < nv; v++)
      if ((s = render_view(ctx, v, st.side[v % DrState::kSide])) != LRT_OK) return s;
    for (int k = 0; k < used; k++) {
      LRT_CUDA(ctx, cudaEventRecord(st.join[k], st.side[k]));
      LRT_CUDA(ctx, cudaStreamWaitEvent(0, st.join[k], 0));
    }
  } else {
    for (uint32_t v = 0; v < nv; v++) {
      // the reference refills its gradient buffer for every image of the batch (:412)
      if (!st.preset.accumulate_batch) LRT_CUDA(ctx, cudaMemsetAsync(st.d_grad.p, 0, sizeof(float) * st.n_params, 0));
      if ((s = render_view(ctx, v, 0)) != LRT_OK) return s;
    }
  }
  const lrt_dr_preset &p = st.preset;
  if (p.reg_function != 0) {   // :453-456, into the batch gradient before the division
    drk::launch_regularize(dev_scene(ctx), st.n_nodes, p.reg_lambda, p.reg_power, 0);
    st.last_launches += 1;
  }
  if (p.redistancing_enable && p.redistancing_interval && iter % p.redistancing_interval == 0) {   // :459-466
    const uint32_t bc = uint32_t(std::cbrt(double(st.n_nodes)));
    const uint32_t pc = bc * st.hdr.brick_size + 1;
    if (uint64_t(pc) * pc * pc > st.n_params) return fail(ctx, LRT_ERR_INVALID, "redistancing needs a cubic grid set");
    LRT_CUDA(ctx, drk::launch_redistance(st.d_params.p, pc, 2.f / float(pc), pc, 0));
    st.last_launches += pc + 1;
  }
  const double c1 = 1.0 - std::pow(double(p.opt_beta_1), double(iter + 1));
  const double c2 = 1.0 - std::pow(double(p.opt_beta_2), double(iter + 1));
  drk::launch_adam(st.d_params.p, st.d_adam.p, st.d_adam.p + st.n_params, st.d_grad.p, st.n_params, float(nv),
                   p.opt_lr, p.opt_beta_1, p.opt_beta_2, p.opt_eps, c1, c2, 0);
  st.last_launches += 1;
  LRT_CUDA(ctx, cudaGetLastError());
  if (losses) {
    std::vector<double> l(nv);
    LRT_CUDA(ctx, cudaMemcpy(l.data(), st.d_loss.p, nv * sizeof(double), cudaMemcpyDeviceToHost));
    for (uint32_t v = 0; v < nv; v++) losses[v] = l[v] / double(size_t(st.views[v].width) * st.views[v].height);
    if ((s = read_status(ctx)) != LRT_OK) return s;
  }
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_optimize(lrt_ctx *ctx, uint32_t first_iter, uint32_t iterations, double *last_losses) {
  lrt_status s = check_ready(ctx);
  if (s != LRT_OK) return s;
  for (uint32_t i = 0; i < iterations; i++)
    if ((s = lrt_dr_step(ctx, first_iter + i, i + 1 == iterations ? last_losses : nullptr)) != LRT_OK) return s;
  LRT_CUDA(ctx, cudaDeviceSynchronize());
  return read_status(ctx);
}

namespace {
// malloc'd arrays of one grid (lrt_dr_grid_resample's outputs)
struct GridArrays {
  lrt_sbs_header hdr{};
  lrt_sbs_node *nodes = nullptr;
  uint32_t n_nodes = 0, n_params = 0;
  uint32_t *values = nullptr;
  uint64_t n_values = 0;
  float *params = nullptr;
  void clear() {
    std::free(nodes); std::free(values); std::free(params);
    nodes = nullptr; values = nullptr; params = nullptr;
  }
  ~GridArrays() { clear(); }
};
}  // namespace

extern "C" lrt_status lrt_dr_optimize_grid(lrt_ctx *ctx, uint32_t start_grid_size, uint32_t no_last_step_resize,
                                           const lrt_dr_preset *presets, const uint32_t *iterations,
                                           const uint32_t *render_sizes, uint32_t n_stages, lrt_sbs_header *hdr,
                                           lrt_sbs_node **nodes,
                                           uint32_t *n_nodes, uint32_t **values, uint64_t *n_values, float **params,
                                           uint32_t *n_params, double *last_losses) {
  if (!ctx) return LRT_ERR_INVALID;
  if (!presets || !iterations || n_stages == 0 || start_grid_size == 0 || !hdr || !nodes || !n_nodes || !values ||
      !n_values || !params || !n_params)
    return fail(ctx, LRT_ERR_INVALID, "lrt_dr_optimize_grid: bad arguments");
  for (uint32_t i = 0; i < n_stages; i++)
    if (iterations[i] == 0) return fail(ctx, LRT_ERR_INVALID, "lrt_dr_optimize_grid: every stage needs iterations");
  lrt_status s = ensure_state(ctx);
  if (s != LRT_OK) return s;
  if (!ctx->dr->has_ref) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_reference first");
  GridArrays g;
  uint32_t bs = 1;
  s = lrt_dr_grid_resample(start_grid_size, bs, nullptr, 0, &g.hdr, &g.nodes, &g.n_nodes, &g.values, &g.n_values,
                           &g.params, &g.n_params);
  if (s != LRT_OK) return fail(ctx, s, "lrt_dr_optimize_grid: starting grid");
  DrState &st = *ctx->dr;
  for (uint32_t i = 0; i < n_stages; i++) {
    // OptimizeFixedStructure (:278-576): the reference images at the stage's render
    // size (PreprocessRefImages, :322-339; 0 x 0 = as given), scene, preset,
    // iterations; the optimised parameters become the grid's values_f (:574)
    const uint32_t rw = render_sizes ? render_sizes[2 * i] : 0, rh = render_sizes ? render_sizes[2 * i + 1] : 0;
    const uint32_t nv = uint32_t(st.orig_views.size());
    if (rw && rh) {
      std::vector<lrt_view> v2(nv);
      std::vector<float> im2(4 * size_t(rw) * rh * nv);
      if ((s = lrt_dr_preprocess_reference(nv, st.orig_views.data(), st.orig_images.data(), rw, rh, v2.data(),
                                           im2.data())) != LRT_OK)
        return fail(ctx, s, "lrt_dr_optimize_grid: render size");
      if ((s = upload_reference(ctx, nv, v2.data(), im2.data())) != LRT_OK) return s;
    } else if ((s = upload_reference(ctx, nv, st.orig_views.data(), st.orig_images.data())) != LRT_OK) {
      return s;
    }
    if ((s = lrt_dr_set_preset(ctx, &presets[i])) != LRT_OK) return s;
    if ((s = lrt_dr_set_scene(ctx, &g.hdr, g.nodes, g.n_nodes, g.values, g.n_values, g.params, g.n_params, nullptr,
                              0)) != LRT_OK)
      return s;
    if ((s = lrt_dr_optimize(ctx, 0, iterations[i], last_losses)) != LRT_OK) return s;
    LRT_CUDA(ctx, cudaMemcpy(g.params, ctx->dr->d_params.p, sizeof(float) * g.n_params, cudaMemcpyDeviceToHost));
    // the grid resampled into bricks twice as large, or as large after the last stage
    // with no_last_step_resize (:264-273)
    const uint32_t nbs = (i + 1 == n_stages && no_last_step_resize) ? bs : 2 * bs;
    GridArrays n;
    s = lrt_dr_grid_resample(start_grid_size, nbs, g.params, bs, &n.hdr, &n.nodes, &n.n_nodes, &n.values, &n.n_values,
                             &n.params, &n.n_params);
    if (s != LRT_OK) return fail(ctx, s, "lrt_dr_optimize_grid: resampled grid");
    g.clear();
    std::swap(g.hdr, n.hdr);
    std::swap(g.nodes, n.nodes);
    std::swap(g.n_nodes, n.n_nodes);
    std::swap(g.values, n.values);
    std::swap(g.n_values, n.n_values);
    std::swap(g.params, n.params);
    std::swap(g.n_params, n.n_params);
    bs = nbs;
  }
  *hdr = g.hdr;
  *nodes = g.nodes;
  *n_nodes = g.n_nodes;
  *values = g.values;
  *n_values = g.n_values;
  *params = g.params;
  *n_params = g.n_params;
  g.nodes = nullptr; g.values = nullptr; g.params = nullptr;
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_get(lrt_ctx *ctx, uint32_t what, uint32_t view, void *out, uint64_t bytes) {
  if (!ctx || !ctx->dr || !ctx->dr->has_scene || !out) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_scene first");
  DrState &st = *ctx->dr;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  const void *src = nullptr;
  uint64_t want = 0;
  if (what == LRT_DR_PARAMS) { src = st.d_params.p; want = 4ull * st.n_params; }
  else if (what == LRT_DR_GRAD) { src = st.d_grad.p; want = 4ull * st.n_params; }
  else if (what == LRT_DR_ADAM) { src = st.d_adam.p; want = 8ull * st.n_params; }
  else {
    if (!st.has_ref || view >= st.views.size()) return fail(ctx, LRT_ERR_INVALID, "no such view");
    const uint64_t px = uint64_t(st.views[view].width) * st.views[view].height;
    if (what == LRT_DR_IMAGE) { src = st.d_img.p + st.off[view]; want = 16 * px; }
    else if (what == LRT_DR_DEPTH) { src = st.d_depth.p + st.off[view]; want = 4 * px; }
    else if (what == LRT_DR_BORDER) { src = st.d_border_mask.p + st.off[view]; want = px; }
    else if (what == LRT_DR_CAST_MASK) {
      if (!st.preset.raycasting_mask || !st.d_cast_mask.p) return fail(ctx, LRT_ERR_STATE, "raycasting_mask is off");
      src = st.d_cast_mask.p + st.off[view];
      want = px;
    } else return fail(ctx, LRT_ERR_INVALID, "unknown item");
  }
  if (bytes != want) return fail(ctx, LRT_ERR_INVALID, "output size mismatch");
  LRT_CUDA(ctx, cudaMemcpy(out, src, bytes, cudaMemcpyDeviceToHost));
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_query_rays(lrt_ctx *ctx, uint32_t flags, const float *pos_near, const float *dir_far,
                                        uint32_t n, uint32_t *out) {
  if (!ctx || !ctx->dr || !ctx->dr->has_scene) return fail(ctx, LRT_ERR_STATE, "lrt_dr_set_scene first");
  if (!pos_near || !dir_far || !out || n == 0) return fail(ctx, LRT_ERR_INVALID, "empty ray batch");
  if (flags & ~63u) return fail(ctx, LRT_ERR_INVALID, "unknown ray flags");
  DrState &st = *ctx->dr;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  DevBuf<float4> dp, dd;
  DevBuf<uint32_t> dout;
  cudaError_t e;
  if ((e = upload(dp, reinterpret_cast<const float4 *>(pos_near), n)) != cudaSuccess ||
      (e = upload(dd, reinterpret_cast<const float4 *>(dir_far), n)) != cudaSuccess ||
      (e = dout.ensure(size_t(n) * 32)) != cudaSuccess) {
    dp.release(); dd.release(); dout.release();
    return cuda_fail(ctx, e, "lrt_dr_query_rays buffers");
  }
  drk::launch_brick_bounds(dev_scene(ctx), st.n_nodes, st.d_bounds.p, 0);
  drk::DevScene s = dev_scene(ctx);
  drk::launch_query(s, flags, st.preset.border_relax_eps, dp.p, dd.p, n, dout.p, 0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(out, dout.p, size_t(n) * 32 * 4, cudaMemcpyDeviceToHost);
  dp.release(); dd.release(); dout.release();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "lrt_dr_query_rays");
  return read_status(ctx);
}

extern "C" uint32_t lrt_dr_last_launch_count(const lrt_ctx *ctx) {
  return (ctx && ctx->dr) ? ctx->dr->last_launches : 0;
}

using DistFn = std::function<float(float, float, float)>;
using ColorFn = std::function<void(float, float, float, float *)>;

// create_grid_sbs (diff_render/DR_common.cpp:47-146) + SBS_ind_to_SBS_ind_with_neighbors
static lrt_status make_grid(uint32_t bc, uint32_t bs, const DistFn &dist, const ColorFn &color, lrt_sbs_header *hdr,
                            lrt_sbs_node **nodes_out, uint32_t *n_nodes, uint32_t **values_out, uint64_t *n_values,
                            float **params_out, uint32_t *n_params) {
  if (!hdr || !nodes_out || !n_nodes || !values_out || !n_values || !params_out || !n_params || bc == 0 || bs == 0 ||
      bc > 1024 || bs > 64)
    return LRT_ERR_INVALID;
  const uint64_t v = bs + 1, dist_per_node = v * v * v, pc = uint64_t(bc) * bs + 1, cc = uint64_t(bc) + 1;
  const uint64_t c_off = pc * pc * pc, nn = uint64_t(bc) * bc * bc;
  const uint64_t per_old = dist_per_node + 8, per_new = dist_per_node + 8 + 27;
  const uint64_t np = pc * pc * pc + 3 * cc * cc * cc;
  if (np >= 0x80000000ull || nn * per_new >= (1ull << 40)) return LRT_ERR_UNSUPPORTED;
  float *P = static_cast<float *>(std::malloc(np * sizeof(float)));
  lrt_sbs_node *nodes = static_cast<lrt_sbs_node *>(std::calloc(nn, sizeof(lrt_sbs_node)));
  uint32_t *vals = static_cast<uint32_t *>(std::malloc(nn * per_new * sizeof(uint32_t)));
  if (!P || !nodes || !vals) {
    std::free(P); std::free(nodes); std::free(vals);
    return LRT_ERR_OOM;
  }
  hdr->brick_size = bs;
  hdr->brick_pad = 0;
  hdr->bytes_per_value = 4;
  hdr->aux_data = 5u << 24;   // SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F_IN
  // distances at 2 * (i / (bc * bs)) - 1 (DR_common.cpp:72-85)
  const float gdiv = float(bc * bs);
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < int64_t(pc); x++)
    for (uint64_t y = 0; y < pc; y++)
      for (uint64_t z = 0; z < pc; z++)
        P[uint64_t(x) * pc * pc + y * pc + z] = dist(2.0f * (float(x) / gdiv) - 1.0f, 2.0f * (float(y) / gdiv) - 1.0f,
                                                     2.0f * (float(z) / gdiv) - 1.0f);
  // colours at the brick corners (:87-102)
  const float cdiv = float(bc);
  for (uint64_t x = 0; x < cc; x++)
    for (uint64_t y = 0; y < cc; y++)
      for (uint64_t z = 0; z < cc; z++) {
        const uint64_t idx = x * cc * cc + y * cc + z;
        float c[3];
        color(2.0f * (float(x) / cdiv) - 1.0f, 2.0f * (float(y) / cdiv) - 1.0f, 2.0f * (float(z) / cdiv) - 1.0f, c);
        for (int k = 0; k < 3; k++) P[c_off + 3 * idx + k] = c[k];
      }
  // nodes and indices (:104-143)
  for (uint64_t bx = 0; bx < bc; bx++)
    for (uint64_t by = 0; by < bc; by++)
      for (uint64_t bz = 0; bz < bc; bz++) {
        const uint64_t n = bx * bc * bc + by * bc + bz, off = n * per_new;
        nodes[n].pos_xy = uint32_t((bx << 16) | by);
        nodes[n].pos_z_lod_size = uint32_t((bz << 16) | bc);
        nodes[n].data_offset = uint32_t(off);
        for (uint64_t x = 0; x < v; x++)
          for (uint64_t y = 0; y < v; y++)
            for (uint64_t z = 0; z < v; z++)
              vals[off + x * v * v + y * v + z] = uint32_t((bx * bs + x) * pc * pc + (by * bs + y) * pc + (bz * bs + z));
        for (uint64_t k = 0; k < 8; k++) {
          const uint64_t x = k >> 2, y = (k >> 1) & 1, z = k & 1;
          vals[off + dist_per_node + k] = uint32_t(c_off + 3 * ((bx + x) * cc * cc + (by + y) * cc + (bz + z)));
        }
        for (int k = 0; k < 27; k++) vals[off + per_old + k] = drk::kInvalidIdx;
      }
  // neighbours through shared corners (utils/sparse_octree_builder.cpp:2802-2850): for every
  // brick-corner value, the bricks holding it and at which corner; bricks sharing a corner
  // value are neighbours, the direction being the difference of their corner positions.
  // Only the 8 corners of each brick take part, so the table is indexed by corner record
  // (sorted by value) instead of by every value as the reference's adjacency list is.
  struct CornerRef { uint32_t value, node, r; };
  std::vector<CornerRef> refs(8 * nn);
  for (uint64_t n = 0; n < nn; n++)
    for (uint32_t r = 0; r < 8; r++) {
      const uint64_t ix = (v - 1) * ((r & 4) >> 2), iy = (v - 1) * ((r & 2) >> 1), iz = (v - 1) * (r & 1);
      refs[8 * n + r] = CornerRef{vals[nodes[n].data_offset + ix * v * v + iy * v + iz], uint32_t(n), r};
    }
  std::sort(refs.begin(), refs.end(), [](const CornerRef &a, const CornerRef &b) {
    return a.value != b.value ? a.value < b.value : a.r < b.r;
  });
  for (size_t a = 0; a < refs.size();) {
    size_t b = a;
    while (b < refs.size() && refs[b].value == refs[a].value) b++;
    for (size_t i = a; i < b; i++)
      for (size_t j = a; j < b; j++) {
        if (refs[i].r == refs[j].r) continue;
        const uint32_t r1 = refs[i].r, r2 = refs[j].r;
        const int dx = int((r2 & 4) >> 2) - int((r1 & 4) >> 2) + 1, dy = int((r2 & 2) >> 1) - int((r1 & 2) >> 1) + 1,
                  dz = int(r2 & 1) - int(r1 & 1) + 1;
        vals[uint64_t(nodes[refs[j].node].data_offset) + per_old + uint64_t(9 * dx + 3 * dy + dz)] = refs[i].node;
      }
    a = b;
  }
  *nodes_out = nodes;
  *n_nodes = uint32_t(nn);
  *values_out = vals;
  *n_values = nn * per_new;
  *params_out = P;
  *n_params = uint32_t(np);
  return LRT_OK;
}

extern "C" lrt_status lrt_dr_grid_sbs(uint32_t bc, uint32_t bs, const lrt_sdf_desc *sdf, const float *color3,
                                      lrt_sbs_header *hdr, lrt_sbs_node **nodes_out, uint32_t *n_nodes,
                                      uint32_t **values_out, uint64_t *n_values, float **params_out,
                                      uint32_t *n_params) {
  if (!sdf || (sdf->n_spheres + sdf->n_boxes) == 0) return LRT_ERR_INVALID;
  const lrt_sdf_desc f = *sdf;
  const DistFn dist = [f](float x, float y, float z) { return sdf_eval(f, x, y, z); };
  const ColorFn color = [color3](float x, float y, float z, float *c) {
    if (color3) {
      c[0] = color3[0]; c[1] = color3[1]; c[2] = color3[2];
    } else {
      const float q[3] = {x, y, z};
      for (int k = 0; k < 3; k++) c[k] = 0.5f + 0.5f * q[k];
    }
  };
  return make_grid(bc, bs, dist, color, hdr, nodes_out, n_nodes, values_out, n_values, params_out, n_params);
}

// gradient_color (diff_render/DR_common.cpp:25-35): eight weighted corner colours
// summed as float3 values, zero components included
static void gradient_color(float px, float py, float pz, float *c) {
  const float w[8] = {(1 - px) * (1 - py) * (1 - pz), (1 - px) * (1 - py) * (pz), (1 - px) * (py) * (1 - pz),
                      (1 - px) * (py) * (pz),         (px) * (1 - py) * (1 - pz), (px) * (1 - py) * (pz),
                      (px) * (py) * (1 - pz),         (px) * (py) * (pz)};
  static const float col[8][3] = {{1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 1, 0}, {1, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 1, 0}};
  for (int k = 0; k < 3; k++) {
    float a = w[0] * col[0][k];
    for (int i = 1; i < 8; i++) a = a + w[i] * col[i][k];
    c[k] = a;
  }
}

// OptimizeGrid's grid_sampler (diff_render/MultiRendererDR.cpp:242-262): trilinear
// in the dense distance grid of gs bricks of bs voxels, clamped to the cube
static float grid_sample(const float *d, uint32_t gs, uint32_t bs, float px, float py, float pz) {
  const uint32_t pc = gs * bs + 1u;
  const float p[3] = {px, py, pz};
  float f[3], dp[3];
  uint32_t i[3];
  for (int k = 0; k < 3; k++) {
    float c = 0.5f * (p[k] + 1.0f);
    c = std::min(std::max(c, 0.0f), 1.0f + 1e-6f);
    f[k] = (c * float(gs)) * float(bs);
    i[k] = uint32_t(f[k] + 1e-6f);
    dp[k] = f[k] - float(i[k]);
  }
  auto at = [&](uint32_t x, uint32_t y, uint32_t z) { return d[x * pc * pc + y * pc + z]; };
  if (i[0] < pc - 1 && i[1] < pc - 1 && i[2] < pc - 1) {
    const float x = dp[0], y = dp[1], z = dp[2];
    return (1 - x) * (1 - y) * (1 - z) * at(i[0], i[1], i[2]) + (1 - x) * (1 - y) * z * at(i[0], i[1], i[2] + 1) +
           (1 - x) * y * (1 - z) * at(i[0], i[1] + 1, i[2]) + (1 - x) * y * z * at(i[0], i[1] + 1, i[2] + 1) +
           x * (1 - y) * (1 - z) * at(i[0] + 1, i[1], i[2]) + x * (1 - y) * z * at(i[0] + 1, i[1], i[2] + 1) +
           x * y * (1 - z) * at(i[0] + 1, i[1] + 1, i[2]) + x * y * z * at(i[0] + 1, i[1] + 1, i[2] + 1);
  }
  return at(i[0], i[1], i[2]);
}

extern "C" lrt_status lrt_dr_grid_resample(uint32_t bc, uint32_t bs, const float *old_params, uint32_t old_bs,
                                           lrt_sbs_header *hdr, lrt_sbs_node **nodes, uint32_t *n_nodes,
                                           uint32_t **values, uint64_t *n_values, float **params, uint32_t *n_params) {
  if (old_params && (old_bs == 0 || old_bs > 64)) return LRT_ERR_INVALID;
  DistFn dist;
  if (old_params) {
    dist = [=](float x, float y, float z) { return grid_sample(old_params, bc, old_bs, x, y, z); };
  } else {   // circle_sdf(float3(0, -0.15, 0), 0.7, p) (:232-235; DR_common.cpp:16-19)
    dist = [](float x, float y, float z) {
      const float dx = x - 0.0f, dy = y - (-0.15f), dz = z - 0.0f;
      return std::sqrt(dx * dx + dy * dy + dz * dz) - 0.7f;
    };
  }
  return make_grid(bc, bs, dist, gradient_color, hdr, nodes, n_nodes, values, n_values, params, n_params);
}
