// C ABI of the learned proposal: weights, triple collection, training and the
// render dispatch between the plain and the proposal kernels.  Host code only;
// kernels live in proposal.cu.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "ctx_internal.h"
#include "lrt_proposal.h"
#include "mlp_image.h"
#include "proposal_internal.h"

namespace lrt {

struct ProposalState {
  DevBuf<float> master, grad, adam_m, adam_v, losses;
  DevBuf<__nv_bfloat16> wbf;
  DevBuf<unsigned int> ticket;
  DevBuf<__nv_bfloat16> feat;
  DevBuf<float> target;
  DevBuf<unsigned long long> count, stats;
  DevBuf<DevView> views;
  uint64_t n = 0;
  bool has_weights = false;
};

void proposal_state_free(ProposalState *st) {
  if (!st) return;
  for (auto *b : {&st->master, &st->grad, &st->adam_m, &st->adam_v, &st->losses, &st->target}) b->release();
  st->wbf.release();
  st->ticket.release();
  st->feat.release();
  st->count.release();
  st->stats.release();
  st->views.release();
  delete st;
}

namespace {
MlpState mlp_state(ProposalState &p, float *loss) {
  MlpState m;
  m.master = p.master.p;
  m.wbf = p.wbf.p;
  m.grad = p.grad.p;
  m.adam_m = p.adam_m.p;
  m.adam_v = p.adam_v.p;
  m.ticket = p.ticket.p;
  m.loss = loss;
  return m;
}

// round to nearest even BF16 (the device's __float2bfloat16_rn for finite values)
uint16_t f2bf(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return uint16_t(u >> 16);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}
float bf2f(uint16_t b) {
  const uint32_t u = uint32_t(b) << 16;
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

lrt_status ensure(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  if (ctx->prop) return LRT_OK;
  ProposalState *p = new (std::nothrow) ProposalState();
  if (!p) return fail(ctx, LRT_ERR_OOM, "proposal state allocation failed");
  ctx->prop = p;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  for (auto *b : {&p->master, &p->grad, &p->adam_m, &p->adam_v}) LRT_CUDA(ctx, b->ensure(LRT_MLP_PARAMS));
  LRT_CUDA(ctx, p->wbf.ensure(lrt::mlp::kBfWords));
  LRT_CUDA(ctx, p->ticket.ensure(1));
  LRT_CUDA(ctx, p->count.ensure(1));
  LRT_CUDA(ctx, p->stats.ensure(4));
  LRT_CUDA(ctx, cudaMemset(p->grad.p, 0, 4 * LRT_MLP_PARAMS));
  LRT_CUDA(ctx, cudaMemset(p->ticket.p, 0, 4));
  LRT_CUDA(ctx, cudaMemset(p->stats.p, 0, 32));
  return LRT_OK;
}
}  // namespace

// the reference's first-hit walk when "first_hit" is set (SDF scenes), else the
// plain kernels, or the proposal kernel for DX-layout SBS scenes with the NEWTON
// finder when it is switched on and the network has weights
static bool proposal_renders(const lrt_ctx *ctx, bool count) {
  const DevScene &s = ctx->dev;
  const uint32_t layout = s.sbs_hdr.aux_data & 0xFF000000u;
  const bool dx = s.type == LRT_TYPE_SDF_SBS && layout != LRT_SBS_LAYOUT_ID32F_IRGB32F &&
                  layout != LRT_SBS_LAYOUT_ID32F_IRGB32F_IN;
  return ctx->use_proposal && !count && dx && s.n_inst <= 1 && s.preset.sdf_node_intersect == LRT_INTERSECT_NEWTON &&
         ctx->prop && ctx->prop->has_weights && s.preset.spp <= 1;
}

cudaError_t dispatch_render(lrt_ctx *ctx, const RenderLaunch &L, cudaStream_t st, bool count) {
  const DevScene &s = ctx->dev;
  if (ctx->tuning.first_hit && sdf_scene(s) && s.pairs) return launch_render_ref(s, L, ctx->num_sms, st);
  if (proposal_renders(ctx, count))
    return launch_render_proposal(s, L, mlp_state(*ctx->prop, nullptr), ctx->prop->stats.p, ctx->num_sms, st);
  return launch_render(s, L, ctx->num_sms, st, count, ctx->tuning);
}

// whether the kernel dispatch_render picks (without counters) publishes chunk_done:
// the first-hit walk and launch_render's render_kernel paths do
bool dispatch_publishes_chunks(const lrt_ctx *ctx, bool color, uint32_t total_tiles) {
  const DevScene &s = ctx->dev;
  if (ctx->tuning.first_hit && sdf_scene(s) && s.pairs) return true;
  if (proposal_renders(ctx, false)) return false;
  return render_publishes_chunks(s, color, total_tiles, ctx->tuning);
}

}  // namespace lrt

using lrt::ProposalState;

extern "C" lrt_status lrt_proposal_set_weights(lrt_ctx *ctx, const float *params) {
  lrt_status s = lrt::ensure(ctx);
  if (s != LRT_OK) return s;
  if (!params) return fail(ctx, LRT_ERR_INVALID, "null parameters");
  for (int i = 0; i < LRT_MLP_PARAMS; i++)
    if (!std::isfinite(params[i])) return fail(ctx, LRT_ERR_INVALID, "non-finite parameter");
  ProposalState &p = *ctx->prop;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemcpy(p.master.p, params, 4 * LRT_MLP_PARAMS, cudaMemcpyHostToDevice));
  std::vector<uint16_t> bf(lrt::mlp::kBfWords, 0);
  for (int i = 0; i < lrt::mlp::kBfWords; i++) bf[i] = lrt::mlp::weight_image_word(params, i);
  LRT_CUDA(ctx, cudaMemcpy(p.wbf.p, bf.data(), bf.size() * 2, cudaMemcpyHostToDevice));
  LRT_CUDA(ctx, cudaMemset(p.adam_m.p, 0, 4 * LRT_MLP_PARAMS));
  LRT_CUDA(ctx, cudaMemset(p.adam_v.p, 0, 4 * LRT_MLP_PARAMS));
  LRT_CUDA(ctx, cudaMemset(p.grad.p, 0, 4 * LRT_MLP_PARAMS));
  p.has_weights = true;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_get_weights(lrt_ctx *ctx, float *params) {
  if (!ctx || !ctx->prop || !ctx->prop->has_weights || !params) return fail(ctx, LRT_ERR_STATE, "no weights set");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemcpy(params, ctx->prop->master.p, 4 * LRT_MLP_PARAMS, cudaMemcpyDeviceToHost));
  return LRT_OK;
}

static lrt_status reserve(lrt_ctx *ctx, uint64_t capacity) {
  ProposalState &p = *ctx->prop;
  if (p.feat.cap >= lrt::feat_elems(capacity) && p.target.cap >= capacity) return LRT_OK;
  // grow, keeping what is held (whole tiles; the tile layout does not depend on the capacity)
  lrt::DevBuf<__nv_bfloat16> nf;
  lrt::DevBuf<float> nt;
  LRT_CUDA(ctx, nf.ensure(size_t(lrt::feat_elems(capacity))));
  LRT_CUDA(ctx, nt.ensure(size_t(capacity)));
  LRT_CUDA(ctx, cudaMemset(nf.p, 0, size_t(lrt::feat_elems(capacity)) * 2));   // padding rows of a tile stay zero
  if (p.n) {
    LRT_CUDA(ctx, cudaMemcpy(nf.p, p.feat.p, size_t(lrt::feat_elems(p.n)) * 2, cudaMemcpyDeviceToDevice));
    LRT_CUDA(ctx, cudaMemcpy(nt.p, p.target.p, size_t(p.n) * 4, cudaMemcpyDeviceToDevice));
  }
  p.feat.release();
  p.target.release();
  p.feat = nf;
  p.target = nt;
  nf.p = nullptr;
  nt.p = nullptr;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_collect(lrt_ctx *ctx, const lrt_view *views, uint32_t n_views, uint64_t capacity,
                                           uint64_t *n_total) {
  lrt_status s = lrt::ensure(ctx);
  if (s != LRT_OK) return s;
  if (!views || n_views == 0) return fail(ctx, LRT_ERR_INVALID, "no views");
  if (!ctx->committed || ctx->dev.type != LRT_TYPE_SDF_SBS)
    return fail(ctx, LRT_ERR_STATE, "collect needs a committed SBS scene");
  const uint32_t layout = ctx->dev.sbs_hdr.aux_data & 0xFF000000u;
  if (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN)
    return fail(ctx, LRT_ERR_UNSUPPORTED, "the proposal reads DX-layout bricks");
  ProposalState &p = *ctx->prop;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  if (capacity > p.n) {
    if ((s = reserve(ctx, capacity)) != LRT_OK) return s;
  }
  std::vector<DevView> hv(n_views);
  uint64_t pix = 0;
  for (uint32_t v = 0; v < n_views; v++) {
    if (views[v].width == 0 || views[v].height == 0 || views[v].width > 65535 || views[v].height > 65535)
      return fail(ctx, LRT_ERR_INVALID, "bad view size");
    std::memset(&hv[v], 0, sizeof(DevView));
    hv[v].width = views[v].width;
    hv[v].height = views[v].height;
    hv[v].pix_offset = uint32_t(pix);
    lrt_inverse4x4(views[v].proj, hv[v].proj_inv);
    lrt_inverse4x4(views[v].world_view, hv[v].wv_inv);
    pix += uint64_t(views[v].width) * views[v].height;
    if (pix >= (1ull << 32)) return fail(ctx, LRT_ERR_INVALID, "batch too large");
  }
  LRT_CUDA(ctx, p.views.ensure(n_views));
  LRT_CUDA(ctx, cudaMemcpy(p.views.p, hv.data(), n_views * sizeof(DevView), cudaMemcpyHostToDevice));
  const unsigned long long start = p.n;
  LRT_CUDA(ctx, cudaMemcpy(p.count.p, &start, 8, cudaMemcpyHostToDevice));
  lrt::TripleBuf out{p.feat.p, p.target.p, p.count.p, capacity};
  LRT_CUDA(ctx, lrt::launch_gen_triples(ctx->dev, p.views.p, n_views, pix, out,
                                         uint32_t(ctx->tuning.proposal_target), nullptr));
  unsigned long long cnt = 0;
  LRT_CUDA(ctx, cudaMemcpy(&cnt, p.count.p, 8, cudaMemcpyDeviceToHost));
  p.n = cnt < capacity ? cnt : capacity;
  if (n_total) *n_total = p.n;
  ctx->last_launches = 1;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_clear(lrt_ctx *ctx) {
  if (!ctx) return LRT_ERR_INVALID;
  if (ctx->prop) ctx->prop->n = 0;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_set_triples(lrt_ctx *ctx, const float *features, const float *targets, uint64_t n) {
  lrt_status s = lrt::ensure(ctx);
  if (s != LRT_OK) return s;
  if (!features || !targets || n == 0) return fail(ctx, LRT_ERR_INVALID, "empty triples");
  ProposalState &p = *ctx->prop;
  p.n = 0;
  if ((s = reserve(ctx, n)) != LRT_OK) return s;
  std::vector<uint16_t> bf(size_t(lrt::feat_elems(n)), 0);
  for (uint64_t r = 0; r < n; r++)
    for (uint32_t k = 0; k < 16; k++) bf[lrt::feat_u4(r, k >> 3) * 8 + (k & 7)] = lrt::f2bf(features[r * 16 + k]);
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, cudaMemcpy(p.feat.p, bf.data(), bf.size() * 2, cudaMemcpyHostToDevice));
  LRT_CUDA(ctx, cudaMemcpy(p.target.p, targets, size_t(n) * 4, cudaMemcpyHostToDevice));
  p.n = n;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_get_triples(lrt_ctx *ctx, uint64_t first, uint64_t n, float *features,
                                               float *targets) {
  if (!ctx || !ctx->prop || first + n > ctx->prop->n) return fail(ctx, LRT_ERR_INVALID, "triple range");
  ProposalState &p = *ctx->prop;
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  if (features && n) {
    const uint64_t t0 = first >> 7, t1 = (first + n - 1) >> 7;   // the tiles holding the range
    std::vector<uint16_t> bf(size_t(t1 - t0 + 1) * 2048);
    LRT_CUDA(ctx, cudaMemcpy(bf.data(), p.feat.p + size_t(t0) * 2048, bf.size() * 2, cudaMemcpyDeviceToHost));
    for (uint64_t i = 0; i < n; i++)
      for (uint32_t k = 0; k < 16; k++)
        features[i * 16 + k] = lrt::bf2f(bf[(lrt::feat_u4(first + i, k >> 3) - t0 * 256) * 8 + (k & 7)]);
  }
  if (targets) LRT_CUDA(ctx, cudaMemcpy(targets, p.target.p + first, size_t(n) * 4, cudaMemcpyDeviceToHost));
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_train(lrt_ctx *ctx, uint32_t first_step, uint32_t steps, uint32_t batch, float lr,
                                         uint32_t seed, float *losses) {
  if (!ctx || !ctx->prop || !ctx->prop->has_weights) return fail(ctx, LRT_ERR_STATE, "set weights first");
  ProposalState &p = *ctx->prop;
  if (p.n == 0) return fail(ctx, LRT_ERR_STATE, "no triples");
  if (batch == 0 || batch % 32 != 0 || batch > (1u << 20) || steps == 0)
    return fail(ctx, LRT_ERR_INVALID, "batch must be a positive multiple of 32");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, p.losses.ensure(steps));
  LRT_CUDA(ctx, cudaMemset(p.losses.p, 0, 4 * size_t(steps)));
  const lrt::TripleView data{p.feat.p, p.target.p, 0, p.n};
  for (uint32_t k = 0; k < steps; k++) {
    const lrt::MlpState m = lrt::mlp_state(p, p.losses.p + k);
    LRT_CUDA(ctx, lrt::launch_mlp_step(data, m, batch, first_step + k, seed, true, true, lr, 0.9f, 0.999f, 1e-8f,
                                       nullptr));
  }
  if (losses) LRT_CUDA(ctx, cudaMemcpy(losses, p.losses.p, 4 * size_t(steps), cudaMemcpyDeviceToHost));
  else LRT_CUDA(ctx, cudaDeviceSynchronize());
  ctx->last_launches = steps;
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_gradient(lrt_ctx *ctx, uint32_t n, float *grad, float *loss) {
  if (!ctx || !ctx->prop || !ctx->prop->has_weights) return fail(ctx, LRT_ERR_STATE, "set weights first");
  ProposalState &p = *ctx->prop;
  if (n == 0 || n % 32 != 0 || n > p.n) return fail(ctx, LRT_ERR_INVALID, "n must be a multiple of 32 within the triples");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  LRT_CUDA(ctx, p.losses.ensure(1));
  LRT_CUDA(ctx, cudaMemset(p.losses.p, 0, 4));
  LRT_CUDA(ctx, cudaMemset(p.grad.p, 0, 4 * LRT_MLP_PARAMS));
  const lrt::TripleView data{p.feat.p, p.target.p, 0, p.n};
  const lrt::MlpState m = lrt::mlp_state(p, p.losses.p);
  LRT_CUDA(ctx, lrt::launch_mlp_step(data, m, n, 0, 0, false, false, 0.0f, 0.9f, 0.999f, 1e-8f, nullptr));
  if (grad) LRT_CUDA(ctx, cudaMemcpy(grad, p.grad.p, 4 * LRT_MLP_PARAMS, cudaMemcpyDeviceToHost));
  if (loss) LRT_CUDA(ctx, cudaMemcpy(loss, p.losses.p, 4, cudaMemcpyDeviceToHost));
  LRT_CUDA(ctx, cudaMemset(p.grad.p, 0, 4 * LRT_MLP_PARAMS));
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_infer_ex(lrt_ctx *ctx, uint64_t first, uint64_t n, float *out, int engine,
                                            float *ms) {
  if (!ctx || !ctx->prop || !ctx->prop->has_weights) return fail(ctx, LRT_ERR_STATE, "set weights first");
  ProposalState &p = *ctx->prop;
  if (!out || n == 0 || first + n > p.n) return fail(ctx, LRT_ERR_INVALID, "triple range");
  if (engine != LRT_MLP_ENGINE_MMA && engine != LRT_MLP_ENGINE_TCGEN05) return fail(ctx, LRT_ERR_INVALID, "engine");
  if ((n + 127) / 128 > 0x7FFFFFFFull) return fail(ctx, LRT_ERR_INVALID, "too many triples for one launch");
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  lrt::DevBuf<float> d;
  lrt::DevBuf<unsigned int> status;
  LRT_CUDA(ctx, d.ensure(size_t(n)));
  LRT_CUDA(ctx, status.ensure(1));
  LRT_CUDA(ctx, cudaMemset(status.p, 0, 4));
  const lrt::TripleView data{p.feat.p, p.target.p, first, n};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t e = cudaSuccess;
  if (ms) {
    e = cudaEventCreate(&ev[0]);
    if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
    if (e == cudaSuccess) e = cudaEventRecord(ev[0], nullptr);
  }
  if (e == cudaSuccess)
    e = engine == LRT_MLP_ENGINE_TCGEN05 ? lrt::launch_mlp_infer_tc(data, lrt::mlp_state(p, nullptr), d.p, status.p, nullptr,
                                                                   uint32_t(ctx->tuning.tc_wait))
                                         : lrt::launch_mlp_infer(data, lrt::mlp_state(p, nullptr), d.p, nullptr);
  if (e == cudaSuccess && ms) e = cudaEventRecord(ev[1], nullptr);
  if (e == cudaSuccess) e = ms ? cudaEventSynchronize(ev[1]) : cudaStreamSynchronize(nullptr);
  if (e == cudaSuccess && ms) e = cudaEventElapsedTime(ms, ev[0], ev[1]);
  unsigned int st = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&st, status.p, 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(out, d.p, size_t(n) * 4, cudaMemcpyDeviceToHost);
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  d.release();
  status.release();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "lrt_proposal_infer");
  if (st) return fail(ctx, LRT_ERR_TIMEOUT, "tensor-core wait timed out");
  return LRT_OK;
}

extern "C" lrt_status lrt_proposal_infer(lrt_ctx *ctx, uint64_t first, uint64_t n, float *out) {
  return lrt_proposal_infer_ex(ctx, first, n, out, LRT_MLP_ENGINE_MMA, nullptr);
}

extern "C" lrt_status lrt_proposal_stats(lrt_ctx *ctx, unsigned long long out[4]) {
  if (!ctx || !out) return LRT_ERR_INVALID;
  if (!ctx->prop) {
    out[0] = out[1] = out[2] = out[3] = 0;
    return LRT_OK;
  }
  LRT_CUDA(ctx, cudaSetDevice(ctx->device));
  unsigned long long h[4];
  LRT_CUDA(ctx, cudaMemcpy(h, ctx->prop->stats.p, 32, cudaMemcpyDeviceToHost));
  LRT_CUDA(ctx, cudaMemset(ctx->prop->stats.p, 0, 32));
  out[0] = h[0];
  out[1] = h[1];
  out[2] = h[2];
  out[3] = h[3];
  return LRT_OK;
}
