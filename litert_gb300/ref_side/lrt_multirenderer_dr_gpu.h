// The reference-side binding of the lrt differentiable renderer: what a LiteRT
// maintainer adds to the reference tree to run MultiRendererDR's optimisation
// (diff_render/MultiRendererDR.h:71-155) on this engine.
//
//   MultiRendererDR_GPU  a dr::MultiRendererDR whose SetReference,
//                        OptimizeFixedStructure, getLastImage and getLastdLoss_dS
//                        run the optimisation through include/lrt_dr.h: the
//                        indexed SBS, the reference images and their cameras go
//                        to the device once, every iteration (forward, adjoint,
//                        border integral, Adam) runs there, and the optimised
//                        values_f come back into the caller's SdfSBS (the
//                        reference writes them there too,
//                        diff_render/MultiRendererDR.cpp:575).
//
// These members are not virtual in the reference, so the binding is used through
// its own type; code holding the object as a MultiRenderer keeps the base's
// rendering.  The renderer's seed (setSeed) and lights (SetLights: direct and
// ambient; the reference's DR has no point-light derivative) carry over.
//
// Header-only: include it after the reference's diff_render/MultiRendererDR.h and
// link liblrt_gb300.so.  Engine errors are kept in last_error() (the reference's
// interface has none: a failed optimisation leaves values_f as it was).
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "lrt_dr.h"
#include "lrt_gpu.h"

class MultiRendererDR_GPU : public dr::MultiRendererDR {
 public:
  explicit MultiRendererDR_GPU(int device = 0, uint32_t maxPrimitives = 10'000'000)
      : dr::MultiRendererDR(maxPrimitives) {
    if (lrt_create(&m_ctx, device) != LRT_OK) {
      m_ctx = nullptr;
      m_err = "lrt_create failed (no usable GPU)";
    }
  }
  ~MultiRendererDR_GPU() {
    if (m_ctx) lrt_destroy(m_ctx);
  }
  MultiRendererDR_GPU(const MultiRendererDR_GPU &) = delete;
  MultiRendererDR_GPU &operator=(const MultiRendererDR_GPU &) = delete;

  bool ok() const { return m_ctx != nullptr; }
  const std::string &last_error() const { return m_err; }
  const char *Name() const { return "MultiRendererDR_GPU"; }

  // SetReference (diff_render/MultiRendererDR.cpp:147-160): the target images and
  // their cameras, kept until the optimisation starts
  void SetReference(const std::vector<LiteImage::Image2D<LiteMath::float4>> &images,
                    const std::vector<LiteMath::float4x4> &worldView, const std::vector<LiteMath::float4x4> &proj) {
    m_views.clear();
    m_pixels.clear();
    for (size_t i = 0; i < images.size() && i < worldView.size() && i < proj.size(); i++) {
      lrt_view v;
      v.width = images[i].width();
      v.height = images[i].height();
      rows(worldView[i], v.world_view);
      rows(proj[i], v.proj);
      m_views.push_back(v);
      const float *px = reinterpret_cast<const float *>(images[i].data());
      m_pixels.insert(m_pixels.end(), px, px + 4 * size_t(v.width) * v.height);
    }
    m_worldViewRef = worldView;
    m_projRef = proj;
  }

  // OptimizeFixedStructure (:278-576): preset.opt_iterations Adam steps on sbs
  // (an indexed SBS, ID32F_IRGB32F(_IN)), its values_f updated in place
  void OptimizeFixedStructure(dr::MultiRendererDRPreset preset, SdfSBS &sbs) {
    if (!ok()) return;
    lrt_dr_preset p;
    lrt_dr_default_preset(&p);
    p.render_mode = preset.dr_render_mode;
    p.reconstruction_flags = preset.dr_reconstruction_flags;
    p.input_type = preset.dr_input_type;
    p.loss_function = preset.dr_loss_function;
    p.spp = preset.spp;
    p.border_spp = preset.border_spp;
    p.border_relax_eps = preset.border_relax_eps;
    p.border_sampling = preset.dr_border_sampling;
    p.raycasting_mask = preset.dr_raycasting_mask;
    p.opt_lr = preset.opt_lr;
    p.opt_beta_1 = preset.opt_beta_1;
    p.opt_beta_2 = preset.opt_beta_2;
    p.opt_eps = preset.opt_eps;
    p.reg_function = preset.reg_function;
    p.reg_lambda = preset.reg_lambda;
    p.reg_power = preset.reg_power;
    p.redistancing_enable = preset.redistancing_enable ? 1u : 0u;
    p.redistancing_interval = preset.redistancing_interval;
    p.seed = m_seed;
    p.n_lights = 0;
    for (const Light &l : m_lights) {
      if (p.n_lights == 4 || l.type == LIGHT_TYPE_POINT) {
        m_err = "MultiRendererDR_GPU: at most 4 direct/ambient lights";
        return;
      }
      lrt_dr_light &o = p.lights[p.n_lights++];
      o.type = l.type;
      o.dir[0] = l.space.x; o.dir[1] = l.space.y; o.dir[2] = l.space.z;
      o.color[0] = l.color.x; o.color[1] = l.color.y; o.color[2] = l.color.z;
    }
    const uint32_t n_params = uint32_t(sbs.values_f.size());
    if (!check(lrt_dr_set_preset(m_ctx, &p)) ||
        !check(lrt_dr_set_scene(m_ctx, reinterpret_cast<const lrt_sbs_header *>(&sbs.header),
                                reinterpret_cast<const lrt_sbs_node *>(sbs.nodes.data()),
                                uint32_t(sbs.nodes.size()), sbs.values.data(), sbs.values.size(),
                                sbs.values_f.data(), n_params, nullptr, 0)) ||
        !check(lrt_dr_set_reference(m_ctx, uint32_t(m_views.size()), m_views.data(), m_pixels.data())) ||
        !check(lrt_dr_optimize(m_ctx, 0, preset.opt_iterations, nullptr)))
      return;
    std::vector<float> params(n_params);
    if (!check(lrt_dr_get(m_ctx, LRT_DR_PARAMS, 0, params.data(), 4ull * n_params))) return;
    sbs.values_f = params;
    // what getLastImage / getLastdLoss_dS return afterwards
    m_images.resize(m_views.size());
    for (size_t i = 0; i < m_views.size(); i++) {
      m_images[i] = LiteImage::Image2D<LiteMath::float4>(m_views[i].width, m_views[i].height);
      check(lrt_dr_get(m_ctx, LRT_DR_IMAGE, uint32_t(i), m_images[i].data(),
                       16ull * m_views[i].width * m_views[i].height));
    }
    m_dLoss_dS_tmp.assign(n_params, 0.0f);
    check(lrt_dr_get(m_ctx, LRT_DR_GRAD, 0, m_dLoss_dS_tmp.data(), 4ull * n_params));
  }

  lrt_ctx *context() const { return m_ctx; }

 private:
  static void rows(const LiteMath::float4x4 &m, float a[16]) {
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) a[4 * i + j] = m(i, j);
  }
  bool check(lrt_status s) {
    if (s == LRT_OK) return true;
    m_err = lrt_last_error(m_ctx);
    return false;
  }
  lrt_ctx *m_ctx = nullptr;
  std::string m_err;
  std::vector<lrt_view> m_views;
  std::vector<float> m_pixels;
};
