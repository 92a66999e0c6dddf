// Compile-and-link check of the reference-side bindings
// (litert_gb300/ref_side/lrt_bvhrt_gpu.h, lrt_multirenderer_dr_gpu.h) against the
// reference's own headers (BVH/BVH2Common.h, Renderer/eye_ray.h,
// diff_render/MultiRendererDR.h) and the engine library: BVHRT_GPU must override
// every pure virtual of ISceneObject, MultiRendererGPU every member it replaces
// and MultiRendererDR_GPU must build as a dr::MultiRendererDR, or this program
// does not build.  Run, it constructs them; without a GPU the engine contexts
// fail cleanly ("no-device"), with one it renders a tiny sphere SBS through
// MultiRenderer::RenderFloat and runs two optimisation steps on a 2^3-brick grid.
#include <cstdio>

#include "BVH/BVH2Common.h"
#include "Renderer/eye_ray.h"
#include "diff_render/MultiRendererDR.h"
#include "lrt_bvhrt_gpu.h"
#include "lrt_multirenderer_dr_gpu.h"

static void dr_binding() {
  MultiRendererDR_GPU d(0);
  if (!d.ok()) {
    std::printf("no-device %s %s\n", d.Name(), d.last_error().c_str());
    return;
  }
  SdfSBS sbs = dr::create_grid_sbs(2, 4, [](float3 p) { return dr::circle_sdf(float3(0, 0, 0), 0.6f, p); },
                                   dr::single_color);
  std::vector<LiteImage::Image2D<float4>> ref(1, LiteImage::Image2D<float4>(16, 16, float4(0.5f, 0.5f, 0.5f, 1.0f)));
  d.SetReference(ref, {LiteMath::lookAt(float3(0, 0, 3), float3(0, 0, 0), float3(0, 1, 0))},
                 {LiteMath::perspectiveMatrix(60.0f, 1.0f, 0.01f, 100.0f)});
  dr::MultiRendererDRPreset p = dr::getDefaultPresetDR();
  p.opt_iterations = 2;
  d.OptimizeFixedStructure(p, sbs);
  std::printf("optimised %s %s\n", d.Name(), d.last_error().c_str());
}

int main() {
  MultiRendererGPU r(0);
  ISceneObject *as_scene = &r.gpu();
  if (!r.gpu().ok()) {
    std::printf("no-device %s %s\n", as_scene->Name(), r.gpu().last_error().c_str());
    dr_binding();
    return 0;
  }
  // 2x2x2 bricks of one voxel around a sphere, DX layout, 4-byte values
  SdfSBSHeader h{1, 0, 4, SDF_SBS_NODE_LAYOUT_DX};
  std::vector<SdfSBSNode> nodes;
  std::vector<uint32_t> values;
  for (uint32_t i = 0; i < 8; i++) {
    SdfSBSNode n{};
    n.pos_xy = ((i >> 2) << 16) | ((i >> 1) & 1u);
    n.pos_z_lod_size = ((i & 1u) << 16) | 2u;
    n.data_offset = uint32_t(values.size());
    for (int c = 0; c < 8; c++) values.push_back(c == 7 - int(i) ? 0x40000000u : 0xC0000000u);
    nodes.push_back(n);
  }
  SdfSBSView v(h, nodes, values);
  r.SetScene(v);
  std::vector<LiteMath::float4> img(32 * 32);
  r.RenderFloat(img.data(), 32, 32, LiteMath::lookAt(LiteMath::float3(0, 0, 3), LiteMath::float3(0, 0, 0),
                                                     LiteMath::float3(0, 1, 0)),
                LiteMath::perspectiveMatrix(60.0f, 1.0f, 0.01f, 100.0f), getDefaultPreset(), 1);
  std::printf("rendered %s %s\n", as_scene->Name(), r.gpu().last_error().c_str());
  dr_binding();
  return 0;
}
