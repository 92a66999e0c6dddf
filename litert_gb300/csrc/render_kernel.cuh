// The persistent primary-ray render kernel, shared by the translation units
// that instantiate it: trace.cu (compiled without floating-point contraction, so
// every a * b + c rounds twice as in the reference's x86-64 build: bit-exact
// parity) and trace_fused.cu (compiled with contraction: a * b + c becomes one
// FMA).  The FP template argument only tags which unit an instantiation belongs
// to, so the two sets of kernels have distinct symbols.
#pragma once
#include "traverse.cuh"

namespace lrt {
namespace dev {

// Persistent render kernel: each warp pulls 32-pixel tiles (8x4 by default, the
// shape is tunable) of the flattened multi-view tile space from a global queue
// head and traces one ray per lane.
template <int TYPE, bool COUNT, int MODE, int STACK, int FP>
__global__ void __launch_bounds__(128, 5) render_kernel(DevScene s, RenderLaunch L) {
  const uint32_t lane = threadIdx.x & 31u;
  Counters cnt = {0, 0, 0, 0};
  const uint32_t spp = s.preset.spp ? s.preset.spp : 1u;
  const uint32_t spp_sqrt = uint32_t(sqrtf(float(spp)));
  const float i_spp_sqrt = 1.0f / float(spp_sqrt);
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(L.tile_counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= L.total_tiles) break;
    uint32_t v = 0;
    while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
    const DevView &V = L.views[v];
    const uint32_t lt = tile - V.tile_offset, lw = V.tile_w_log2;
    const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (lane & ((1u << lw) - 1u));
    const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (lane >> lw);
    if (x >= V.width || y >= V.height) continue;   // all lanes meet again at the queue shuffle
    float4 acc = make_float4(0, 0, 0, 0);
    Hit first;
    for (uint32_t si = 0; si < spp; si++) {
      const float dx = i_spp_sqrt * float(double(si / spp_sqrt) + 0.5);
      const float dy = i_spp_sqrt * float(double(si % spp_sqrt) + 0.5);
      float3 pos, dir;
      eye_ray(x, y, V.width, V.height, dx, dy, V.proj_inv, V.wv_inv, pos, dir);
      Hit hit;
      trace<TYPE, COUNT, MODE, STACK>(s, pos, 0.0f, dir, 1e9f, hit, cnt);
      if (si == 0) first = hit;
      if (L.rgba || L.rgba8) {
        const float4 c = shade(s, hit, dir);
        acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
      }
    }
    const size_t pix = size_t(V.pix_offset) + size_t(y) * V.width + x;
    if (L.hits16) {
      lrt_hit16 o;
      o.t = first.t;
      o.primId = (first.prim != kMiss && (first.geom >> 24) == LRT_TYPE_MESH_TRIANGLE) ? s.prim_indices[first.prim]
                                                                                        : first.prim;
      o.nx = first.c2;
      o.ny = first.c3;
      reinterpret_cast<float4 *>(L.hits16)[pix] = *reinterpret_cast<const float4 *>(&o);
    }
    const float fs = float(spp);
    const float4 col = make_float4(acc.x / fs, acc.y / fs, acc.z / fs, acc.w / fs);
    if (L.rgba) L.rgba[pix] = col;
    if (L.rgba8) L.rgba8[pix] = encode_rgba8(col);
  }
  if (COUNT) {
    atomicAdd(&L.counters[0], (unsigned long long)cnt.nodes);
    atomicAdd(&L.counters[1], (unsigned long long)cnt.leaves);
    atomicAdd(&L.counters[2], (unsigned long long)cnt.voxels);
    atomicAdd(&L.counters[3], (unsigned long long)cnt.finder);
  }
}

}  // namespace dev
}  // namespace lrt
