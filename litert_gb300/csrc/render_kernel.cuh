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

// PHONG / PHONG_NO_TEX shading (Renderer/eye_ray.cpp:420-483) with the default
// lights: the direct light adds an unshadowed Lambert term and a shadowed Phong
// term (Kd = Ks = 0.25, exponent 32); ambient adds its colour.  The reference's
// shadow ray is a nearest-hit query from just before the hit point towards the
// light with the eye ray's tNear and tFar; only hit / miss is used, so an any-hit
// query (the first leaf that reports a hit) decides the same.
// MI: the scene has several instances (the shadow ray tests them all).
template <int TYPE, int MODE, int STACK, int MI = 0>
__device__ __noinline__ float4 shade_phong(const DevScene &s, const Hit &hit, float3 pos, float3 dir) {
  if (hit.prim == kMiss) return make_float4(0, 0, 0, 1);
  const uint32_t type = hit.geom >> 24;
  float3 norm;
  if (type == LRT_TYPE_MESH_TRIANGLE) {
    const float4 a = s.tri_verts[3 * hit.prim + 0], b = s.tri_verts[3 * hit.prim + 1], c = s.tri_verts[3 * hit.prim + 2];
    const float3 e1 = f3(b.x - a.x, b.y - a.y, b.z - a.z), e2 = f3(c.x - a.x, c.y - a.y, c.z - a.z);
    norm = normalize(matmul4x3(s.inst_inv_t, cross(e1, e2)));
  } else {
    norm = decode_normal(hit.c2, hit.c3);
  }
  norm = scl(signf(dot(scl(-1.0f, dir), norm)), norm);
  const float Kd = 0.25f, Ks = 0.25f, BIAS = 1e-6f;
  float3 color = s.preset.render_mode == LRT_RENDER_MODE_PHONG_NO_TEX ? f3(1, 1, 1) : f3(0, 1, 1);
  if (s.preset.render_mode == LRT_RENDER_MODE_PHONG && type == LRT_TYPE_SDF_SBS_COL) {
    color.x = roundf(hit.c0) / 255.0f;
    color.y = hit.c0 - floorf(hit.c0);
    color.z = roundf(hit.c1) / 255.0f;
  }
  float3 fc = f3(0, 0, 0);
  {  // direct light, normalize(1, 1, 1), colour 2/3
    const float3 ld = normalize(f3(1, 1, 1));
    const float l = 2.0f / 3.0f;
    const float3 lc = f3(l, l, l);
    const float3 surf = add(pos, scl(hit.t - BIAS, dir));
    const float q = mx(0.0f, dot(norm, ld));
    fc = add(fc, scl(q, mul(lc, color)));
    Hit sh;
    Counters cnt = {0, 0, 0, 0};
    trace<TYPE, false, MODE, STACK, MI>(s, surf, 0.0f, ld, -1e9f, sh, cnt);   // tFar <= 0: any hit
    const float shade = (sh.prim == kMiss) ? 1.0f : 0.0f;
    const float3 refl = add(scl(-1.0f, ld), scl(2.0f * dot(norm, ld), norm));
    const float inner = Kd * mx(0.0f, dot(norm, ld)) + Ks * powf(mx(0.0f, dot(norm, refl)), 32.0f);
    fc = add(fc, mul(scl(inner, scl(shade, lc)), color));
  }
  fc = add(fc, mul(f3(0.25f, 0.25f, 0.25f), color));   // ambient
  return make_float4(fc.x, fc.y, fc.z, 1);
}

// Persistent render kernel: each warp pulls 32-pixel tiles (8x4 by default, the
// shape is tunable) of the flattened multi-view tile space from a global queue
// head and traces one ray per lane.  With L.chunk_done set, a warp adds its
// finished tiles to their output chunk's count, with every lane's stores fenced
// first, when it moves on to a tile of another chunk and when it ends (tiles are
// handed out in order, so a warp fences about once per chunk): a copy of a
// chunk can start while later tiles render.
__device__ __forceinline__ void publish_tiles(uint32_t *chunk_done, uint32_t chunk, uint32_t tiles, uint32_t lane) {
  asm volatile("fence.acq_rel.gpu;" ::: "memory");   // this lane's stores before what follows, device-wide
  __syncwarp();                                       // every lane's fence (the warp is converged here)
  if (lane == 0) atomicAdd(&chunk_done[chunk], tiles);
}

template <int TYPE, bool COUNT, int MODE, int STACK, int FP, bool PHONG = false, int FEAT = 0>
__global__ void __launch_bounds__(128, 5) render_kernel(DevScene s, RenderLaunch L) {
  const uint32_t lane = threadIdx.x & 31u;
  Counters cnt = {0, 0, 0, 0};
  const uint32_t spp = s.preset.spp ? s.preset.spp : 1u;
  const uint32_t spp_sqrt = uint32_t(sqrtf(float(spp)));
  const float i_spp_sqrt = 1.0f / float(spp_sqrt);
  uint32_t chunk = 0, pending = 0;   // finished tiles of output chunk `chunk` not yet counted
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(L.tile_counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= L.total_tiles) {
      if (L.chunk_done && pending) publish_tiles(L.chunk_done, chunk, pending, lane);
      break;
    }
    uint32_t v = 0;
    while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
    const DevView &V = L.views[v];
    const uint32_t lt = tile - V.tile_offset, lw = V.tile_w_log2;
    if (L.chunk_done) {   // the same for the whole grid
      const uint32_t c = V.chunk_offset + lt / (V.tiles_x * V.rows_per_chunk);   // floor(floor(a/b)/c) = floor(a/(bc))
      if (pending && c != chunk) {
        publish_tiles(L.chunk_done, chunk, pending, lane);
        pending = 0;
      }
      chunk = c;
      pending++;
    }
    const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (lane & ((1u << lw) - 1u));
    const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (lane >> lw);
    if (x >= V.width || y >= V.height) continue;   // all lanes meet again at the queue shuffle
    float4 acc = make_float4(0, 0, 0, 0);
    Hit first;
    for (uint32_t si = 0; si < spp; si++) {
      // sub-pixel offset, CastRaySingle (Renderer/eye_ray.cpp:100-107): the regular
      // grid, or rand2(x, y, i + m_seed % 2) for RAY_GEN_MODE_RANDOM
      float dx, dy;
      if (s.preset.ray_gen_mode == 1) {
        const float2 r = rand2(x, y, si + s.seed % 2u, s.seed);
        dx = r.x;
        dy = r.y;
      } else {
        dx = i_spp_sqrt * float(double(si / spp_sqrt) + 0.5);
        dy = i_spp_sqrt * float(double(si % spp_sqrt) + 0.5);
      }
      float3 pos, dir;
      eye_ray(x, y, V.width, V.height, dx, dy, V.proj_inv, V.wv_inv, pos, dir);
      Hit hit;
      // the contracted kernels (FP = 1) also test inner-node slabs with one FMA per plane
      trace<TYPE, COUNT, MODE, STACK, FEAT | (FP == 1 ? 16 : 0)>(s, pos, 0.0f, dir, 1e9f, hit, cnt);
      if (FEAT & 8) {   // colours and shading in the frame of the instance hit
        const DevScene sh = scene_of_instance(s, hit.prim != kMiss ? hit.inst : 0u);
        if (TYPE == LRT_TYPE_SDF_SBS && !(FEAT & 2)) hit_colour(sh, pos, dir, hit);
        if (L.rgba || L.rgba8) {
          const float4 c = PHONG ? shade_phong<TYPE, MODE, STACK, 8>(sh, hit, pos, dir) : shade(sh, hit, pos, dir);
          acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
        }
      } else {
        if (TYPE == LRT_TYPE_SDF_SBS && !(FEAT & 2)) hit_colour(s, pos, dir, hit);
        if (L.rgba || L.rgba8) {
          const float4 c = PHONG ? shade_phong<TYPE, MODE, STACK>(s, hit, pos, dir) : shade(s, hit, pos, dir);
          acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
        }
      }
      if (si == 0) first = hit;
    }
    const size_t pix = size_t(V.pix_offset) + size_t(y) * V.width + x;
    const bool direct = pix >= L.direct_from;
    if (L.hits16) {
      lrt_hit16 o;
      o.t = first.t;
      o.primId = (first.prim != kMiss && (first.geom >> 24) == LRT_TYPE_MESH_TRIANGLE) ? s.prim_indices[first.prim]
                                                                                        : first.prim;
      o.nx = first.c2;
      o.ny = first.c3;
      // outputs are written once and not read again here: evict-first stores keep
      // the tree and the bricks in L2
      __stcs(reinterpret_cast<float4 *>(direct ? L.hits16_direct : L.hits16) + pix, *reinterpret_cast<const float4 *>(&o));
    }
    const float fs = float(spp);
    const float4 col = make_float4(acc.x / fs, acc.y / fs, acc.z / fs, acc.w / fs);
    if (L.rgba) __stcs((direct ? L.rgba_direct : L.rgba) + pix, col);
    if (L.rgba8) __stcs((direct ? L.rgba8_direct : L.rgba8) + pix, encode_rgba8(col));
  }
  if (COUNT) {
    atomicAdd(&L.counters[0], (unsigned long long)cnt.nodes);
    atomicAdd(&L.counters[1], (unsigned long long)cnt.leaves);
    atomicAdd(&L.counters[2], (unsigned long long)cnt.voxels);
    atomicAdd(&L.counters[3], (unsigned long long)cnt.finder);
  }
}

// Batched RayQuery_NearestHit: one thread per ray, full CRT_Hit output.
template <int TYPE, int FEAT = 0>
__global__ void __launch_bounds__(128) query_kernel(DevScene s, const float4 *pos_near, const float4 *dir_far,
                                                   uint32_t n, lrt_hit *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos_near[i], d = dir_far[i];
  Counters cnt = {0, 0, 0, 0};
  Hit hit;
  trace<TYPE, false, -1, kStackSize, FEAT>(s, f3(p.x, p.y, p.z), p.w, f3(d.x, d.y, d.z), d.w, hit, cnt);
  if (TYPE == LRT_TYPE_SDF_SBS && !(FEAT & 2)) {
    if (FEAT & 8)
      hit_colour(scene_of_instance(s, hit.prim != kMiss ? hit.inst : 0u), f3(p.x, p.y, p.z), f3(d.x, d.y, d.z), hit);
    else
      hit_colour(s, f3(p.x, p.y, p.z), f3(d.x, d.y, d.z), hit);
  }
  lrt_hit o;
  o.t = hit.t;
  o.primId = (hit.prim != kMiss && (hit.geom >> 24) == LRT_TYPE_MESH_TRIANGLE) ? s.prim_indices[hit.prim] : hit.prim;
  o.instId = hit.prim == kMiss ? kMiss : ((FEAT & 8) ? hit.inst : 0u);
  o.geomId = hit.geom;
  o.coords[0] = hit.c0;
  o.coords[1] = hit.c1;
  o.coords[2] = hit.c2;
  o.coords[3] = hit.c3;
  out[i] = o;
}

}  // namespace dev
}  // namespace lrt
