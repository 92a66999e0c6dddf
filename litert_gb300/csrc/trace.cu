// Primary-ray kernels for sm_103a: BVH traversal with SBS-brick, SVS-voxel and
// triangle leaves (the hot path of BVHRT::RayQuery_NearestHit,
// BVH/BVH2Common.cpp:3407-3559) plus eye-ray generation and shading
// (MultiRenderer::CastRaySingle / kernel_RayTrace, Renderer/eye_ray.cpp:83-489).
//
// Traversal returns the closest hit: the reference stops at the first SDF leaf
// that reports a hit (BVH/BVH2Common.cpp:3402-3405), which is the closest one
// except where sibling boxes overlap; the closest hit does not depend on the BVH
// topology, so the GPU may use its own 4-wide tree.  Leaf tests use the leaf box
// and the reference's slab arithmetic exactly, internal boxes enclose their leaf
// boxes, so culling never removes a leaf the reference would have entered.
#include "traverse.cuh"

namespace lrt {
namespace dev {

// Persistent render kernel: each warp pulls 32-pixel tiles (8x4 by default, the
// shape is tunable) of the flattened multi-view tile space from a global queue
// head and traces one ray per lane.
template <int TYPE, bool COUNT, int MODE, int STACK>
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

// Batched RayQuery_NearestHit: one thread per ray, full CRT_Hit output.
template <int TYPE>
__global__ void __launch_bounds__(128) query_kernel(DevScene s, const float4 *pos_near, const float4 *dir_far,
                                                   uint32_t n, lrt_hit *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 p = pos_near[i], d = dir_far[i];
  Counters cnt = {0, 0, 0, 0};
  Hit hit;
  trace<TYPE, false>(s, f3(p.x, p.y, p.z), p.w, f3(d.x, d.y, d.z), d.w, hit, cnt);
  lrt_hit o;
  o.t = hit.t;
  o.primId = (hit.prim != kMiss && (hit.geom >> 24) == LRT_TYPE_MESH_TRIANGLE) ? s.prim_indices[hit.prim] : hit.prim;
  o.instId = hit.prim == kMiss ? kMiss : 0u;
  o.geomId = hit.geom;
  o.coords[0] = hit.c0;
  o.coords[1] = hit.c1;
  o.coords[2] = hit.c2;
  o.coords[3] = hit.c3;
  out[i] = o;
}

}  // namespace dev

template <int TYPE, bool COUNT, int MODE, int STACK>
static cudaError_t launch_render_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_kernel<TYPE, COUNT, MODE, STACK>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, COUNT, MODE, STACK><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

template <int TYPE, bool COUNT>
static cudaError_t launch_render_c(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   const Tuning &tu) {
  if (TYPE == LRT_TYPE_MESH_TRIANGLE) return launch_render_m<TYPE, COUNT, -1, kStackSize>(s, L, num_sms, st);
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON:
      // the headline configuration also comes with a 32-entry stack for shallow trees
      if (TYPE == LRT_TYPE_SDF_SBS && !COUNT && tu.stack == 32)
        return launch_render_m<TYPE, COUNT, LRT_INTERSECT_NEWTON, 32>(s, L, num_sms, st);
      return launch_render_m<TYPE, COUNT, LRT_INTERSECT_NEWTON, kStackSize>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_render_m<TYPE, COUNT, LRT_INTERSECT_ST, kStackSize>(s, L, num_sms, st);
    default: return launch_render_m<TYPE, COUNT, -1, kStackSize>(s, L, num_sms, st);
  }
}

template <int TYPE>
static cudaError_t launch_render_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                                   const Tuning &tu) {
  return count ? launch_render_c<TYPE, true>(s, L, num_sms, st, tu) : launch_render_c<TYPE, false>(s, L, num_sms, st, tu);
}

cudaError_t launch_render(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                          const Tuning &tu) {
  const bool sbs = s.type == LRT_TYPE_SDF_SBS || s.type == LRT_TYPE_SDF_SBS_COL;
  if (sbs && tu.variant == 1) return launch_render_packet(s, L, num_sms, st, count, tu);
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: return launch_render_t<LRT_TYPE_MESH_TRIANGLE>(s, L, num_sms, st, count, tu);
    case LRT_TYPE_SDF_SVS: return launch_render_t<LRT_TYPE_SDF_SVS>(s, L, num_sms, st, count, tu);
    default: return launch_render_t<LRT_TYPE_SDF_SBS>(s, L, num_sms, st, count, tu);
  }
}

cudaError_t launch_query(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n, lrt_hit *out,
                         cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint32_t blocks = (n + 127) / 128;
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: dev::query_kernel<LRT_TYPE_MESH_TRIANGLE><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
    case LRT_TYPE_SDF_SVS: dev::query_kernel<LRT_TYPE_SDF_SVS><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
    default: dev::query_kernel<LRT_TYPE_SDF_SBS><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
  }
  return cudaGetLastError();
}

}  // namespace lrt

// ---------------------------------------------------------------- rendering without allocation
// Scratch of lrt_render_noalloc: the persistent kernel's work-queue head and the
// per-view table live in this file-scope device array instead of context
// buffers, so that entry point allocates nothing.  Every GPU that loads the
// library holds the array until exit.  Host code must not pass the symbol
// itself to a kernel (on the host it is only a stand-in); the device address
// is looked up once per device with cudaGetSymbolAddress, with that device
// current, on the first call on that device.
#include <mutex>

namespace lrt {
namespace {
constexpr size_t kNoAllocViewOffset = 256;   // [0, 256): queue head; then the view table
constexpr size_t kNoAllocScratchBytes = kNoAllocViewOffset + size_t(LRT_NOALLOC_MAX_VIEWS) * sizeof(DevView);
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kNoAllocMaxDevices];   // device address of g_noalloc_scratch, per device

cudaError_t noalloc_scratch(int device, unsigned char **out) {
  if (device < 0 || device >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);   // `device` is current
    if (e != cudaSuccess) return e;
    g_noalloc_addr[device] = p;
  }
  *out = static_cast<unsigned char *>(g_noalloc_addr[device]);
  return cudaSuccess;
}
}  // namespace

cudaError_t launch_render_noalloc(const DevScene &s, const DevView *host_views, uint32_t n_views,
                                  uint32_t total_tiles, lrt_hit16 *hits16, float4 *rgba, uint32_t *rgba8,
                                  int device, int num_sms, cudaStream_t st, const Tuning &tu) {
  if (n_views == 0 || n_views > LRT_NOALLOC_MAX_VIEWS) return cudaErrorInvalidValue;
  unsigned char *scratch = nullptr;
  cudaError_t e = noalloc_scratch(device, &scratch);
  if (e != cudaSuccess) return e;
  uint32_t *head = reinterpret_cast<uint32_t *>(scratch);
  DevView *views = reinterpret_cast<DevView *>(scratch + kNoAllocViewOffset);
  // The array keeps the previous call's contents: the view table is rewritten and
  // the queue head cleared on every call.
  e = cudaMemcpyAsync(views, host_views, n_views * sizeof(DevView), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(head, 0, sizeof(uint32_t), st);
  if (e != cudaSuccess) return e;
  RenderLaunch L;
  L.views = views;
  L.n_views = n_views;
  L.total_tiles = total_tiles;
  L.hits16 = hits16;
  L.rgba = rgba;
  L.rgba8 = rgba8;
  L.tile_counter = head;
  L.counters = nullptr;
  return launch_render(s, L, num_sms, st, false, tu);
}

}  // namespace lrt
