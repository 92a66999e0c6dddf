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
#include "render_kernel.cuh"
#include "render_lq.cuh"

namespace lrt {
namespace dev {

// Persistent render kernel with per-lane ray refill: a lane whose ray has
// finished takes the next ray of the global ray sequence (ray r = lane r % 32 of
// tile r / 32, so consecutive rays stay neighbours) as soon as `refill` lanes of
// its warp are idle, instead of waiting for the whole warp's tile.  Each ray is
// traced exactly as by render_kernel (spp 1), so results are identical; only
// the assignment of rays to lanes changes.
template <int TYPE, int MODE, int STACK>
__global__ void __launch_bounds__(128, 5) render_refill_kernel(DevScene s, RenderLaunch L, uint32_t refill) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint64_t total = uint64_t(L.total_tiles) * 32u;
  Counters cnt = {0, 0, 0, 0};
  bool live = false, exhausted = false;
  uint32_t pix_out = 0;
  float3 dir = f3(0, 0, 1), org = f3(0, 0, 0), rp = f3(0, 0, 0), rd = f3(0, 0, 1), inv = f3(0, 0, 0);
  Hit hit;
  hit.t = 1e9f; hit.prim = kMiss; hit.geom = kMiss; hit.c0 = 1.0f; hit.c1 = hit.c2 = hit.c3 = 0.0f;
  uint2 st[STACK];
  int sp = 0;
  const float tNearSdf = 0.1f;
  for (;;) {
    const unsigned idle = __ballot_sync(0xffffffffu, !live);
    if (!exhausted && __popc(idle) >= int(refill)) {
      uint32_t base = 0;
      if (lane == 0) base = atomicAdd(L.tile_counter, uint32_t(__popc(idle)));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (uint64_t(base) + __popc(idle) >= total) exhausted = true;
      if (!live) {
        const uint64_t r = uint64_t(base) + __popc(idle & ((1u << lane) - 1u));
        if (r < total) {
          const uint32_t tile = uint32_t(r >> 5), tl = uint32_t(r & 31u);
          uint32_t v = 0;
          while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
          const DevView &V = L.views[v];
          const uint32_t lt = tile - V.tile_offset, lw = V.tile_w_log2;
          const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (tl & ((1u << lw) - 1u));
          const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (tl >> lw);
          if (x < V.width && y < V.height) {
            float3 pos;
            eye_ray(x, y, V.width, V.height, 0.5f, 0.5f, V.proj_inv, V.wv_inv, pos, dir);
            org = pos;
            pix_out = V.pix_offset + y * V.width + x;
            hit.t = 1e9f; hit.prim = kMiss; hit.geom = kMiss; hit.c0 = 1.0f; hit.c1 = hit.c2 = hit.c3 = 0.0f;
            live = true;
            sp = 0;
            const float3 invw = safe_inverse(dir);   // TLAS leaf box of the single instance
            const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                                      s.inst_bmax[1], s.inst_bmax[2]);
            if ((bh.x <= bh.y) && (bh.y > 0.0f) && (bh.x < hit.t)) {
              rp = matmul4x3(s.inst_inv, pos);
              rd = matmul3x3(s.inst_inv, dir);
              inv = safe_inverse(rd);
              st[0] = make_uint2(0u, __float_as_uint(-3.4e38f));
              sp = 1;
            }
          }
        }
      }
    }
    if (exhausted && !__any_sync(0xffffffffu, live)) break;
    uint32_t leaf = 0;
    bool have_leaf = false;
    if (live) {
      while (sp > 0) {
        sp--;
        const uint2 top = st[sp];
        const uint32_t ref = top.x;
        if (__uint_as_float(top.y) > hit.t) continue;
        if (ref & kLeafBit) {
          leaf = ref & ~kLeafBit;
          have_leaf = true;
          break;
        }
        visit_node<false, STACK>(s, ref, rp, inv, 0.0f, hit.t, st, sp, cnt);
      }
    }
    if (have_leaf) {
      if (TYPE == LRT_TYPE_MESH_TRIANGLE)
        tri_intersect<false>(s, rp, rd, tNearSdf, leaf & 0x00FFFFFFu, (leaf >> 24) & 0x7Fu, hit, cnt);
      else if (TYPE == LRT_TYPE_SDF_SVS)
        svs_intersect<false, MODE>(s, rp, rd, tNearSdf, leaf, hit, cnt);
      else
        brick_intersect<false, false, MODE>(s, rp, rd, inv, tNearSdf, leaf, hit, cnt);
    } else if (live) {   // stack empty: the ray is done
      if (L.hits16) {
        lrt_hit16 o;
        o.t = hit.t;
        o.primId = (hit.prim != kMiss && (hit.geom >> 24) == LRT_TYPE_MESH_TRIANGLE) ? s.prim_indices[hit.prim]
                                                                                    : hit.prim;
        o.nx = hit.c2;
        o.ny = hit.c3;
        reinterpret_cast<float4 *>(L.hits16)[pix_out] = *reinterpret_cast<const float4 *>(&o);
      }
      if (L.rgba || L.rgba8) {
        const float4 c = shade(s, hit, org, dir);
        if (L.rgba) L.rgba[pix_out] = c;
        if (L.rgba8) L.rgba8[pix_out] = encode_rgba8(c);
      }
      live = false;
    }
  }
}

}  // namespace dev

template <int TYPE, bool COUNT, int MODE, int STACK>
static cudaError_t launch_render_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_kernel<TYPE, COUNT, MODE, STACK, 0>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, COUNT, MODE, STACK, 0><<<blocks, 128, 0, st>>>(s, L);
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

template <int TYPE, int MODE, int STACK>
static cudaError_t launch_refill_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   uint32_t refill) {
  int per_sm = 0;
  cudaError_t e =
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_refill_kernel<TYPE, MODE, STACK>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_refill_kernel<TYPE, MODE, STACK><<<blocks, 128, 0, st>>>(s, L, refill);
  return cudaGetLastError();
}

// the refill kernel for the SBS and triangle configurations (spp 1)
static cudaError_t launch_refill(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                 const Tuning &tu) {
  const uint32_t refill = uint32_t(tu.refill < 1 ? 1 : (tu.refill > 32 ? 32 : tu.refill));
  if (s.type == LRT_TYPE_MESH_TRIANGLE)
    return launch_refill_m<LRT_TYPE_MESH_TRIANGLE, -1, kStackSize>(s, L, num_sms, st, refill);
  if (tu.stack == 32)
    return launch_refill_m<LRT_TYPE_SDF_SBS, LRT_INTERSECT_NEWTON, 32>(s, L, num_sms, st, refill);
  return launch_refill_m<LRT_TYPE_SDF_SBS, LRT_INTERSECT_NEWTON, kStackSize>(s, L, num_sms, st, refill);
}

// Kernels with the less common features, variant 0 and no counters (the counters of
// these renders stay zero): PHONG / PHONG_NO_TEX with colour outputs, whose shading
// traces shadow rays, and smoothed SDF normals (NORMAL_MODE_SDF_SMOOTHED on the
// neighbour layout).  Separate instantiations keep both out of the other kernels.
template <int TYPE, int MODE, bool PHONG, int FEAT>
static cudaError_t launch_feature_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, dev::render_kernel<TYPE, false, MODE, kStackSize, 0, PHONG, FEAT>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_kernel<TYPE, false, MODE, kStackSize, 0, PHONG, FEAT><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

template <int TYPE, bool PHONG, int FEAT>
static cudaError_t launch_feature_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  if (TYPE == LRT_TYPE_MESH_TRIANGLE) return launch_feature_m<TYPE, -1, PHONG, 0>(s, L, num_sms, st);
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON: return launch_feature_m<TYPE, LRT_INTERSECT_NEWTON, PHONG, FEAT>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_feature_m<TYPE, LRT_INTERSECT_ST, PHONG, FEAT>(s, L, num_sms, st);
    default: return launch_feature_m<TYPE, -1, PHONG, FEAT>(s, L, num_sms, st);
  }
}

template <int TYPE>
static cudaError_t launch_phong_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  return launch_feature_t<TYPE, true, 0>(s, L, num_sms, st);
}

template <int MODE, int STACK>
static cudaError_t launch_lq_m0(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_lq_kernel<MODE, STACK, 0>,
                                                                dev::kLqThreads, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_lq_kernel<MODE, STACK, 0><<<blocks, dev::kLqThreads, 0, st>>>(s, L);
  return cudaGetLastError();
}

// variant 3: traversal and leaf phases regrouped across the block (render_lq.cuh)
cudaError_t launch_render_lq(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                              const Tuning &tu) {
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON:
      if (tu.stack == 32) return launch_lq_m0<LRT_INTERSECT_NEWTON, 32>(s, L, num_sms, st);
      return launch_lq_m0<LRT_INTERSECT_NEWTON, kStackSize>(s, L, num_sms, st);
    case LRT_INTERSECT_ST: return launch_lq_m0<LRT_INTERSECT_ST, kStackSize>(s, L, num_sms, st);
    default: return launch_lq_m0<-1, kStackSize>(s, L, num_sms, st);
  }
}

// The kernel launch_render runs, decided from the scene, the outputs and the tuning.
enum class RenderChoice { kInstances, kFeature1, kFeature2, kPhong, kPacket, kRefill, kLeafQueue, kFused, kPlain };

static RenderChoice render_choice(const DevScene &s, bool color, uint32_t total_tiles, bool count, const Tuning &tu) {
  if (s.n_inst > 1) return RenderChoice::kInstances;
  const uint32_t rm = s.preset.render_mode;
  const bool phong = (rm == LRT_RENDER_MODE_PHONG || rm == LRT_RENDER_MODE_PHONG_NO_TEX) && color;
  switch (render_features(s)) {   // SBS only; smoothed normals need a normal mode, so never with ST_ITERATIONS
    case 1: return RenderChoice::kFeature1;
    case 2: return RenderChoice::kFeature2;
    default: break;
  }
  if (phong) return RenderChoice::kPhong;
  const bool sbs = s.type == LRT_TYPE_SDF_SBS || s.type == LRT_TYPE_SDF_SBS_COL || s.type == LRT_TYPE_SDF_SBS_TEX;
  if (sbs && tu.variant == 1) return RenderChoice::kPacket;
  const bool refill_ok = (s.type == LRT_TYPE_MESH_TRIANGLE ||
                          (s.type == LRT_TYPE_SDF_SBS && s.preset.sdf_node_intersect == LRT_INTERSECT_NEWTON)) &&
                         s.preset.spp <= 1 && !count && uint64_t(total_tiles) * 32u < (1ull << 31);
  if (tu.variant == 2 && refill_ok) return RenderChoice::kRefill;
  if (tu.variant == 3 && sbs && render_features(s) == 0 && s.preset.spp <= 1 && !count) return RenderChoice::kLeafQueue;
  // contraction only for the SDF leaves: in the triangle test it would open cracks along shared edges
  if (tu.fma && !count && tu.variant != 1 && s.type != LRT_TYPE_MESH_TRIANGLE) return RenderChoice::kFused;
  return RenderChoice::kPlain;
}

bool render_publishes_chunks(const DevScene &s, bool color, uint32_t total_tiles, const Tuning &tu) {
  const RenderChoice c = render_choice(s, color, total_tiles, false, tu);
  return c != RenderChoice::kPacket && c != RenderChoice::kRefill && c != RenderChoice::kLeafQueue;
}

cudaError_t launch_render(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                          const Tuning &tu) {
  const bool color = L.rgba || L.rgba8;
  switch (render_choice(s, color, L.total_tiles, count, tu)) {
    case RenderChoice::kInstances: return launch_render_inst(s, L, num_sms, st, false);
    case RenderChoice::kFeature1: {
      const uint32_t rm = s.preset.render_mode;
      const bool phong = (rm == LRT_RENDER_MODE_PHONG || rm == LRT_RENDER_MODE_PHONG_NO_TEX) && color;
      return phong ? launch_feature_t<LRT_TYPE_SDF_SBS, true, 1>(s, L, num_sms, st)
                   : launch_feature_t<LRT_TYPE_SDF_SBS, false, 1>(s, L, num_sms, st);
    }
    case RenderChoice::kFeature2: return launch_feature_t<LRT_TYPE_SDF_SBS, false, 2>(s, L, num_sms, st);
    case RenderChoice::kPhong:
      switch (s.type) {
        case LRT_TYPE_MESH_TRIANGLE: return launch_phong_t<LRT_TYPE_MESH_TRIANGLE>(s, L, num_sms, st);
        case LRT_TYPE_SDF_SVS: return launch_phong_t<LRT_TYPE_SDF_SVS>(s, L, num_sms, st);
        default: return launch_phong_t<LRT_TYPE_SDF_SBS>(s, L, num_sms, st);
      }
    case RenderChoice::kPacket: return launch_render_packet(s, L, num_sms, st, count, tu);
    case RenderChoice::kRefill: return launch_refill(s, L, num_sms, st, tu);
    case RenderChoice::kLeafQueue:
      return tu.fma ? launch_render_lq_fused(s, L, num_sms, st, tu) : launch_render_lq(s, L, num_sms, st, tu);
    case RenderChoice::kFused: return launch_render_fused(s, L, num_sms, st, tu);
    case RenderChoice::kPlain: break;
  }
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: return launch_render_t<LRT_TYPE_MESH_TRIANGLE>(s, L, num_sms, st, count, tu);
    case LRT_TYPE_SDF_SVS: return launch_render_t<LRT_TYPE_SDF_SVS>(s, L, num_sms, st, count, tu);
    default: return launch_render_t<LRT_TYPE_SDF_SBS>(s, L, num_sms, st, count, tu);
  }
}

cudaError_t launch_query(const DevScene &s, const float4 *pos_near, const float4 *dir_far, uint32_t n, lrt_hit *out,
                         cudaStream_t st) {
  if (s.n_inst > 1) return launch_query_inst(s, pos_near, dir_far, n, out, st, false);
  if (n == 0) return cudaSuccess;
  const uint32_t blocks = (n + 127) / 128;
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: dev::query_kernel<LRT_TYPE_MESH_TRIANGLE><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
    case LRT_TYPE_SDF_SVS: dev::query_kernel<LRT_TYPE_SDF_SVS><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
    default:
      switch (render_features(s)) {
        case 1: dev::query_kernel<LRT_TYPE_SDF_SBS, 1><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
        case 2: dev::query_kernel<LRT_TYPE_SDF_SBS, 2><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
        default: dev::query_kernel<LRT_TYPE_SDF_SBS><<<blocks, 128, 0, st>>>(s, pos_near, dir_far, n, out); break;
      }
      break;
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
#include <cstring>
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

// The view table travels as a kernel argument (10 KB, inside the 32 KB argument
// limit) and this kernel writes it into the scratch array and clears the queue
// head: no host buffer has to outlive the call, pageable or not.
struct NoAllocViews {
  DevView v[LRT_NOALLOC_MAX_VIEWS];
};
static_assert(sizeof(NoAllocViews) <= 30000, "view table must fit the kernel argument space");

__global__ void __launch_bounds__(256) noalloc_setup_kernel(const __grid_constant__ NoAllocViews tab, uint32_t n_views,
                                                            DevView *views, uint32_t *head) {
  const uint32_t words = n_views * uint32_t(sizeof(DevView) / sizeof(uint32_t));
  const uint32_t *src = reinterpret_cast<const uint32_t *>(tab.v);
  uint32_t *dst = reinterpret_cast<uint32_t *>(views);
  for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
  if (threadIdx.x == 0) *head = 0u;
}
}  // namespace

cudaError_t launch_render_noalloc(const DevScene &s, const DevView *host_views, uint32_t n_views,
                                  uint32_t total_tiles, lrt_hit16 *hits16, float4 *rgba, uint32_t *rgba8,
                                  int device, int num_sms, cudaStream_t st, const Tuning &tu, bool first_hit) {
  if (n_views == 0 || n_views > LRT_NOALLOC_MAX_VIEWS) return cudaErrorInvalidValue;
  unsigned char *scratch = nullptr;
  cudaError_t e = noalloc_scratch(device, &scratch);
  if (e != cudaSuccess) return e;
  uint32_t *head = reinterpret_cast<uint32_t *>(scratch);
  DevView *views = reinterpret_cast<DevView *>(scratch + kNoAllocViewOffset);
  // The array keeps the previous call's contents: the view table is rewritten and
  // the queue head cleared on every call, by a kernel on the caller's stream.
  NoAllocViews tab;
  std::memcpy(tab.v, host_views, n_views * sizeof(DevView));
  noalloc_setup_kernel<<<1, 256, 0, st>>>(tab, n_views, views, head);
  e = cudaGetLastError();
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
  return first_hit ? launch_render_ref(s, L, num_sms, st) : launch_render(s, L, num_sms, st, false, tu);
}

}  // namespace lrt
