// Warp-packet primary-ray kernel for SBS scenes (sm_103a).
//
// A warp owns an 8x4-pixel tile and walks the 4-wide BVH as one packet: the
// traversal stack lives in shared memory and is shared by the warp, so node
// fetches are warp-uniform broadcast loads and the traversal loop never
// diverges.  A stack entry holds the child reference, the mask of lanes whose
// rays enter the child box, and the smallest entry distance over those lanes
// (a warp reduction); popping skips the entry when no lane's current closest
// hit lies beyond that distance.  Leaf entries are re-tested per lane against
// the exact BVH leaf box, so a lane marches a brick exactly when the per-ray
// traversal would (tm.x <= tm.y, tm.y >= tNear, tm.x <= hit.t;
// BVH/BVH2Common.cpp:3432-3435).
//
// With STAGED, when the packet reaches a brick the warp stages the brick's
// corner values into shared memory once -- 16-byte loads from the
// 16-byte-aligned device brick layout, decoded to float with the reference's
// formula -- and the lanes that enter it march the voxels from shared memory
// (OctreeBrickIntersect, BVH/BVH2Common.cpp:764-984); without, lanes read the
// corners of occupied voxels from global memory.  Both produce identical values;
// each instantiation carries a single brick path (the march is large, and two
// inlined copies overflow the instruction cache).
#include "leaves.cuh"

namespace lrt {
namespace dev {

constexpr int kPktStack = kStackSize;

// per warp: staged brick floats, then the stack (ref, lane mask, min distance)
__host__ __device__ inline size_t pkt_warp_bytes(uint32_t brick_floats) {
  return size_t(brick_floats) * 4 + size_t(kPktStack) * 12;
}

// float -> unsigned with the same order (for warp min reductions)
__device__ __forceinline__ uint32_t ord_bits(float f) {
  const uint32_t b = __float_as_uint(f);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float ord_float(uint32_t u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Decode one brick into shared memory, warp-cooperatively.  `data` points at the
// brick's first word (16-byte aligned in the device layout).
__device__ __forceinline__ void stage_brick(const DevScene &s, const uint32_t *data, float sz_inv, float *dst,
                                            uint32_t lane) {
  const lrt_sbs_header &h = s.sbs_hdr;
  const uint32_t v_size = h.brick_size + 2 * h.brick_pad + 1, v3 = v_size * v_size * v_size;
  const uint32_t layout = h.aux_data & 0xFF000000u;
  if (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN) {
    for (uint32_t i = lane; i < v3; i += 32) dst[i] = __ldg(&s.values_f[__ldg(&data[i])]);
    return;
  }
  const float d_max = 1.73205081f * sz_inv;
  if (h.bytes_per_value == 4) {
    const float mult = 2 * d_max / float(0xFFFFFFFFu);
    const uint4 *src = reinterpret_cast<const uint4 *>(data);
    const uint32_t n4 = (v3 + 3) / 4;
    for (uint32_t j = lane; j < n4; j += 32) {
      const uint4 q = __ldg(&src[j]);
      float4 o;
      o.x = -d_max + mult * float(q.x);
      o.y = -d_max + mult * float(q.y);
      o.z = -d_max + mult * float(q.z);
      o.w = -d_max + mult * float(q.w);
      reinterpret_cast<float4 *>(dst)[j] = o;   // the tail beyond v3 lands in the padding
    }
    return;
  }
  const uint32_t lg = h.bytes_per_value == 2 ? 1u : 2u, bits = 8 * h.bytes_per_value;
  const uint32_t max_val = (1u << bits) - 1;
  const float mult = 2 * d_max / float(max_val);
  for (uint32_t i = lane; i < v3; i += 32) dst[i] = decode_dx(data, i, lg, bits, max_val, d_max, mult);
}

template <bool COUNT, int MODE, bool STAGED>
__global__ void __launch_bounds__(256) render_packet_kernel(DevScene s, RenderLaunch L, uint32_t brick_floats) {
  extern __shared__ float4 smem4[];
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  char *wbase = reinterpret_cast<char *>(smem4) + size_t(warp) * pkt_warp_bytes(brick_floats);
  float *sbrick = reinterpret_cast<float *>(wbase);
  uint32_t *st_ref = reinterpret_cast<uint32_t *>(wbase + size_t(brick_floats) * 4);
  uint32_t *st_mask = st_ref + kPktStack;
  float *st_t = reinterpret_cast<float *>(st_mask + kPktStack);
  const uint32_t FULL = 0xffffffffu;

  Counters cnt = {0, 0, 0, 0};
  const uint32_t spp = s.preset.spp ? s.preset.spp : 1u;
  const uint32_t spp_sqrt = uint32_t(sqrtf(float(spp)));
  const float i_spp_sqrt = 1.0f / float(spp_sqrt);
  const float tNear = 0.0f;
  const float tNearSdf = mx(tNear, 0.1f);
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(L.tile_counter, 1u);
    tile = __shfl_sync(FULL, tile, 0);
    if (tile >= L.total_tiles) break;
    uint32_t v = 0;
    while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
    const DevView &V = L.views[v];
    const uint32_t lt = tile - V.tile_offset;
    const uint32_t lw = V.tile_w_log2;
    const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (lane & ((1u << lw) - 1u));
    const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (lane >> lw);
    const bool in_img = x < V.width && y < V.height;
    float4 acc = make_float4(0, 0, 0, 0);
    Hit first;
    for (uint32_t si = 0; si < spp; si++) {
      const float dx = i_spp_sqrt * float(double(si / spp_sqrt) + 0.5);
      const float dy = i_spp_sqrt * float(double(si % spp_sqrt) + 0.5);
      float3 pos, dir;
      eye_ray(in_img ? x : 0u, in_img ? y : 0u, V.width, V.height, dx, dy, V.proj_inv, V.wv_inv, pos, dir);
      Hit hit;
      hit.t = 1e9f;
      hit.prim = kMiss;
      hit.geom = kMiss;
      hit.c0 = 1.0f;
      hit.c1 = hit.c2 = hit.c3 = 0.0f;
      bool active = in_img;
      {  // TLAS: one leaf node holding the instance box (BVH/BVH2Common.cpp:3508-3529)
        const float3 invw = safe_inverse(dir);
        const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                                  s.inst_bmax[1], s.inst_bmax[2]);
        active = active && (bh.x <= bh.y) && (bh.y > tNear) && (bh.x < hit.t);
      }
      const float3 rp = matmul4x3(s.inst_inv, pos);
      const float3 rd = matmul3x3(s.inst_inv, dir);
      const float3 inv = safe_inverse(rd);
      const uint32_t act = __ballot_sync(FULL, active);
      int sp = 0;
      if (act) {
        if (lane == 0) { st_ref[0] = 0u; st_mask[0] = act; st_t[0] = -3.4e38f; }
        sp = 1;
        __syncwarp();
      }
      while (sp > 0) {
        sp--;
        const uint32_t ref = st_ref[sp];
        const uint32_t m = st_mask[sp];
        const float tmin_w = st_t[sp];
        __syncwarp();   // every lane has read slot sp before it is pushed over
        bool mine = ((m >> lane) & 1u) && !(tmin_w > hit.t);
        if (__ballot_sync(FULL, mine) == 0) continue;
        if (ref & kLeafBit) {
          const uint32_t brick = ref & ~kLeafBit;
          // exact per-lane leaf test against the BVH leaf box
          const float4 bl = __ldg(&s.leaf_boxes[2 * brick]), bh = __ldg(&s.leaf_boxes[2 * brick + 1]);
          const float2 tm = ray_box(rp, inv, bl.x, bl.y, bl.z, bh.x, bh.y, bh.z);
          mine = mine && !(tm.x > hit.t);
          const uint32_t mm = __ballot_sync(FULL, mine);
          if (mm == 0) continue;
          if (STAGED) {
            const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
            stage_brick(s, s.values + nd.z, 2.0f / float(nd.y & 0x0000FFFF), sbrick, lane);
            __syncwarp();
            if (mine) brick_intersect<COUNT, true, MODE>(s, rp, rd, inv, tNearSdf, brick, hit, cnt, sbrick);
            __syncwarp();   // the buffer is rewritten by the next brick
          } else if (mine) {
            brick_intersect<COUNT, false, MODE>(s, rp, rd, inv, tNearSdf, brick, hit, cnt);
          }
          continue;
        }
        const WNode4 *nd = s.nodes + ref;
        if (COUNT && mine) cnt.nodes++;
        const float4 lx = __ldg(reinterpret_cast<const float4 *>(nd->lo_x));
        const float4 hx = __ldg(reinterpret_cast<const float4 *>(nd->hi_x));
        const float4 ly = __ldg(reinterpret_cast<const float4 *>(nd->lo_y));
        const float4 hy = __ldg(reinterpret_cast<const float4 *>(nd->hi_y));
        const float4 lz = __ldg(reinterpret_cast<const float4 *>(nd->lo_z));
        const float4 hz = __ldg(reinterpret_cast<const float4 *>(nd->hi_z));
        const uint4 ch = __ldg(reinterpret_cast<const uint4 *>(nd->child));
        const float lxa[4] = {lx.x, lx.y, lx.z, lx.w}, hxa[4] = {hx.x, hx.y, hx.z, hx.w};
        const float lya[4] = {ly.x, ly.y, ly.z, ly.w}, hya[4] = {hy.x, hy.y, hy.z, hy.w};
        const float lza[4] = {lz.x, lz.y, lz.z, lz.w}, hza[4] = {hz.x, hz.y, hz.z, hz.w};
        const uint32_t cha[4] = {ch.x, ch.y, ch.z, ch.w};
        float key[4];
        uint32_t cmask[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const float2 tm = ray_box(rp, inv, lxa[i], lya[i], lza[i], hxa[i], hya[i], hza[i]);
          const bool hc = mine && (tm.x <= tm.y) && (tm.y >= tNear) && (tm.x <= hit.t) && cha[i] != kEmptyChild;
          cmask[i] = __ballot_sync(FULL, hc);
          key[i] = ord_float(__reduce_min_sync(FULL, hc ? ord_bits(tm.x) : 0xFFFFFFFFu));
        }
        // order children far -> near (warp-uniform), push the ones some lane enters
        int ord[4] = {0, 1, 2, 3};
#pragma unroll
        for (int a = 0; a < 3; a++)
#pragma unroll
          for (int b = 0; b < 3 - a; b++)
            if (key[ord[b]] < key[ord[b + 1]]) { const int t = ord[b]; ord[b] = ord[b + 1]; ord[b + 1] = t; }
#pragma unroll
        for (int i = 0; i < 4; i++) {
          const int c = ord[i];
          if (cmask[c] && sp < kPktStack) {   // depth is bounded on the host: never drops
            if (lane == 0) { st_ref[sp] = cha[c]; st_mask[sp] = cmask[c]; st_t[sp] = key[c]; }
            sp++;
          }
        }
        __syncwarp();
      }
      hit_colour(s, pos, dir, hit);   // a lane outside the image holds no hit
      if (si == 0) first = hit;
      if (L.rgba || L.rgba8) {
        const float4 c = shade(s, hit, pos, dir);
        acc.x += c.x; acc.y += c.y; acc.z += c.z; acc.w += c.w;
      }
    }
    if (!in_img) continue;
    const size_t pix = size_t(V.pix_offset) + size_t(y) * V.width + x;
    if (L.hits16) {
      lrt_hit16 o;
      o.t = first.t;
      o.primId = first.prim;
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

template <bool COUNT, int MODE, bool STAGED>
static cudaError_t launch_packet_s(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   const Tuning &tu) {
  const uint32_t v_size = s.sbs_hdr.brick_size + 2 * s.sbs_hdr.brick_pad + 1;
  const uint32_t brick_floats = (v_size * v_size * v_size + 3u) & ~3u;
  const int warps = tu.block_warps;
  const size_t smem = size_t(warps) * dev::pkt_warp_bytes(STAGED ? brick_floats : 0u);
  const void *fn = reinterpret_cast<const void *>(&dev::render_packet_kernel<COUNT, MODE, STAGED>);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, warps * 32, smem);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + warps - 1) / warps;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_packet_kernel<COUNT, MODE, STAGED><<<blocks, warps * 32, smem, st>>>(s, L, STAGED ? brick_floats : 0u);
  return cudaGetLastError();
}

template <bool COUNT, int MODE>
static cudaError_t launch_packet_m(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   const Tuning &tu) {
  return tu.stage ? launch_packet_s<COUNT, MODE, true>(s, L, num_sms, st, tu)
                  : launch_packet_s<COUNT, MODE, false>(s, L, num_sms, st, tu);
}

template <bool COUNT>
static cudaError_t launch_packet_c(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st,
                                   const Tuning &tu) {
  switch (s.preset.sdf_node_intersect) {
    case LRT_INTERSECT_NEWTON: return launch_packet_m<COUNT, LRT_INTERSECT_NEWTON>(s, L, num_sms, st, tu);
    case LRT_INTERSECT_ST: return launch_packet_m<COUNT, LRT_INTERSECT_ST>(s, L, num_sms, st, tu);
    default: return launch_packet_m<COUNT, -1>(s, L, num_sms, st, tu);
  }
}

cudaError_t launch_render_packet(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count,
                                 const Tuning &tu) {
  return count ? launch_packet_c<true>(s, L, num_sms, st, tu) : launch_packet_c<false>(s, L, num_sms, st, tu);
}

}  // namespace lrt
