// Persistent SBS render kernel with the traversal and leaf phases regrouped
// across the warps of a block ("variant" 3).
//
// In the per-lane kernel a warp's lanes walk the BVH until each holds a brick,
// then the lanes holding one march it together while the others idle; a brick
// march (voxel steps + the trilinear finder) is most of a ray's instructions
// and the lanes that run it are few.  Here the two phases are separated by block
// barriers:
//
//   traversal  every live lane of the block's 4 warps walks the 4-wide BVH
//              until it holds a brick or its stack is empty (the ray is done);
//              a lane holding a brick appends (owner, brick) to a block queue
//              with a warp-aggregated shared-memory atomic and waits;
//   leaf       the queued marches are dealt out to the block's threads in queue
//              order, so they run in as few warps as possible, each nearly full;
//              a march reads its ray from the owner's shared-memory slot and
//              writes the hit back there;
//   resume     owners read their hit back and walk on with the new closest t.
//
// Each ray has at most one march in flight and resumes only after its hit is
// written back, so every march and every culling test sees exactly the hit
// state of the per-lane kernel: the records are identical.  A warp keeps its
// 32-pixel tile until all its rays are done, then takes the next tile of the
// persistent queue.  SBS scenes, spp 1, no shading features beyond kernel_RayTrace's
// plain modes.
#pragma once
#include "traverse.cuh"

namespace lrt {
namespace dev {

constexpr int kLqThreads = 128;

template <int MODE, int STACK, int FP>
__global__ void __launch_bounds__(kLqThreads, 5) render_lq_kernel(DevScene s, RenderLaunch L) {
  // the rays of the block: object-space origin, direction, inverse direction and
  // the current closest hit, one slot per thread
  __shared__ float s_rp[3][kLqThreads], s_rd[3][kLqThreads], s_inv[3][kLqThreads];
  __shared__ float s_t[kLqThreads], s_c2[kLqThreads], s_c3[kLqThreads];
  __shared__ uint32_t s_prim[kLqThreads];
  __shared__ uint32_t s_job_brick[kLqThreads], s_job_owner[kLqThreads];
  __shared__ uint32_t s_nq[2];             // queue lengths, alternating by round
  const uint32_t tid = threadIdx.x, lane = tid & 31u;
  Counters cnt = {0, 0, 0, 0};
  const uint32_t geom = s.geom_id | (s.type << 24);
  if (tid < 2) s_nq[tid] = 0;

  bool live = false;         // this lane holds an unfinished ray
  bool tiles_left = true;    // this warp may still find tiles
  float3 pos = f3(0, 0, 0), dir = f3(0, 0, 1), rp = pos, rd = dir, inv = dir;
  Hit hit;
  hit.t = 1e9f; hit.prim = kMiss; hit.geom = kMiss; hit.c0 = 1.0f; hit.c1 = hit.c2 = hit.c3 = 0.0f;
  uint2 st[STACK];
  int sp = 0;
  size_t pix = 0;
  uint32_t round = 0;

  // a finished ray: colours of layouts that carry them, shading, outputs
  auto finish = [&]() {
    hit_colour(s, pos, dir, hit);
    if (L.hits16) {
      lrt_hit16 o;
      o.t = hit.t;
      o.primId = hit.prim;
      o.nx = hit.c2;
      o.ny = hit.c3;
      reinterpret_cast<float4 *>(L.hits16)[pix] = *reinterpret_cast<const float4 *>(&o);
    }
    if (L.rgba || L.rgba8) {
      const float4 c = shade(s, hit, pos, dir);
      if (L.rgba) L.rgba[pix] = c;
      if (L.rgba8) L.rgba8[pix] = encode_rgba8(c);
    }
  };
  __syncthreads();

  for (;;) {
    // ---- a warp whose rays are all done takes tiles until one holds a ray that
    // enters the scene (tiles whose rays all miss finish here, in the same round)
    while (tiles_left && !__any_sync(0xffffffffu, live)) {
      uint32_t tile = 0;
      if (lane == 0) tile = atomicAdd(L.tile_counter, 1u);
      tile = __shfl_sync(0xffffffffu, tile, 0);
      if (tile >= L.total_tiles) {
        tiles_left = false;
      } else {
        uint32_t v = 0;
        while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
        const DevView &V = L.views[v];
        const uint32_t lt = tile - V.tile_offset, lw = V.tile_w_log2;
        const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (lane & ((1u << lw) - 1u));
        const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (lane >> lw);
        if (x < V.width && y < V.height) {
          eye_ray(x, y, V.width, V.height, 0.5f, 0.5f, V.proj_inv, V.wv_inv, pos, dir);
          pix = size_t(V.pix_offset) + size_t(y) * V.width + x;
          hit.t = 1e9f; hit.prim = kMiss; hit.geom = kMiss; hit.c0 = 1.0f; hit.c1 = hit.c2 = hit.c3 = 0.0f;
          // TLAS: the single instance's box (BVH/BVH2Common.cpp:3508-3529)
          const float3 invw = safe_inverse(dir);
          const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                                    s.inst_bmax[1], s.inst_bmax[2]);
          if ((bh.x <= bh.y) && (bh.y > 0.0f) && (bh.x < hit.t)) {
            rp = matmul4x3(s.inst_inv, pos);
            rd = matmul3x3(s.inst_inv, dir);
            inv = safe_inverse(rd);
            s_rp[0][tid] = rp.x; s_rp[1][tid] = rp.y; s_rp[2][tid] = rp.z;
            s_rd[0][tid] = rd.x; s_rd[1][tid] = rd.y; s_rd[2][tid] = rd.z;
            s_inv[0][tid] = inv.x; s_inv[1][tid] = inv.y; s_inv[2][tid] = inv.z;
            st[0] = make_uint2(0u, __float_as_uint(-3.4e38f));
            sp = 1;
            live = true;
          } else {
            finish();   // outside the instance box: a miss
          }
        }
      }
    }
    // ---- traversal: walk until a brick is held or the stack is empty
    const uint32_t q = round & 1u;
    if (live) {
      uint32_t leaf = 0;
      bool have_leaf = false;
      while (sp > 0) {
        sp--;
        const uint2 top = st[sp];
        if (__uint_as_float(top.y) > hit.t) continue;
        if (top.x & kLeafBit) {
          leaf = top.x & ~kLeafBit;
          have_leaf = true;
          break;
        }
        visit_node<false, STACK>(s, top.x, rp, inv, 0.0f, hit.t, st, sp, cnt);
      }
      if (have_leaf) {
        s_t[tid] = hit.t;
        s_prim[tid] = hit.prim;
        s_c2[tid] = hit.c2;
        s_c3[tid] = hit.c3;
        // warp-aggregated append to this round's queue
        const uint32_t m = __activemask();
        const uint32_t want = __ballot_sync(m, true);
        const uint32_t leader = __ffs(want) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&s_nq[q], uint32_t(__popc(want)));
        base = __shfl_sync(m, base, leader);
        const uint32_t slot = base + __popc(want & ((1u << lane) - 1u));
        s_job_brick[slot] = leaf;
        s_job_owner[slot] = tid;
      } else {
        live = false;   // stack empty: the closest hit is final
        finish();
      }
    }
    // ---- leaf phase: the block's queued marches, dealt out in queue order
    const int more = __syncthreads_or(live || tiles_left);
    const uint32_t nq = s_nq[q];
    if (tid == 0) s_nq[q ^ 1u] = 0;   // next round's queue (appended to only after the barrier below)
    if (tid < nq) {
      const uint32_t o = s_job_owner[tid], brick = s_job_brick[tid];
      Hit h;
      h.t = s_t[o];
      h.prim = s_prim[o];
      const bool had = h.prim != kMiss;
      h.geom = had ? geom : kMiss;
      h.c0 = had ? 0.0f : 1.0f;
      h.c1 = 0.0f;
      h.c2 = s_c2[o];
      h.c3 = s_c3[o];
      const float3 jrp = f3(s_rp[0][o], s_rp[1][o], s_rp[2][o]);
      const float3 jrd = f3(s_rd[0][o], s_rd[1][o], s_rd[2][o]);
      const float3 jinv = f3(s_inv[0][o], s_inv[1][o], s_inv[2][o]);
      const float t0 = h.t;
      brick_intersect<false, false, MODE, 0>(s, jrp, jrd, jinv, 0.1f, brick, h, cnt);
      if (h.t != t0) {
        s_t[o] = h.t;
        s_prim[o] = h.prim;
        s_c2[o] = h.c2;
        s_c3[o] = h.c3;
      }
    }
    __syncthreads();
    if (!more) break;
    // ---- resume: owners read their hit back
    if (live) {
      hit.t = s_t[tid];
      hit.prim = s_prim[tid];
      if (hit.prim != kMiss) {
        hit.geom = geom;
        hit.c0 = 0.0f;
        hit.c1 = 0.0f;
        hit.c2 = s_c2[tid];
        hit.c3 = s_c3[tid];
      }
    }
    round++;
  }
}

}  // namespace dev
}  // namespace lrt
