// BVH traversal shared by the render kernels (trace.cu) and the proposal
// kernels (proposal.cu): the per-ray closest-hit walk over the 4-wide BVH.
#pragma once
#include "leaves.cuh"

namespace lrt {
namespace dev {

template <bool COUNT, int STACK, bool FMA_SLAB = false>
__device__ __forceinline__ void visit_node(const DevScene &s, uint32_t ref, float3 rp, float3 inv, float tNear,
                                           float hit_t, uint2 *st, int &sp, Counters &cnt,
                                           float3 noi = make_float3(0.0f, 0.0f, 0.0f));

constexpr int kRefStack = 80;   // BVH2TraverseF32's stack, BVH/BVH2Common.cpp:3412

// BVH2TraverseF32 (BVH/BVH2Common.cpp:3407-3488) on the reference's fat-pair
// layout: both children of a pair are slab-tested, the nearer entered child is
// walked first and the other pushed, and the walk stops after the first SDF leaf
// that reports a hit (:3402-3405, :3478) -- the reference's result, which depends
// on the tree's topology.  SBS / SVS leaves only (their payload is the brick or
// voxel index).  The host checks that the tree is acyclic, that every index lies
// inside the pair and brick arrays and that no path needs more than kRefStack
// entries before it uploads the pairs, so neither bound below ever binds.
template <int TYPE, bool COUNT, int MODE, int FEAT>
__device__ void walk_bvh2(const DevScene &s, float3 rp, float3 rd, float3 inv, float tNear, float tNearSdf,
                          Hit &hit, Counters &cnt) {
  uint32_t stack[kRefStack];
  int top = 0;
  uint32_t left = 0;
  bool found = false;
  uint32_t visits = 0;
  while (top >= 0 && !found) {
    while (top >= 0 && (left & kLeafBit) == 0) {
      if (++visits > s.n_pairs) return;
      if (COUNT) cnt.nodes++;
      const float4 a0 = __ldg(&s.pairs[4 * left + 0]), a1 = __ldg(&s.pairs[4 * left + 1]);
      const float4 b0 = __ldg(&s.pairs[4 * left + 2]), b1 = __ldg(&s.pairs[4 * left + 3]);
      const uint32_t n0 = __float_as_uint(a0.w), n1 = __float_as_uint(b0.w);
      const float2 tm0 = ray_box(rp, inv, a0.x, a0.y, a0.z, a1.x, a1.y, a1.z);
      const float2 tm1 = ray_box(rp, inv, b0.x, b0.y, b0.z, b1.x, b1.y, b1.z);
      const bool h0 = (tm0.x <= tm0.y) && (tm0.y >= tNear) && (tm0.x <= hit.t);
      const bool h1 = (tm1.x <= tm1.y) && (tm1.y >= tNear) && (tm1.x <= hit.t);
      left = h0 ? n0 : n1;
      if (h0 && h1) {
        left = (tm0.x <= tm1.x) ? n0 : n1;
        if (top >= kRefStack) return;
        stack[top] = (tm0.x <= tm1.x) ? n1 : n0;
        top++;
      }
      if (!h0 && !h1) {
        top--;
        left = stack[top > 0 ? top : 0];
      }
    }
    if (top >= 0 && left != 0xFFFFFFFFu) {
      const float t_before = hit.t;
      const uint32_t prim = left & 0x00FFFFFFu;   // EXTRACT_START
      if (TYPE == LRT_TYPE_SDF_SVS)
        svs_intersect<COUNT, MODE>(s, rp, rd, tNearSdf, prim, hit, cnt);
      else
        brick_intersect<COUNT, false, MODE, FEAT>(s, rp, rd, inv, tNearSdf, prim, hit, cnt);
      found = hit.t < t_before;
    }
    top--;
    left = stack[top > 0 ? top : 0];
  }
}

// One instance of RayQuery_NearestHit (BVH/BVH2Common.cpp:3490-3559): the
// instance box (the TLAS leaf), the ray in object space, the BLAS walk.  `s`
// carries the instance in its instance-0 fields.  Returns after the first hit
// when stop_first (RayQuery_AnyHit).
template <int TYPE, bool COUNT, int MODE, int STACK, int FEAT>
__device__ __forceinline__ void trace_instance(const DevScene &s, float3 pos, float tNear, float3 dir, bool stop_first,
                                               Hit &hit, Counters &cnt) {
  {  // TLAS leaf: the instance box (:3508-3529)
    const float3 invw = safe_inverse(dir);
    const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                              s.inst_bmax[1], s.inst_bmax[2]);
    if (!((bh.x <= bh.y) && (bh.y > tNear) && (bh.x < hit.t))) return;
  }
  const float3 rp = matmul4x3(s.inst_inv, pos);
  const float3 rd = matmul3x3(s.inst_inv, dir);
  const float3 inv = safe_inverse(rd);
  const float tNearSdf = mx(tNear, 0.1f);   // SDF bias passed to every leaf type (:3472-3476)
  if (FEAT & 4) {   // the reference's first-hit walk over its BVH2 layout
    walk_bvh2<TYPE, COUNT, MODE, FEAT & 3>(s, rp, rd, inv, tNear, tNearSdf, hit, cnt);
    return;
  }

  const float3 noi = f3(-(rp.x * inv.x), -(rp.y * inv.y), -(rp.z * inv.z));   // FEAT bit 4's slab test
  // per-ray stack of (node ref, entry distance as float bits), one 8-byte entry each
  uint2 st[STACK];
  int sp = 0;
  st[sp] = make_uint2(0u, __float_as_uint(-3.4e38f));   // root wide node
  sp++;
  // "while-while" structure: each lane walks inner nodes until it holds a leaf
  // (or its stack is empty); the warp reconverges, and all lanes holding a leaf
  // intersect it together.  Leaf work then runs with the lanes that need it at
  // the same time instead of one lane per iteration of a mixed loop.
  for (;;) {
    uint32_t leaf = 0;
    bool have_leaf = false;
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
      if (FEAT & 16)
        visit_node<COUNT, STACK, true>(s, ref, rp, inv, tNear, hit.t, st, sp, cnt, noi);
      else
        visit_node<COUNT, STACK>(s, ref, rp, inv, tNear, hit.t, st, sp, cnt);
    }
    if (!have_leaf) break;
    const float t_before = hit.t;
    if (TYPE == LRT_TYPE_MESH_TRIANGLE)
      tri_intersect<COUNT>(s, rp, rd, tNearSdf, leaf & 0x00FFFFFFu, (leaf >> 24) & 0x7Fu, hit, cnt);
    else if (TYPE == LRT_TYPE_SDF_SVS)
      svs_intersect<COUNT, MODE>(s, rp, rd, tNearSdf, leaf, hit, cnt);
    else
      brick_intersect<COUNT, false, MODE, FEAT & 19>(s, rp, rd, inv, tNearSdf, leaf, hit, cnt);
    if (stop_first && hit.t < t_before) break;
  }
}

// RayQuery_NearestHit (BVH/BVH2Common.cpp:3490-3559) over the 4-wide BVH.
// stopOnFirstHit (tFar <= 0) returns the first hit found (RayQuery_AnyHit).
// SBS brick colours are added by the caller (hit_colour) unless FEAT bit 1 has
// them computed in the leaf loop.  FEAT bit 2: the reference's BVH2 walk with
// its first-hit early-out (walk_bvh2) instead of the closest-hit 4-wide walk.
// FEAT bit 3: several instances of the geometry (s.insts), each tested and
// walked in instance order with the closest hit so far -- the reference walks
// its TLAS over the instance boxes (:3508-3547) with the same hit.t culling, so
// the closest hit is the same; hit.inst names the instance hit.  FEAT bit 4
// (value 16): inner-node slab tests as one FMA per plane (ray_box_fma), for the
// kernels compiled with contraction.
template <int TYPE, bool COUNT, int MODE = -1, int STACK = kStackSize, int FEAT = 0>
__device__ void trace(const DevScene &s, float3 pos, float tNear, float3 dir, float tFar, Hit &hit, Counters &cnt) {
  const bool stop_first = (tFar <= 0.0f);
  if (stop_first) tFar *= -1.0f;
  hit.t = tFar;
  hit.prim = kMiss;
  hit.geom = kMiss;
  hit.c0 = 1.0f;
  hit.c1 = hit.c2 = hit.c3 = 0.0f;
  if (FEAT & 8) {
    hit.inst = kMiss;
    for (uint32_t ii = 0; ii < s.n_inst; ii++) {
      const DevScene si = scene_of_instance(s, ii);
      const float t_before = hit.t;
      trace_instance<TYPE, COUNT, MODE, STACK, FEAT & 7>(si, pos, tNear, dir, stop_first, hit, cnt);
      if (hit.t < t_before) hit.inst = ii;
      if (stop_first && hit.prim != kMiss) break;
    }
    return;
  }
  trace_instance<TYPE, COUNT, MODE, STACK, FEAT>(s, pos, tNear, dir, stop_first, hit, cnt);
}

// One inner node of the per-ray traversal: test the four child boxes with the
// reference slab test and push the entered ones far-to-near.
template <bool COUNT, int STACK, bool FMA_SLAB>
__device__ __forceinline__ void visit_node(const DevScene &s, uint32_t ref, float3 rp, float3 inv, float tNear,
                                           float hit_t, uint2 *st, int &sp, Counters &cnt, float3 noi) {
  {
    const WNode4 *nd = s.nodes + ref;
    if (COUNT) cnt.nodes++;
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
    // child entry distances and refs; a missed child sorts last (key -inf)
    float kt[4];
    uint32_t kr[4];
    int nk = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const float2 tm = FMA_SLAB ? ray_box_fma(inv, noi, lxa[i], lya[i], lza[i], hxa[i], hya[i], hza[i])
                                 : ray_box(rp, inv, lxa[i], lya[i], lza[i], hxa[i], hya[i], hza[i]);
      const bool h = (tm.x <= tm.y) && (tm.y >= tNear) && (tm.x <= hit_t) && cha[i] != kEmptyChild;
      kt[i] = h ? tm.x : -__int_as_float(0x7f800000);
      kr[i] = cha[i];
      nk += h ? 1 : 0;
    }
    // a vote among the lanes that are here together (the traversal loop diverges)
    if (__any_sync(__activemask(), nk > 1)) {
      // far-to-near order (the nearest child is popped first) by a 5-exchange
      // sorting network on registers, descending entry distance
#define LRT_CE(a, b)                                                \
      {                                                             \
        const bool sw = kt[b] > kt[a];                              \
        const float t0 = sw ? kt[b] : kt[a], t1 = sw ? kt[a] : kt[b]; \
        const uint32_t r0 = sw ? kr[b] : kr[a], r1 = sw ? kr[a] : kr[b]; \
        kt[a] = t0; kt[b] = t1; kr[a] = r0; kr[b] = r1;             \
      }
      LRT_CE(0, 1) LRT_CE(2, 3) LRT_CE(0, 2) LRT_CE(1, 3) LRT_CE(1, 2)
#undef LRT_CE
    } else {
      // no lane voting here entered more than one child: move the entered one (if
      // any) to the front, no ordering needed
#pragma unroll
      for (int i = 1; i < 4; i++)
        if (kt[i] > kt[0]) { kt[0] = kt[i]; kr[0] = kr[i]; }
    }
    // The host rejects trees deeper than the stack allows ((W-1)*depth + 1 entries),
    // so this bound never drops an entry.
#pragma unroll
    for (int i = 0; i < 4; i++) {
      if (i < nk && sp < STACK) { st[sp] = make_uint2(kr[i], __float_as_uint(kt[i])); sp++; }
    }
  }
}

}  // namespace dev
}  // namespace lrt
