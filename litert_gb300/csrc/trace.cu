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
#include "trace_common.cuh"

namespace lrt {
namespace dev {

// LocalSurfaceIntersection, BVH/BVH2Common.cpp:274-631 (trilinear; ST, ANALYTIC,
// NEWTON, BBOX, IT).  Updates `hit` when the crossing is closer.
template <bool COUNT>
__device__ __forceinline__ void local_surface(const lrt_preset &pr, const DevScene &s, uint32_t type, float3 ray_dir,
                                              const float values[8], uint32_t prim_id, float d, float qNear,
                                              float qFar, float2 fNearFar, float3 start_q, Hit &hit,
                                              Counters &cnt) {
  const float EPS = 1e-6f;
  const float d_inv = 1.0f / d;
  float t = qNear;
  bool is_hit = false;
  unsigned iter = 0;
  float start_sign = 1;
  float start_dist = trilinear(values, add(start_q, scl(t, ray_dir)));
  if (COUNT) cnt.finder++;
  if (pr.representation_mode == 0) start_sign = signf(start_dist);
  start_dist *= start_sign;

  if (start_dist <= EPS || pr.sdf_node_intersect == LRT_INTERSECT_BBOX) {
    is_hit = true;
  } else if (pr.sdf_node_intersect == LRT_INTERSECT_ST) {
    float dist = start_dist;
    while (t < qFar && dist > EPS && iter < 256u) {
      t += dist * d_inv;
      dist = start_sign * trilinear(values, add(start_q, scl(t, ray_dir)));
      iter++;
    }
    is_hit = (dist <= EPS);
  } else {
    const float s000 = values[0] * d_inv, s001 = values[1] * d_inv, s010 = values[2] * d_inv,
                s011 = values[3] * d_inv, s100 = values[4] * d_inv, s101 = values[5] * d_inv,
                s110 = values[6] * d_inv, s111 = values[7] * d_inv;
    const float a = s101 - s001;
    const float k0 = s000, k1 = s100 - s000, k2 = s010 - s000, k3 = s110 - s010 - k1;
    const float k4 = k0 - s001, k5 = k1 - a, k6 = k2 - (s011 - s001), k7 = k3 - (s111 - s011 - a);
    const float3 o = start_q, d3 = ray_dir;
    const float m0 = o.x * o.y, m1 = d3.x * d3.y, m2 = o.x * d3.y + o.y * d3.x;
    const float m3 = k5 * o.z - k1, m4 = k6 * o.z - k2, m5 = k7 * o.z - k3;
    const float c0 = (k4 * o.z - k0) + o.x * m3 + o.y * m4 + m0 * m5;
    const float c1 = d3.x * m3 + d3.y * m4 + m2 * m5 + d3.z * (k4 + k5 * o.x + k6 * o.y + k7 * m0);
    const float c2 = m1 * m5 + d3.z * (k5 * d3.x + k6 * d3.y + k7 * m2);
    const float c3 = k7 * m1 * d3.z;

    if (pr.sdf_node_intersect == LRT_INTERSECT_NEWTON) {           // :437-522
      const float aa = 3 * c3, b = 2 * c2, c = c1;
      const float t0 = 0, t3 = qFar;
      float t1 = qFar, t2 = qFar;
      const float D = b * b - 4 * aa * c;
      if (D >= 0) {
        const float q = -0.5f * (b + signf(b) * sqrtf(D));
        t1 = fabsf(aa) > EPS ? q / aa : t0;
        t2 = fabsf(q) > EPS ? c / q : qFar;
        const float tmp = mn(t1, t2);
        t2 = mx(t1, t2);
        t1 = tmp;
        t1 = clampf(t1, t0, t3);
        t2 = clampf(t2, t0, t3);
      }
      const bool s0 = c0 > 0;
      const bool s1 = (c0 + t1 * (c1 + t1 * (c2 + t1 * c3))) > 0;
      const bool s2 = (c0 + t2 * (c1 + t2 * (c2 + t2 * c3))) > 0;
      const bool s3 = (c0 + t3 * (c1 + t3 * (c2 + t3 * c3))) > 0;
      float nwt_min = t0, nwt_max = t0;
      if (s0 != s1) { nwt_min = t0; nwt_max = t1; }
      else if (s1 != s2) { nwt_min = t1; nwt_max = t2; }
      else if (s2 != s3) { nwt_min = t2; nwt_max = t3; }
      if (nwt_min < nwt_max) {
        unsigned it = 0;
        float rtn = 0.5f * (nwt_min + nwt_max);
        float f = 1000;
        while (it < 10u && fabsf(f) >= EPS) {
          f = c0 + rtn * (c1 + rtn * (c2 + rtn * c3));
          const float df = c1 + rtn * (2 * c2 + rtn * 3 * c3);
          const float dx = f / (df + signf(df) * 1e-9f);
          rtn -= dx;
          it++;
        }
        t = rtn;
        is_hit = (t >= 0 && t <= qFar && fabsf(f) < EPS);
      } else {
        is_hit = false;
      }
    } else if (pr.sdf_node_intersect == LRT_INTERSECT_ANALYTIC) {   // :367-436
      float x1 = 1000, x2 = 1000, x3 = 1000;
      if (fabsf(c3) > 1e-2) {
        const float aa = c2 / c3, b = c1 / c3, c = c0 / c3;
        const float Q = (aa * aa - 3 * b) / 9;
        const float R = (2 * aa * aa - 9 * aa * b + 27 * c) / 54;
        const float Q3 = Q * Q * Q;
        if (R * R < Q3) {
          const float theta = acosf(R / sqrtf(Q3));
          x1 = -2 * sqrtf(Q) * cosf(theta / 3) - aa / 3;
          x2 = -2 * sqrtf(Q) * cosf((theta + 2 * 3.14159265358979323846f) / 3) - aa / 3;
          x3 = -2 * sqrtf(Q) * cosf((theta - 2 * 3.14159265358979323846f) / 3) - aa / 3;
        } else {
          const float A = -signf(R) * powf(fabsf(R) + sqrtf(R * R - Q3), 1.0f / 3.0f);
          const float B = fabsf(A) > EPS ? Q / A : 0;
          x1 = A + B - aa / 3;
        }
      } else if (fabsf(c2) > 1e-4) {
        const float D = c1 * c1 - 4 * c2 * c0;
        if (D > 0) {
          const float q = -0.5f * (c1 + signf(c1) * sqrtf(D));
          x1 = q / c2;
          if (fabsf(q) > EPS) x2 = c0 / q;
        }
      } else if (fabsf(c1) > EPS) {
        x1 = -c0 / c1;
      }
      x1 = x1 < 0 ? 1000 : x1;
      x2 = x2 < 0 ? 1000 : x2;
      x3 = x3 < 0 ? 1000 : x3;
      t = mn(x1, mn(x2, x3));
      is_hit = (t >= 0 && t <= qFar);
    } else {                                                        // IT, :523-550
      float e = 0.1f * qFar;
      const float t_max = fabsf(c3) < EPS ? 1e6f : -c2 / (3 * c3);
      const float df_max = 3 * c3 * t_max * t_max + 2 * c2 * t_max + c1;
      float dist = start_dist;
      while (t < qFar && dist > EPS && iter < 256u) {
        const float df_1 = 3 * c3 * t * t + 2 * c2 * t + c1;
        const float df_2 = 3 * c3 * (t + e) * (t + e) + 2 * c2 * (t + e) + c1;
        float L = (t_max > t && t_max < t + e) ? mx(df_max, mx(df_1, df_2)) : mx(df_1, df_2);
        L = mx(L, EPS);
        const float st = mn((dist * d_inv) / L, e);
        t += st;
        e = 2 * st;
        dist = start_sign * trilinear(values, add(start_q, scl(t, ray_dir)));
        iter++;
      }
      is_hit = (dist <= EPS);
    }
  }

  const float tReal = fNearFar.x + d * t;
  if (t <= qFar && is_hit && tReal < hit.t) {                      // :569-601
    float3 norm = f3(0, 0, 1);
    if (need_normal(pr.render_mode)) {
      const float3 p0 = add(start_q, scl(t, ray_dir));
      const float h = 0.001f;
      const float ddx = (trilinear(values, add(p0, f3(h, 0, 0))) - trilinear(values, add(p0, f3(-h, 0, 0)))) / (2 * h);
      const float ddy = (trilinear(values, add(p0, f3(0, h, 0))) - trilinear(values, add(p0, f3(0, -h, 0)))) / (2 * h);
      const float ddz = (trilinear(values, add(p0, f3(0, 0, h))) - trilinear(values, add(p0, f3(0, 0, -h)))) / (2 * h);
      norm = scl(start_sign, normalize(matmul4x3(s.inst_inv_t, f3(ddx, ddy, ddz))));
    }
    const float2 en = encode_normal(norm);
    hit.t = tReal;
    hit.prim = (pr.render_mode == 10) ? iter : prim_id;
    hit.geom = s.geom_id | (type << 24);
    hit.c0 = 0;
    hit.c1 = 0;
    hit.c2 = en.x;
    hit.c3 = en.y;
  }
}

// load_distance_values, BVH/BVH2Common.cpp:725-762 (SBS_v_to_i, sdfScene/sdf_scene.h:201-204)
__device__ __forceinline__ float load_values(const DevScene &s, uint32_t data_offset, float3 vp, uint32_t v_size,
                                             float sz_inv, float values[8]) {
  const lrt_sbs_header &h = s.sbs_hdr;
  float vmin = 1e6f;
  const uint32_t layout = h.aux_data & 0xFF000000u;
  const uint32_t ix = uint32_t(vp.x), iy = uint32_t(vp.y), iz = uint32_t(vp.z);
  if (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN) {
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const uint32_t vId = (ix + ((i & 4) >> 2) + h.brick_pad) * v_size * v_size +
                           (iy + ((i & 2) >> 1) + h.brick_pad) * v_size + (iz + (i & 1) + h.brick_pad);
      values[i] = __ldg(&s.values_f[__ldg(&s.values[data_offset + vId])]);
      vmin = mn(vmin, values[i]);
    }
  } else {
    const uint32_t vals_per_int = 4 / h.bytes_per_value;
    const uint32_t bits = 8 * h.bytes_per_value;
    const uint32_t max_val = h.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
    const float d_max = 1.73205081f * sz_inv;
    const float mult = 2 * d_max / float(max_val);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const uint32_t vId = (ix + ((i & 4) >> 2) + h.brick_pad) * v_size * v_size +
                           (iy + ((i & 2) >> 1) + h.brick_pad) * v_size + (iz + (i & 1) + h.brick_pad);
      const uint32_t q = (__ldg(&s.values[data_offset + vId / vals_per_int]) >> (bits * (vId % vals_per_int))) & max_val;
      values[i] = -d_max + mult * float(q);
      vmin = mn(vmin, values[i]);
    }
  }
  return vmin;
}

// OctreeBrickIntersect, BVH/BVH2Common.cpp:764-984 (trilinear, colour for indexed layouts)
template <bool COUNT>
__device__ void brick_intersect(const DevScene &s, float3 ray_pos, float3 ray_dir, float3 inv, float tNear,
                                uint32_t brick, Hit &hit, Counters &cnt) {
  const lrt_sbs_header &h = s.sbs_hdr;
  const lrt_preset &pr = s.preset;
  const uint32_t type = s.type;
  const uint32_t v_size = h.brick_size + 2 * h.brick_pad + 1;
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF);
  const float pz = float(nd.y >> 16), sz = float(nd.y & 0x0000FFFF);
  const float sz_inv = 2.0f / sz;
  const float bs = float(h.brick_size);
  const float d = 2.0f / (sz * bs);
  const float3 bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(px, py, pz)));
  const float3 bmax = add(bmin, scl(sz_inv, f3(1, 1, 1)));
  float2 bnf = ray_box(ray_pos, inv, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z);
  const float old_t = hit.t;
  const float scale = 0.5f * sz * bs;
  float values[8];
  if (COUNT) cnt.leaves++;
  // A ray crosses at most 3*brick_size voxels.  The reference's loop has no
  // bound; its +1e-6 step stops advancing beyond t ~ 32, where a degenerate
  // voxel would loop forever.  The bound below never binds otherwise.
  const uint32_t max_steps = 8u * h.brick_size + 16u;
  for (uint32_t step = 0; bnf.x < bnf.y && hit.t == old_t && step < max_steps; step++) {
    const float3 hit_pos = add(ray_pos, scl(bnf.x, ray_dir));
    const float3 local_pos = scr(sub(hit_pos, bmin), scale);
    const float3 vp = f3(floorf(clampf(local_pos.x, 1e-6f, bs - 1e-6f)), floorf(clampf(local_pos.y, 1e-6f, bs - 1e-6f)),
                         floorf(clampf(local_pos.z, 1e-6f, bs - 1e-6f)));
    const float3 min_pos = add(bmin, scl(d, vp));
    const float3 max_pos = add(min_pos, scl(d, f3(1, 1, 1)));
    const float vmin = load_values(s, nd.z, vp, v_size, sz_inv, values);
    if (COUNT) cnt.voxels++;
    const float2 fnf = ray_box(ray_pos, inv, min_pos.x, min_pos.y, min_pos.z, max_pos.x, max_pos.y, max_pos.z);
    if (tNear < fnf.x && vmin <= 0.0f) {
      const float3 start_pos = add(ray_pos, scl(fnf.x, ray_dir));
      const float3 start_q = scr(sub(start_pos, min_pos), scale);
      const float qFar = (fnf.y - fnf.x) * scale;
      local_surface<COUNT>(pr, s, type, ray_dir, values, brick, d, 0.0f, qFar, fnf, start_q, hit, cnt);
    }
    bnf.x += mx(0.0f, fnf.y - bnf.x) + 1e-6f;
  }
  if (hit.t < old_t) {
    const uint32_t layout = h.aux_data & 0xFF000000u;
    if (layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN) {
      const float3 pos = add(ray_pos, scl(hit.t, ray_dir));
      const float3 dp = scr(sub(pos, bmin), 0.5f * sz);
      const uint32_t t_off = nd.z + v_size * v_size * v_size;
      const float w[8] = {(1 - dp.x) * (1 - dp.y) * (1 - dp.z), (1 - dp.x) * (1 - dp.y) * (dp.z),
                          (1 - dp.x) * (dp.y) * (1 - dp.z),     (1 - dp.x) * (dp.y) * (dp.z),
                          (dp.x) * (1 - dp.y) * (1 - dp.z),     (dp.x) * (1 - dp.y) * (dp.z),
                          (dp.x) * (dp.y) * (1 - dp.z),         (dp.x) * (dp.y) * (dp.z)};
      float3 col = f3(0, 0, 0);
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const float *c = &s.values_f[__ldg(&s.values[t_off + i])];
        const float3 ci = f3(w[i] * c[0], w[i] * c[1], w[i] * c[2]);
        col = i == 0 ? ci : add(col, ci);
      }
      col = f3(clampf(floorf(255.0f * col.x + 0.5f), 0.0f, 255.0f), clampf(floorf(255.0f * col.y + 0.5f), 0.0f, 255.0f),
               clampf(floorf(255.0f * col.z + 0.5f), 0.0f, 255.0f));
      hit.c0 = col.x + col.y / 256.0f;
      hit.c1 = col.z;
    }
  }
}

// SVS voxel: OctreeNodeIntersect + RayNodeIntersection, BVH/BVH2Common.cpp:126-153, 633-655
template <bool COUNT>
__device__ void svs_intersect(const DevScene &s, float3 ray_pos, float3 ray_dir, float tNear, uint32_t node_id,
                              Hit &hit, Counters &cnt) {
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.svs) + node_id);
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF);
  const float pz = float(nd.y >> 16), sz = float(nd.y & 0x0000FFFF);
  const float d_max = 2 * 1.73205081f / sz;
  const float3 min_pos = add(f3(-1, -1, -1), f3(2.0f * px / sz, 2.0f * py / sz, 2.0f * pz / sz));
  const float3 max_pos = add(min_pos, f3(2.0f * 1 / sz, 2.0f * 1 / sz, 2.0f * 1 / sz));
  const float3 size = sub(max_pos, min_pos);
  float values[8];
  // -d_max + 2*d_max*(1.0/255.0f)*q: the double literal promotes the sum to double
  const double c = double(2 * d_max) * (1.0 / 255.0);
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t word = (i < 4) ? nd.z : nd.w;
    const double q = double((word >> (8 * (i % 4))) & 0xFF);
    values[i] = float(double(-d_max) + c * q);
  }
  const float2 fnf = ray_box(ray_pos, safe_inverse(ray_dir), min_pos.x, min_pos.y, min_pos.z, max_pos.x, max_pos.y,
                             max_pos.z);
  const float3 start_pos = add(ray_pos, scl(fnf.x, ray_dir));
  const float d = mx(size.x, mx(size.y, size.z));
  const float3 start_q = f3((start_pos.x - min_pos.x) / d, (start_pos.y - min_pos.y) / d, (start_pos.z - min_pos.z) / d);
  const float qFar = (fnf.y - fnf.x) / d;
  const float qNear = tNear > fnf.x ? (tNear - fnf.x) / d : 0.0f;
  if (COUNT) { cnt.leaves++; cnt.voxels++; }
  if (qNear > 0.0f) return;
  local_surface<COUNT>(s.preset, s, LRT_TYPE_SDF_SVS, ray_dir, values, node_id, d, qNear, qFar, fnf, start_q, hit, cnt);
}

// IntersectAllTrianglesInLeaf, BVH/BVH2Common.cpp:2776-2840 (geometry normal)
template <bool COUNT>
__device__ void tri_intersect(const DevScene &s, float3 ray_pos, float3 ray_dir, float tNear, uint32_t start,
                              uint32_t count, Hit &hit, Counters &cnt) {
  for (uint32_t tri = start; tri < start + count; tri++) {
    const float4 a = __ldg(&s.tri_verts[3 * tri + 0]);
    const float4 b = __ldg(&s.tri_verts[3 * tri + 1]);
    const float4 c = __ldg(&s.tri_verts[3 * tri + 2]);
    const float3 A = f3(a.x, a.y, a.z), B = f3(b.x, b.y, b.z), C = f3(c.x, c.y, c.z);
    const float3 edge1 = sub(B, A), edge2 = sub(C, A);
    const float3 pvec = cross(ray_dir, edge2);
    const float3 tvec = sub(ray_pos, A);
    const float3 qvec = cross(tvec, edge1);
    const float invDet = 1.0f / dot(edge1, pvec);
    const float v = dot(tvec, pvec) * invDet;
    const float u = dot(qvec, ray_dir) * invDet;
    const float t = dot(edge2, qvec) * invDet;
    if (COUNT) cnt.voxels++;
    if (v >= -1e-6f && u >= -1e-6f && (u + v <= 1.0f + 1e-6f) && t > tNear && t < hit.t) {
      hit.t = t;
      hit.prim = tri;
      hit.geom = s.geom_id | (LRT_TYPE_MESH_TRIANGLE << 24);
      hit.c0 = u;
      hit.c1 = v;
      if (need_normal(s.preset.render_mode)) {
        const float3 n = normalize(matmul4x3(s.inst_inv_t, cross(edge1, edge2)));
        const float2 en = encode_normal(n);
        hit.c2 = en.x;
        hit.c3 = en.y;
      } else {
        hit.c2 = 0;
        hit.c3 = 0;
      }
    }
  }
}

// RayQuery_NearestHit (BVH/BVH2Common.cpp:3490-3559) over the 4-wide BVH.
// stopOnFirstHit (tFar <= 0) returns the first hit found (RayQuery_AnyHit).
template <int TYPE, bool COUNT>
__device__ void trace(const DevScene &s, float3 pos, float tNear, float3 dir, float tFar, Hit &hit, Counters &cnt) {
  const bool stop_first = (tFar <= 0.0f);
  if (stop_first) tFar *= -1.0f;
  hit.t = tFar;
  hit.prim = kMiss;
  hit.geom = kMiss;
  hit.c0 = 1.0f;
  hit.c1 = hit.c2 = hit.c3 = 0.0f;
  {  // TLAS: one leaf node holding the instance box (:3508-3529)
    const float3 invw = safe_inverse(dir);
    const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                              s.inst_bmax[1], s.inst_bmax[2]);
    if (!((bh.x <= bh.y) && (bh.y > tNear) && (bh.x < hit.t))) return;
  }
  const float3 rp = matmul4x3(s.inst_inv, pos);
  const float3 rd = matmul3x3(s.inst_inv, dir);
  const float3 inv = safe_inverse(rd);
  const float tNearSdf = mx(tNear, 0.1f);   // SDF bias passed to every leaf type (:3472-3476)

  uint32_t st_ref[kStackSize];
  float st_t[kStackSize];
  int sp = 0;
  st_ref[sp] = 0;            // root wide node
  st_t[sp] = -3.4e38f;
  sp++;
  while (sp > 0) {
    sp--;
    const uint32_t ref = st_ref[sp];
    if (st_t[sp] > hit.t) continue;
    if (ref & kLeafBit) {
      const uint32_t payload = ref & ~kLeafBit;
      const float t_before = hit.t;
      if (TYPE == LRT_TYPE_MESH_TRIANGLE)
        tri_intersect<COUNT>(s, rp, rd, tNearSdf, payload & 0x00FFFFFFu, (payload >> 24) & 0x7Fu, hit, cnt);
      else if (TYPE == LRT_TYPE_SDF_SVS)
        svs_intersect<COUNT>(s, rp, rd, tNearSdf, payload, hit, cnt);
      else
        brick_intersect<COUNT>(s, rp, rd, inv, tNearSdf, payload, hit, cnt);
      if (stop_first && hit.t < t_before) break;
      continue;
    }
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
    float kt[4];
    uint32_t kr[4];
    int nk = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const float2 tm = ray_box(rp, inv, lxa[i], lya[i], lza[i], hxa[i], hya[i], hza[i]);
      const bool h = (tm.x <= tm.y) && (tm.y >= tNear) && (tm.x <= hit.t) && cha[i] != kEmptyChild;
      if (h) { kt[nk] = tm.x; kr[nk] = cha[i]; nk++; }
    }
    // push far-to-near so the nearest child is popped first
    for (int i = 1; i < nk; i++) {
      const float tv = kt[i];
      const uint32_t rv = kr[i];
      int j = i - 1;
      while (j >= 0 && kt[j] < tv) { kt[j + 1] = kt[j]; kr[j + 1] = kr[j]; j--; }
      kt[j + 1] = tv;
      kr[j + 1] = rv;
    }
    // The host rejects trees deeper than the stack allows ((W-1)*depth + 1 entries),
    // so this bound never drops an entry.
    for (int i = 0; i < nk; i++) {
      if (sp < kStackSize) { st_ref[sp] = kr[i]; st_t[sp] = kt[i]; sp++; }
    }
  }
}

__device__ __forceinline__ void mat_vec4(const float *m, const float v[4], float r[4]) {
#pragma unroll
  for (int i = 0; i < 4; i++) r[i] = m[i * 4 + 0] * v[0] + m[i * 4 + 1] * v[1] + m[i * 4 + 2] * v[2] + m[i * 4 + 3] * v[3];
}

// kernel_InitEyeRay, Renderer/eye_ray.cpp:146-160 with EyeRayDirNormalized and
// transform_ray3f, render_common.h:25-55
__device__ __forceinline__ void eye_ray(uint32_t x, uint32_t y, uint32_t w, uint32_t h, float dx, float dy,
                                        const float *proj_inv, const float *wv_inv, float3 &pos, float3 &dir) {
  const float fx = (float(x) + dx) / float(w), fy = (float(y) + dy) / float(h);
  const float v[4] = {2.0f * fx - 1.0f, -2.0f * fy + 1.0f, 1.0f, 1.0f};
  float r[4];
  mat_vec4(proj_inv, v, r);
  const float ww = r[3];
  float3 d0 = normalize(f3(r[0] / ww, r[1] / ww, r[2] / ww));
  const float3 p00 = f3(0, 0, 0);
  const float3 p0 = matmul4x3(wv_inv, p00);
  const float3 p2 = matmul4x3(wv_inv, add(p00, scl(100.0f, d0)));
  pos = p0;
  dir = normalize(sub(p2, p0));
}

// kernel_RayTrace shading, Renderer/eye_ray.cpp:162-489 (MASK, LAMBERT_NO_TEX,
// LAMBERT for coloured bricks, DEPTH, LINEAR_DEPTH, INVERSE_LINEAR_DEPTH, NORMAL)
__device__ float4 shade(const DevScene &s, const Hit &hit, float3 dir) {
  if (hit.prim == kMiss) return make_float4(0, 0, 0, 1);
  const float z = hit.t, z_near = 0.1f, z_far = 10;
  const uint32_t type = hit.geom >> 24;
  float3 norm;
  if (type == LRT_TYPE_MESH_TRIANGLE) {
    const float4 a = s.tri_verts[3 * hit.prim + 0], b = s.tri_verts[3 * hit.prim + 1], c = s.tri_verts[3 * hit.prim + 2];
    const float3 e1 = f3(b.x - a.x, b.y - a.y, b.z - a.z), e2 = f3(c.x - a.x, c.y - a.y, c.z - a.z);
    norm = normalize(matmul4x3(s.inst_inv_t, cross(e1, e2)));
  } else {
    norm = decode_normal(hit.c2, hit.c3);
  }
  const float ns = signf(dot(scl(-1.0f, dir), norm));
  norm = scl(ns, norm);
  switch (s.preset.render_mode) {
    case LRT_RENDER_MODE_MASK: return make_float4(1, 1, 1, 1);
    case LRT_RENDER_MODE_DEPTH: { const float d = (1 / z - 1 / z_near) / (1 / z_far - 1 / z_near); return make_float4(d, d, d, 1); }
    case LRT_RENDER_MODE_LINEAR_DEPTH: { const float d = ((z - z_near) / (z_far - z_near)); return make_float4(d, d, d, 1); }
    case LRT_RENDER_MODE_INVERSE_LINEAR_DEPTH: { const float d = 1 - ((z - z_near) / (z_far - z_near)); return make_float4(d, d, d, 1); }
    case LRT_RENDER_MODE_NORMAL: return make_float4(fabsf(norm.x), fabsf(norm.y), fabsf(norm.z), 1);
    case LRT_RENDER_MODE_LAMBERT_NO_TEX:
    case LRT_RENDER_MODE_LAMBERT: {
      float3 color = f3(1, 1, 1);
      if (s.preset.render_mode == LRT_RENDER_MODE_LAMBERT && type == LRT_TYPE_SDF_SBS_COL) {
        color.x = roundf(hit.c0) / 255.0f;
        color.y = hit.c0 - floorf(hit.c0);
        color.z = roundf(hit.c1) / 255.0f;
      }
      // default lights, Renderer/eye_ray_host.cpp:40
      const float3 ldir = normalize(f3(1, 1, 1));
      const float lc = 2.0f / 3.0f;
      float3 fc = f3(0, 0, 0);
      const float q = mx(0.0f, dot(norm, ldir));
      fc = add(fc, scl(q, mul(f3(lc, lc, lc), color)));
      fc = add(fc, mul(f3(0.25f, 0.25f, 0.25f), color));
      return make_float4(fc.x, fc.y, fc.z, 1);
    }
    default: return make_float4(1, 0, 1, 1);
  }
}

__device__ __forceinline__ uint32_t encode_rgba8(float4 c) {   // Renderer/eye_ray.cpp:111-115
  const uint32_t r = uint32_t(255 * clampf(c.x, 0.0f, 1.0f)), g = uint32_t(255 * clampf(c.y, 0.0f, 1.0f));
  const uint32_t b = uint32_t(255 * clampf(c.z, 0.0f, 1.0f)), a = uint32_t(255 * clampf(c.w, 0.0f, 1.0f));
  return (a << 24) | (b << 16) | (g << 8) | r;
}

// Persistent render kernel: each warp pulls 8x4-pixel tiles of the flattened
// multi-view tile space from a global queue head and traces one ray per lane.
template <int TYPE, bool COUNT>
__global__ void __launch_bounds__(128) render_kernel(DevScene s, RenderLaunch L) {
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
    const uint32_t lt = tile - V.tile_offset;
    const uint32_t x = (lt % V.tiles_x) * 8u + (lane & 7u), y = (lt / V.tiles_x) * 4u + (lane >> 3);
    if (x >= V.width || y >= V.height) continue;   // all lanes meet again at the queue shuffle
    float4 acc = make_float4(0, 0, 0, 0);
    Hit first;
    for (uint32_t si = 0; si < spp; si++) {
      const float dx = i_spp_sqrt * float(double(si / spp_sqrt) + 0.5);
      const float dy = i_spp_sqrt * float(double(si % spp_sqrt) + 0.5);
      float3 pos, dir;
      eye_ray(x, y, V.width, V.height, dx, dy, V.proj_inv, V.wv_inv, pos, dir);
      Hit hit;
      trace<TYPE, COUNT>(s, pos, 0.0f, dir, 1e9f, hit, cnt);
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

template <int TYPE>
static cudaError_t launch_render_t(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count) {
  int per_sm = 0;
  cudaError_t e = count ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_kernel<TYPE, true>, 128, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_kernel<TYPE, false>, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  const uint32_t warps_needed = L.total_tiles;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (warps_needed + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  if (count) dev::render_kernel<TYPE, true><<<blocks, 128, 0, st>>>(s, L);
  else dev::render_kernel<TYPE, false><<<blocks, 128, 0, st>>>(s, L);
  return cudaGetLastError();
}

cudaError_t launch_render(const DevScene &s, const RenderLaunch &L, int num_sms, cudaStream_t st, bool count) {
  switch (s.type) {
    case LRT_TYPE_MESH_TRIANGLE: return launch_render_t<LRT_TYPE_MESH_TRIANGLE>(s, L, num_sms, st, count);
    case LRT_TYPE_SDF_SVS: return launch_render_t<LRT_TYPE_SDF_SVS>(s, L, num_sms, st, count);
    default: return launch_render_t<LRT_TYPE_SDF_SBS>(s, L, num_sms, st, count);
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
