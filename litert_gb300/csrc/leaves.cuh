// Leaf intersectors, eye rays and shading shared by the primary-ray kernels.
// Each function restates a reference function in its FP32 operation order
// (see trace_common.cuh); the citing comment names the reference lines.
#pragma once
#include "trace_common.cuh"

namespace lrt {
namespace dev {

// LocalSurfaceIntersection, BVH/BVH2Common.cpp:274-631 (trilinear; ST, ANALYTIC,
// NEWTON, BBOX, IT).  Updates `hit` when the crossing is closer.
template <bool COUNT, int MODE = -1>
__device__ __forceinline__ void local_surface(const lrt_preset &pr, const DevScene &s, uint32_t type, float3 ray_dir,
                                              const float values[8], uint32_t prim_id, float d, float qNear,
                                              float qFar, float2 fNearFar, float3 start_q, Hit &hit,
                                              Counters &cnt) {
  const uint32_t mode = MODE >= 0 ? uint32_t(MODE) : pr.sdf_node_intersect;
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

  if (start_dist <= EPS || mode == LRT_INTERSECT_BBOX) {
    is_hit = true;
  } else if (mode == LRT_INTERSECT_ST) {
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

    if (mode == LRT_INTERSECT_NEWTON) {                             // :437-522
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
    } else if (mode == LRT_INTERSECT_ANALYTIC) {                     // :367-436
      float x1 = 1000, x2 = 1000, x3 = 1000;
      if (fabsf(c3) > 1e-2) {
        const float aa = c2 / c3, b = c1 / c3, c = c0 / c3;
        const float Q = (aa * aa - 3 * b) / 9;
        const float R = (2 * aa * aa - 9 * aa * b + 27 * c) / 54;
        const float Q3 = Q * Q * Q;
        // The reference's unqualified sqrt(float) is ::sqrt(double): these
        // expressions are evaluated in double, with std::cos(float) in float.
        if (R * R < Q3) {
          const float theta = float(acos(double(R) / sqrt(double(Q3))));
          x1 = float(-2 * sqrt(double(Q)) * double(cosf(theta / 3)) - double(aa / 3));
          x2 = float(-2 * sqrt(double(Q)) * double(cosf((theta + 2 * 3.14159265358979323846f) / 3)) - double(aa / 3));
          x3 = float(-2 * sqrt(double(Q)) * double(cosf((theta - 2 * 3.14159265358979323846f) / 3)) - double(aa / 3));
        } else {
          const float A = float(double(-signf(R)) * pow(double(fabsf(R)) + sqrt(double(R * R - Q3)), double(1.0f / 3.0f)));
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

// Decode of one stored distance value, BVH/BVH2Common.cpp:749-759: DX layout
// fixed point -d_max + mult*q; `lg` = log2(values per 32-bit word).
__device__ __forceinline__ float decode_dx(const uint32_t *data, uint32_t vId, uint32_t lg, uint32_t bits,
                                           uint32_t max_val, float d_max, float mult) {
  const uint32_t q = (__ldg(&data[vId >> lg]) >> (bits * (vId & ((1u << lg) - 1u)))) & max_val;
  return -d_max + mult * float(q);
}

// load_distance_values, BVH/BVH2Common.cpp:725-762 (SBS_v_to_i, sdfScene/sdf_scene.h:201-204),
// reading the brick from global memory.
struct GlobalLoader {
  const DevScene *s;
  const uint32_t *data;   // brick's first word
  uint32_t v_size, pad, lg, bits, max_val;
  float d_max, mult;
  bool indexed;
  __device__ __forceinline__ GlobalLoader(const DevScene &sc, uint32_t data_offset, float sz_inv) {
    const lrt_sbs_header &h = sc.sbs_hdr;
    s = &sc;
    data = sc.values + data_offset;
    v_size = h.brick_size + 2 * h.brick_pad + 1;
    pad = h.brick_pad;
    const uint32_t layout = h.aux_data & 0xFF000000u;
    indexed = layout == LRT_SBS_LAYOUT_ID32F_IRGB32F || layout == LRT_SBS_LAYOUT_ID32F_IRGB32F_IN;
    lg = h.bytes_per_value == 4 ? 0u : (h.bytes_per_value == 2 ? 1u : 2u);
    bits = 8 * h.bytes_per_value;
    max_val = h.bytes_per_value == 4 ? 0xFFFFFFFFu : ((1u << bits) - 1);
    d_max = 1.73205081f * sz_inv;
    mult = 2 * d_max / float(max_val);
  }
  __device__ __forceinline__ float load(float3 vp, float values[8]) const {
    float vmin = 1e6f;
    const uint32_t ix = uint32_t(vp.x), iy = uint32_t(vp.y), iz = uint32_t(vp.z);
#pragma unroll
    for (int i = 0; i < 8; i++) {
      const uint32_t vId = (ix + ((i & 4) >> 2) + pad) * v_size * v_size + (iy + ((i & 2) >> 1) + pad) * v_size +
                           (iz + (i & 1) + pad);
      values[i] = indexed ? __ldg(&s->values_f[__ldg(&data[vId])]) : decode_dx(data, vId, lg, bits, max_val, d_max, mult);
      vmin = mn(vmin, values[i]);
    }
    return vmin;
  }
};

// The same corner fetch from a brick already decoded into shared memory
// (v_size^3 floats in SBS_v_to_i order).
struct SharedLoader {
  const float *vals;
  uint32_t v_size, pad;
  __device__ __forceinline__ float load(float3 vp, float values[8]) const {
    float vmin = 1e6f;
    const uint32_t base = (uint32_t(vp.x) + pad) * v_size * v_size + (uint32_t(vp.y) + pad) * v_size + uint32_t(vp.z) + pad;
    const uint32_t vv = v_size * v_size;
    const uint32_t off[8] = {0u, 1u, v_size, v_size + 1u, vv, vv + 1u, vv + v_size, vv + v_size + 1u};
#pragma unroll
    for (int i = 0; i < 8; i++) {
      values[i] = vals[base + off[i]];
      vmin = mn(vmin, values[i]);
    }
    return vmin;
  }
};

// eval_dist_trilinear_diff, BVH/BVH2Common.cpp:656-686 (a + -(b) is a - b exactly)
__device__ __forceinline__ float3 tri_diff(const float v[8], float3 dp) {
  const float dx = -(1 - dp.y) * (1 - dp.z) * v[0] - (1 - dp.y) * (dp.z) * v[1] - (dp.y) * (1 - dp.z) * v[2] -
                   (dp.y) * (dp.z) * v[3] + (1 - dp.y) * (1 - dp.z) * v[4] + (1 - dp.y) * (dp.z) * v[5] +
                   (dp.y) * (1 - dp.z) * v[6] + (dp.y) * (dp.z) * v[7];
  const float dy = -(1 - dp.x) * (1 - dp.z) * v[0] - (1 - dp.x) * (dp.z) * v[1] + (1 - dp.x) * (1 - dp.z) * v[2] +
                   (1 - dp.x) * (dp.z) * v[3] - (dp.x) * (1 - dp.z) * v[4] - (dp.x) * (dp.z) * v[5] +
                   (dp.x) * (1 - dp.z) * v[6] + (dp.x) * (dp.z) * v[7];
  const float dz = -(1 - dp.x) * (1 - dp.y) * v[0] + (1 - dp.x) * (1 - dp.y) * v[1] - (1 - dp.x) * (dp.y) * v[2] +
                   (1 - dp.x) * (dp.y) * v[3] - (dp.x) * (1 - dp.y) * v[4] + (dp.x) * (1 - dp.y) * v[5] -
                   (dp.x) * (dp.y) * v[6] + (dp.x) * (dp.y) * v[7];
  return f3(dx, dy, dz);
}

// NORMAL_MODE_SDF_SMOOTHED on the ID32F_IRGB32F_IN layout (BVH/BVH2Common.cpp:838-905):
// the normals of the 8 voxels around the hit, read across brick borders through the
// brick's 27-neighbour table, blended with weights that switch over +-beta of the
// voxel centre.  Compiled only into the kernels instantiated for this layout and mode.
__device__ __forceinline__ void smooth_normal(const DevScene &s, uint32_t node, float3 vox, float3 start_q, float fnear,
                                           float d, float3 ray_dir, uint32_t v_size, Hit &hit) {
  const lrt_sbs_header &h = s.sbs_hdr;
  const float beta = 0.5f;
  const float3 dp = add(start_q, scl((hit.t - fnear) / d, ray_dir));
  auto step01 = [](float e0, float e1, float x) { return clampf((x - e0) / (e1 - e0), 0.0f, 1.0f); };
  const float3 nmq = f3(dp.x < 0.5f ? step01(-beta, beta, dp.x) : step01(-beta, beta, dp.x - 1.0f),
                        dp.y < 0.5f ? step01(-beta, beta, dp.y) : step01(-beta, beta, dp.y - 1.0f),
                        dp.z < 0.5f ? step01(-beta, beta, dp.z) : step01(-beta, beta, dp.z - 1.0f));
  const int v0x = int(dp.x < 0.5f ? vox.x - 1 : vox.x), v0y = int(dp.y < 0.5f ? vox.y - 1 : vox.y),
            v0z = int(dp.z < 0.5f ? vox.z - 1 : vox.z);
  const int bsz = int(h.brick_size);
  const float bsf = float(h.brick_size);
  const uint32_t v3 = v_size * v_size * v_size;
  float3 sm = f3(0, 0, 0);
#pragma unroll 1
  for (int i = 0; i < 8; i++) {
    const int vx = v0x + ((i & 4) >> 2), vy = v0y + ((i & 2) >> 1), vz = v0z + (i & 1);
    const int bx = vx >= 0 ? (vx < bsz ? 0 : 1) : -1, by = vy >= 0 ? (vy < bsz ? 0 : 1) : -1,
              bz = vz >= 0 ? (vz < bsz ? 0 : 1) : -1;
    const uint32_t nb = uint32_t(9 * (bx + 1) + 3 * (by + 1) + (bz + 1));
    const float3 dvox = sub(f3(float(vx), float(vy), float(vz)), vox);
    uint32_t nid;
    float3 nvp;
    if (nb == 9 + 3 + 1) {
      nid = node;
      nvp = f3(float(vx), float(vy), float(vz));
    } else {
      nid = __ldg(&s.values[__ldg(&s.bricks[node].data_offset) + v3 + 8 + nb]);
      nvp = sub(f3(float(vx), float(vy), float(vz)), f3(bsf * float(bx), bsf * float(by), bsf * float(bz)));
    }
    float3 n = f3(0, 0, 0);
    if (nid != 0x80000000u) {
      const uint32_t off = __ldg(&s.bricks[nid].data_offset);
      float vals[8];
#pragma unroll
      for (int c = 0; c < 8; c++) {
        const uint32_t vId = (uint32_t(nvp.x) + ((c & 4) >> 2) + h.brick_pad) * v_size * v_size +
                             (uint32_t(nvp.y) + ((c & 2) >> 1) + h.brick_pad) * v_size +
                             (uint32_t(nvp.z) + (c & 1) + h.brick_pad);
        vals[c] = __ldg(&s.values_f[__ldg(&s.values[off + vId])]);
      }
      n = normalize(tri_diff(vals, sub(dp, dvox)));
    }
    const float w = i == 0 ? (1 - nmq.x) * (1 - nmq.y) * (1 - nmq.z)
                  : i == 1 ? (1 - nmq.x) * (1 - nmq.y) * (nmq.z)
                  : i == 2 ? (1 - nmq.x) * (nmq.y) * (1 - nmq.z)
                  : i == 3 ? (1 - nmq.x) * (nmq.y) * (nmq.z)
                  : i == 4 ? (nmq.x) * (1 - nmq.y) * (1 - nmq.z)
                  : i == 5 ? (nmq.x) * (1 - nmq.y) * (nmq.z)
                  : i == 6 ? (nmq.x) * (nmq.y) * (1 - nmq.z)
                           : (nmq.x) * (nmq.y) * (nmq.z);
    const float3 wn = scl(w, n);
    sm = i == 0 ? wn : add(sm, wn);
  }
  const float2 en = encode_normal(normalize(sm));
  hit.c2 = en.x;
  hit.c3 = en.y;
}

// The hit's colour or texture coordinates for the layouts that carry them
// (OctreeBrickIntersect, BVH/BVH2Common.cpp:912-982), out of line: the plain DX
// layout never reaches it, so the leaf loop of every kernel stays small.
static __device__ __noinline__ void brick_colour(const DevScene &s, uint4 nd, float3 bmin, float sz, uint32_t v_size,
                                                 float3 ray_pos, float3 ray_dir, Hit &hit) {
  const lrt_sbs_header &h = s.sbs_hdr;
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
  } else if (layout == LRT_SBS_LAYOUT_DX_UV16 || layout == LRT_SBS_LAYOUT_DX_RGB8) {
    // 8 words after the packed distances: 16-bit texture coordinates or RGB8 colours
    const float3 pos = add(ray_pos, scl(hit.t, ray_dir));
    const float3 dp = scr(sub(pos, bmin), 0.5f * sz);
    const uint32_t vpi = 4u / h.bytes_per_value;
    const uint32_t *tw = s.values + nd.z + (v_size * v_size * v_size + vpi - 1) / vpi;
    const float w[8] = {(1 - dp.x) * (1 - dp.y) * (1 - dp.z), (1 - dp.x) * (1 - dp.y) * (dp.z),
                        (1 - dp.x) * (dp.y) * (1 - dp.z),     (1 - dp.x) * (dp.y) * (dp.z),
                        (dp.x) * (1 - dp.y) * (1 - dp.z),     (dp.x) * (1 - dp.y) * (dp.z),
                        (dp.x) * (dp.y) * (1 - dp.z),         (dp.x) * (dp.y) * (dp.z)};
    if (layout == LRT_SBS_LAYOUT_DX_UV16) {
      float u = 0, v = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const uint32_t q = __ldg(&tw[i]);
        const float ui = w[i] * (1.5259022e-5f * float(q >> 16));
        const float vi = w[i] * (1.5259022e-5f * float(q & 0xFFFFu));
        u = i == 0 ? ui : u + ui;
        v = i == 0 ? vi : v + vi;
      }
      hit.c0 = u;
      hit.c1 = v;
    } else {
      float3 col = f3(0, 0, 0);
#pragma unroll
      for (int i = 0; i < 8; i++) {
        const uint32_t q = __ldg(&tw[i]);
        const float3 ci = f3(w[i] * float(q & 0xFFu), w[i] * float((q >> 8) & 0xFFu), w[i] * float((q >> 16) & 0xFFu));
        col = i == 0 ? ci : add(col, ci);
      }
      col = f3(clampf(floorf(col.x + 0.5f), 0.0f, 255.0f), clampf(floorf(col.y + 0.5f), 0.0f, 255.0f),
               clampf(floorf(col.z + 0.5f), 0.0f, 255.0f));
      hit.c0 = col.x + col.y / 256.0f;
      hit.c1 = col.z;
    }
  }
}

// OctreeBrickIntersect, BVH/BVH2Common.cpp:764-984 (trilinear, colour for indexed
// layouts).  The voxel walk is the reference's: the voxel is recomputed from the
// current entry distance, the distance advances past the voxel's exit plane by
// 1e-6, and a voxel is intersected when its entry lies beyond tNear and a corner
// value is <= 0.  Two exact shortcuts: the "a corner is <= 0" test reads the
// brick's occupancy bit (built from the same decoded values) so empty voxels
// load no corners, and the exit distance is taken from the far planes alone --
// for each axis max(lo, hi) is the plane the ray direction points to, so the
// value equals RayBoxIntersection2's.  The near planes are evaluated only in
// occupied voxels.
//
// start_t (default: no effect) lets the walk begin at a later distance; the
// proposal path passes the entry of a voxel it has shown every earlier voxel of
// the segment to be empty, where the reference's walk would run no finder.
// FEAT: bit 0 smoothed SDF normals (NORMAL_MODE_SDF_SMOOTHED), bit 1 the hit
// colour computed in this brick as the reference does (kept for ST_ITERATIONS,
// where primId no longer names the brick; otherwise hit_colour computes it once
// for the final hit, which gives the same values: the last brick that reports a
// hit is the hit brick), bit 4 (value 16) the walk's position and voxel planes as
// one FMA each (for the kernels compiled with contraction).
template <bool COUNT, bool STAGED, int MODE = -1, int FEAT = 0>
__device__ void brick_intersect(const DevScene &s, float3 ray_pos, float3 ray_dir, float3 inv, float tNear,
                                uint32_t brick, Hit &hit, Counters &cnt, const float *staged = nullptr,
                                float start_t = -3.4e38f) {
  const lrt_sbs_header &h = s.sbs_hdr;
  const lrt_preset &pr = s.preset;
  const uint32_t type = s.type;
  const uint32_t v_size = h.brick_size + 2 * h.brick_pad + 1;
  const uint32_t bsz = h.brick_size;
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF);
  const float pz = float(nd.y >> 16), sz = float(nd.y & 0x0000FFFF);
  const float sz_inv = 2.0f / sz;
  const float bs = float(bsz);
  const float d = 2.0f / (sz * bs);
  const float3 bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(px, py, pz)));
  const float3 bmax = add(bmin, scl(sz_inv, f3(1, 1, 1)));
  // FEAT bit 4: slab and voxel-plane distances p * inv + noi, local position lp0 + t * rds
  constexpr bool kFma = (FEAT & 16) != 0;
  const float3 noi = f3(-(ray_pos.x * inv.x), -(ray_pos.y * inv.y), -(ray_pos.z * inv.z));
  float2 bnf = kFma ? ray_box_fma(inv, noi, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z)
                    : ray_box(ray_pos, inv, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z);
  bnf.x = fmx(bnf.x, start_t);
  const float old_t = hit.t;
  const float scale = 0.5f * sz * bs;
  const uint32_t *occ = s.occ + size_t(brick) * s.occ_words;
  const bool posx = inv.x > 0.0f, posy = inv.y > 0.0f, posz = inv.z > 0.0f;
  const float3 lp0 = scr(sub(ray_pos, bmin), scale), rds = scl(scale, ray_dir);
  float values[8];
  if (COUNT) cnt.leaves++;
  const uint32_t max_steps = walk_step_bound(bsz, bnf.y - bnf.x);
  const GlobalLoader gl(s, nd.z, sz_inv);
  const SharedLoader sl{staged, v_size, h.brick_pad};
  // Two nested loops: the inner one steps through voxels until one needs the
  // finder (occupied, entered after tNear, some corner value <= 0) or the brick
  // ends; the finder runs after it.  A lane's sequence of voxels and finder calls
  // is the single loop's, but the lanes of a warp that reach a candidate voxel
  // after different numbers of steps run the finder together.
  uint32_t step = 0;
  while (hit.t == old_t) {
    bool cand = false;
    float3 vp, min_pos;
    float2 fnf;
    float exit_t;
    while (bnf.x < bnf.y && step < max_steps) {
      float3 local_pos;
      if (kFma) {
        local_pos = f3(fmaf(bnf.x, rds.x, lp0.x), fmaf(bnf.x, rds.y, lp0.y), fmaf(bnf.x, rds.z, lp0.z));
      } else {
        const float3 hit_pos = add(ray_pos, scl(bnf.x, ray_dir));
        local_pos = scr(sub(hit_pos, bmin), scale);
      }
      vp = f3(floorf(fmn(fmx(local_pos.x, 1e-6f), bs - 1e-6f)), floorf(fmn(fmx(local_pos.y, 1e-6f), bs - 1e-6f)),
              floorf(fmn(fmx(local_pos.z, 1e-6f), bs - 1e-6f)));
      min_pos = add(bmin, scl(d, vp));
      // exit distance: far plane per axis (max_pos = min_pos + d*1)
      const float ex = posx ? min_pos.x + d : min_pos.x, ey = posy ? min_pos.y + d : min_pos.y,
                  ez = posz ? min_pos.z + d : min_pos.z;
      const float fx = kFma ? fmaf(ex, inv.x, noi.x) : inv.x * (ex - ray_pos.x);
      const float fy = kFma ? fmaf(ey, inv.y, noi.y) : inv.y * (ey - ray_pos.y);
      const float fz = kFma ? fmaf(ez, inv.z, noi.z) : inv.z * (ez - ray_pos.z);
      exit_t = fmn(fmn(fx, fy), fz);
      // (x * bsz + y) * bsz + z formed in float (integers below 2^24: exact), one conversion
      const uint32_t vid = uint32_t(fmaf(fmaf(vp.x, bs, vp.y), bs, vp.z));
      step++;
      if (COUNT) cnt.voxels++;
      if ((__ldg(&occ[vid >> 5]) >> (vid & 31u)) & 1u) {
        const float px_ = posx ? min_pos.x : min_pos.x + d, py_ = posy ? min_pos.y : min_pos.y + d,
                    pz_ = posz ? min_pos.z : min_pos.z + d;
        const float nx = kFma ? fmaf(px_, inv.x, noi.x) : inv.x * (px_ - ray_pos.x);
        const float ny = kFma ? fmaf(py_, inv.y, noi.y) : inv.y * (py_ - ray_pos.y);
        const float nz = kFma ? fmaf(pz_, inv.z, noi.z) : inv.z * (pz_ - ray_pos.z);
        fnf = make_float2(fmx(fmx(nx, ny), nz), exit_t);
        if (tNear < fnf.x) {
          float vmin;
          if (STAGED) vmin = sl.load(vp, values);
          else vmin = gl.load(vp, values);
          if (vmin <= 0.0f) {
            cand = true;
            break;
          }
        }
      }
      if (kFma) bnf.x = fmx(bnf.x, exit_t) + 1e-6f;
      else bnf.x += fmx(0.0f, exit_t - bnf.x) + 1e-6f;   // the reference's rounding: t + (step + 1e-6)
    }
    if (!cand) break;
    const float3 start_pos = add(ray_pos, scl(fnf.x, ray_dir));
    const float3 start_q = scr(sub(start_pos, min_pos), scale);
    const float qFar = (fnf.y - fnf.x) * scale;
    local_surface<COUNT, MODE>(pr, s, type, ray_dir, values, brick, d, 0.0f, qFar, fnf, start_q, hit, cnt);
    if ((FEAT & 1) && hit.t != old_t) smooth_normal(s, brick, vp, start_q, fnf.x, d, ray_dir, v_size, hit);
    if (kFma) bnf.x = fmx(bnf.x, exit_t) + 1e-6f;
    else bnf.x += fmx(0.0f, exit_t - bnf.x) + 1e-6f;   // the reference's rounding: t + (step + 1e-6)
  }
  if ((FEAT & 2) && hit.t < old_t && (h.aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_DX &&
      (h.aux_data & 0xFF000000u) != LRT_SBS_LAYOUT_UNDEFINED)
    brick_colour(s, nd, bmin, sz, v_size, ray_pos, ray_dir, hit);
}

// The colour / texture coordinates of the final hit of an SBS with a layout that
// carries them, from its brick (hit.prim) -- once per ray instead of in the leaf
// loop.  pos / dir: the world-space ray, taken to object space as the traversal does.
__device__ __forceinline__ void hit_colour(const DevScene &s, float3 pos, float3 dir, Hit &hit) {
  const uint32_t layout = s.sbs_hdr.aux_data & 0xFF000000u;
  if (hit.prim == kMiss || layout == LRT_SBS_LAYOUT_DX || layout == LRT_SBS_LAYOUT_UNDEFINED) return;
  const float3 ray_pos = matmul4x3(s.inst_inv, pos), ray_dir = matmul3x3(s.inst_inv, dir);
  const lrt_sbs_header &h = s.sbs_hdr;
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + hit.prim);
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF);
  const float pz = float(nd.y >> 16), sz = float(nd.y & 0x0000FFFF);
  const float3 bmin = add(f3(-1, -1, -1), scl(2.0f / sz, f3(px, py, pz)));
  brick_colour(s, nd, bmin, sz, h.brick_size + 2 * h.brick_pad + 1, ray_pos, ray_dir, hit);
}

// SVS voxel: OctreeNodeIntersect + RayNodeIntersection, BVH/BVH2Common.cpp:126-153, 633-655
template <bool COUNT, int MODE = -1>
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
  local_surface<COUNT, MODE>(s.preset, s, LRT_TYPE_SDF_SVS, ray_dir, values, node_id, d, qNear, qFar, fnf, start_q, hit, cnt);
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


// kernel_RayTrace shading, Renderer/eye_ray.cpp:162-489 (MASK, LAMBERT_NO_TEX,
// LAMBERT for coloured bricks, DEPTH, LINEAR_DEPTH, INVERSE_LINEAR_DEPTH, NORMAL)
// MultiRenderer::m_palette (Renderer/eye_ray.h:235-241): the reference's 20 colours,
// kept identical because PRIMITIVE / TYPE / GEOM images are compared with it
__device__ __forceinline__ uint32_t palette_color(uint32_t i) {
  constexpr uint32_t P[20] = {0xffe6194bu, 0xff3cb44bu, 0xffffe119u, 0xff0082c8u, 0xfff58231u, 0xff911eb4u, 0xff46f0f0u,
                              0xfff032e6u, 0xffd2f53cu, 0xfffabebeu, 0xff008080u, 0xffe6beffu, 0xffaa6e28u, 0xfffffac8u,
                              0xff800000u, 0xffaaffc3u, 0xff808000u, 0xffffd8b1u, 0xff000080u, 0xff808080u};
  return P[i % 20u];
}
// decode_RGBA8, Renderer/eye_ray.cpp:15-19
__device__ __forceinline__ float4 decode_rgba8(uint32_t c) {
  return make_float4(float(c & 0xFF) * (1.0f / 255.0f), float((c >> 8) & 0xFF) * (1.0f / 255.0f),
                     float((c >> 16) & 0xFF) * (1.0f / 255.0f), float((c >> 24) & 0xFF) * (1.0f / 255.0f));
}

// The less common shading modes of kernel_RayTrace, out of line so that the
// render kernels carry only a call for them.
static __device__ __noinline__ float4 shade_extra(const DevScene &s, const Hit &hit, uint32_t type, float z,
                                                  float3 pos, float3 dir) {
  switch (s.preset.render_mode) {
    case LRT_RENDER_MODE_PRIMITIVE:   // the reference's primId: original triangle ids
      return decode_rgba8(palette_color(type == LRT_TYPE_MESH_TRIANGLE ? s.prim_indices[hit.prim] : hit.prim));
    case LRT_RENDER_MODE_TYPE: return decode_rgba8(palette_color(type));
    case LRT_RENDER_MODE_GEOM: return decode_rgba8(palette_color(hit.geom & 0x00FFFFFFu));
    case LRT_RENDER_MODE_BARYCENTRIC: return make_float4(hit.c0, hit.c1, 1 - hit.c0 - hit.c1, 1);
    case LRT_RENDER_MODE_ST_ITERATIONS: {   // the finder stored its iteration count as primId
      const uint32_t it = type == LRT_TYPE_MESH_TRIANGLE ? s.prim_indices[hit.prim] : hit.prim;
      if (it == 0) return make_float4(0.5f, 0.5f, 0.5f, 1);
      if (it <= 64) {
        const float q = clampf(float(it) / 64, 0.0f, 1.0f), r = 1 - q;
        return make_float4(q * 0.0f + r * 0.0f, q * 0.0f + r * 1.0f, q * 1.0f + r * 0.0f, q * 1.0f + r * 1.0f);
      }
      const float q = clampf(float(it - 64) / (256 - 64), 0.0f, 1.0f), r = 1 - q;
      return make_float4(q * 1.0f + r * 0.0f, q * 0.0f + r * 0.0f, q * 0.0f + r * 1.0f, q * 1.0f + r * 1.0f);
    }
    case LRT_RENDER_MODE_DIFFUSE: {
      float3 color = f3(0, 1, 1);
      if (type == LRT_TYPE_SDF_SBS_COL) {
        color.x = roundf(hit.c0) / 255.0f;
        color.y = hit.c0 - floorf(hit.c0);
        color.z = roundf(hit.c1) / 255.0f;
      }
      return make_float4(color.x, color.y, color.z, 1);
    }
    case LRT_RENDER_MODE_HSV_DEPTH: {
      const float iz = pos.z + z * dir.z;
      float zt = (iz + 1.f) * 2.f;
      zt = zt - float(int(zt));
      if (zt < 0.f) zt = 1.f + zt;
      // HSV (zt, 1, 1) -> RGB; the two written channels are always distinct
      const float vmin = (1.f - 1.f) * 1.0f;
      float hi;
      const float a = (1.0f - vmin) * modff(zt * 6.f, &hi);
      uint32_t h = uint32_t(hi);
      h = h <= 5u ? h : 5u;
      const uint32_t i0 = (2u + (h >> 1)) % 3u;
      const uint32_t i1 = (h & 1u) ? (h >> 1) : (1u + (h >> 1)) % 3u;
      const float v1 = (h & 1u) ? 1.0f - a : vmin + a;
      const float r = i1 == 0 ? v1 : (i0 == 0 ? vmin : 1.0f);
      const float g = i1 == 1 ? v1 : (i0 == 1 ? vmin : 1.0f);
      const float b = i1 == 2 ? v1 : (i0 == 2 ? vmin : 1.0f);
      return make_float4(r, g, b, 1.f);
    }
    default: return make_float4(1, 0, 1, 1);
  }
}

// kernel_RayTrace, Renderer/eye_ray.cpp:162-489 (the geometry-based modes without
// shadow rays; lights are the reference's defaults, Renderer/eye_ray_host.cpp:40;
// geometry without brick colours takes the default material's texel (0, 1, 1))
static __device__ __noinline__ float4 shade(const DevScene &s, const Hit &hit, float3 pos, float3 dir) {
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
      // LAMBERT_NO_TEX: white; LAMBERT: the brick colour, else the default textured
      // material's constant texel (0, 1, 1) (Renderer/eye_ray_host.cpp:30-33)
      float3 color = s.preset.render_mode == LRT_RENDER_MODE_LAMBERT ? f3(0, 1, 1) : f3(1, 1, 1);
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
    case LRT_RENDER_MODE_PRIMITIVE: case LRT_RENDER_MODE_TYPE: case LRT_RENDER_MODE_GEOM:
    case LRT_RENDER_MODE_BARYCENTRIC: case LRT_RENDER_MODE_ST_ITERATIONS: case LRT_RENDER_MODE_DIFFUSE:
    case LRT_RENDER_MODE_HSV_DEPTH:
      return shade_extra(s, hit, type, z, pos, dir);
    default: return make_float4(1, 0, 1, 1);
  }
}

__device__ __forceinline__ uint32_t encode_rgba8(float4 c) {   // Renderer/eye_ray.cpp:111-115
  const uint32_t r = uint32_t(255 * clampf(c.x, 0.0f, 1.0f)), g = uint32_t(255 * clampf(c.y, 0.0f, 1.0f));
  const uint32_t b = uint32_t(255 * clampf(c.z, 0.0f, 1.0f)), a = uint32_t(255 * clampf(c.w, 0.0f, 1.0f));
  return (a << 24) | (b << 16) | (g << 8) | r;
}


}  // namespace dev
}  // namespace lrt
