// Device-side restatement of the reference's per-ray arithmetic.  Every
// expression keeps the reference's operation order; this translation unit is
// compiled with --fmad=false (no multiply-add contraction) and IEEE division and
// square root, so results match the reference's x86-64 build bit for bit.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "lrt_internal.h"

namespace lrt {
namespace dev {

__device__ __forceinline__ float3 f3(float x, float y, float z) { return make_float3(x, y, z); }
__device__ __forceinline__ float3 add(float3 a, float3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 sub(float3 a, float3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 mul(float3 a, float3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float3 scl(float s, float3 a) { return f3(s * a.x, s * a.y, s * a.z); }
__device__ __forceinline__ float3 scr(float3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// std::min / std::max semantics (NaN and signed-zero behaviour included)
__device__ __forceinline__ float mn(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float mx(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return mn(mx(x, lo), hi); }
// LiteMath sign(): -1 for negative, +1 otherwise (never 0: SafeInverse relies on
// it to avoid a division by zero, raytrace_common.h:59-67)
__device__ __forceinline__ float signf(float a) { return a < 0.0f ? -1.0f : 1.0f; }
// normalize(u) = u / sqrt(dot(u,u))
__device__ __forceinline__ float3 normalize(float3 a) {
  const float l = sqrtf(dot(a, a));
  return f3(a.x / l, a.y / l, a.z / l);
}
// float4x4 (row-major) times (v, 1) and (v, 0): raytrace_common.h:84-92
__device__ __forceinline__ float3 matmul4x3(const float *m, float3 v) {
  return f3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 1.0f, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 1.0f,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 1.0f);
}
__device__ __forceinline__ float3 matmul3x3(const float *m, float3 v) {
  return f3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 0.0f, m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 0.0f,
            m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 0.0f);
}

// SafeInverse, raytrace_common.h:59-67
__device__ __forceinline__ float3 safe_inverse(float3 d) {
  const float ooeps = 1.0e-36f;
  return f3(1.0f / (fabsf(d.x) > ooeps ? d.x : fabsf(ooeps) * signf(d.x)),
            1.0f / (fabsf(d.y) > ooeps ? d.y : fabsf(ooeps) * signf(d.y)),
            1.0f / (fabsf(d.z) > ooeps ? d.z : fabsf(ooeps) * signf(d.z)));
}

// Hardware min/max (FMNMX).  For non-NaN operands they return the same value as
// std::min/std::max except possibly the sign of a zero result; slab distances
// and voxel coordinates are never NaN for finite rays (SafeInverse keeps the
// inverse direction finite), and a zero's sign never reaches an output there.
__device__ __forceinline__ float fmn(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float fmx(float a, float b) { return fmaxf(a, b); }

// Step bound of a voxel walk over a brick segment of t-length `extent`.  The
// reference's loop (BVH/BVH2Common.cpp:764-984, diff_render/BVH2DR.cpp:1160-1240)
// has none: a ray crosses at most 3 * brick_size voxels, but where the position
// rounds back into a voxel the ray has left (grazing rays), a step advances t by
// only +1e-6, which rounds to at least 7.6e-7 for t < 32 and to nothing beyond.
// 8 * brick_size + 16 steps plus 1.5e6 per unit of extent therefore cover every
// walk the reference finishes; beyond t ~ 32 its loop would not end.
__host__ __device__ __forceinline__ uint32_t walk_step_bound(uint32_t brick_size, float extent) {
  const float e = extent > 0.0f ? extent : 0.0f;   // NaN -> 0
  return 8u * brick_size + 16u + uint32_t(e < 2.6f ? e * 1.5e6f : 3.9e6f);
}

// rand3 / rand2, Renderer/eye_ray.cpp:53-80 (the pcg3d hash of JCGT 2020 on the pixel
// and sample index; `seed` is MultiRenderer::m_seed)
__device__ __forceinline__ float2 rand2(uint32_t x, uint32_t y, uint32_t iter, uint32_t seed) {
  x = x + 1233u * (iter + seed) % 171u;
  y = y + 453u * (iter + seed) % 765u;
  uint32_t v0 = x, v1 = y, v2 = x ^ y;
  v0 = v0 * 1664525u + 1013904223u; v1 = v1 * 1664525u + 1013904223u; v2 = v2 * 1664525u + 1013904223u;
  v0 += v1 * v2; v1 += v2 * v0; v2 += v0 * v1;
  v0 ^= v0 >> 16u; v1 ^= v1 >> 16u; v2 ^= v2 >> 16u;
  v0 += v1 * v2; v1 += v2 * v0; v2 += v0 * v1;
  const float k = 1.0f / float(0xffffffffu);
  return make_float2(__uint2float_rn(v0) * k, __uint2float_rn(v1) * k);
}

// RayBoxIntersection2, raytrace_common.h:69-82
__device__ __forceinline__ float2 ray_box(float3 o, float3 inv, float lox, float loy, float loz, float hix,
                                          float hiy, float hiz) {
  const float lo = inv.x * (lox - o.x), hi = inv.x * (hix - o.x);
  const float lo1 = inv.y * (loy - o.y), hi1 = inv.y * (hiy - o.y);
  const float lo2 = inv.z * (loz - o.z), hi2 = inv.z * (hiz - o.z);
  const float tmin = fmx(fmn(lo, hi), fmn(lo1, hi1));
  const float tmax = fmn(fmx(lo, hi), fmx(lo1, hi1));
  return make_float2(fmx(tmin, fmn(lo2, hi2)), fmn(tmax, fmx(lo2, hi2)));
}

// The same slab test with each plane distance as one FMA, lo * inv + noi with
// noi = -(o * inv) per ray (one rounding where RayBoxIntersection2 rounds twice):
// for the kernels compiled with contraction only.  |inv| <= 1e36 (SafeInverse),
// so with boxes and origins within a few hundred units of the origin every term
// is finite.
__device__ __forceinline__ float2 ray_box_fma(float3 inv, float3 noi, float lox, float loy, float loz, float hix,
                                              float hiy, float hiz) {
  const float lo = fmaf(lox, inv.x, noi.x), hi = fmaf(hix, inv.x, noi.x);
  const float lo1 = fmaf(loy, inv.y, noi.y), hi1 = fmaf(hiy, inv.y, noi.y);
  const float lo2 = fmaf(loz, inv.z, noi.z), hi2 = fmaf(hiz, inv.z, noi.z);
  const float tmin = fmx(fmn(lo, hi), fmn(lo1, hi1));
  const float tmax = fmn(fmx(lo, hi), fmx(lo1, hi1));
  return make_float2(fmx(tmin, fmn(lo2, hi2)), fmn(tmax, fmx(lo2, hi2)));
}

// octahedral encode, BVH/BVH2Common.cpp:29-35
__device__ __forceinline__ float2 encode_normal(float3 v) {
  const float s = 1.0f / (fabsf(v.x) + fabsf(v.y) + fabsf(v.z));
  const float px = v.x * s, py = v.y * s;
  const float sx = (px >= 0.0f) ? 1.0f : -1.0f, sy = (py >= 0.0f) ? 1.0f : -1.0f;
  if (v.z <= 0.0f) return make_float2((1.0f - fabsf(py)) * sx, (1.0f - fabsf(px)) * sy);
  return make_float2(px, py);
}

// octahedral decode, Renderer/eye_ray.cpp:22-33
__device__ __forceinline__ float3 decode_normal(float ex, float ey) {
  float3 v = f3(ex, ey, 1.0f - fabsf(ex) - fabsf(ey));
  if (v.z < 0) {
    const float vx = v.x;
    v.x = (1.0f - fabsf(v.y)) * ((v.x >= 0.0) ? +1.0f : -1.0f);
    v.y = (1.0f - fabsf(vx)) * ((v.y >= 0.0) ? +1.0f : -1.0f);
  }
  return normalize(v);
}

// eval_dist_trilinear, BVH/BVH2Common.cpp:62-72
__device__ __forceinline__ float trilinear(const float v[8], float3 dp) {
  return (1 - dp.x) * (1 - dp.y) * (1 - dp.z) * v[0] + (1 - dp.x) * (1 - dp.y) * (dp.z) * v[1] +
         (1 - dp.x) * (dp.y) * (1 - dp.z) * v[2] + (1 - dp.x) * (dp.y) * (dp.z) * v[3] +
         (dp.x) * (1 - dp.y) * (1 - dp.z) * v[4] + (dp.x) * (1 - dp.y) * (dp.z) * v[5] +
         (dp.x) * (dp.y) * (1 - dp.z) * v[6] + (dp.x) * (dp.y) * (dp.z) * v[7];
}

__device__ __forceinline__ bool need_normal(uint32_t render_mode) {   // BVH/BVH2Common.cpp:20-27
  return render_mode == 1 || render_mode == 8 || render_mode == 12 || render_mode == 17 || render_mode == 18;
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

// A hit under construction (CRT_Hit plus the reordered triangle id for shading).
struct Hit {
  float t;
  uint32_t prim;      // brick / voxel / reordered triangle id (remapped at the end)
  uint32_t geom;      // geomId | type << 24
  float c0, c1, c2, c3;
  uint32_t inst;      // instance of the hit (kernels walking several instances only)
};

// The scene as seen from instance `ii`: its box and matrices in the instance-0
// fields the leaf and shading functions read (kernels walking several instances).
__device__ __forceinline__ DevScene scene_of_instance(const DevScene &s, uint32_t ii) {
  DevScene r = s;
  const DevInst &I = s.insts[ii];
#pragma unroll
  for (int k = 0; k < 3; k++) { r.inst_bmin[k] = I.bmin[k]; r.inst_bmax[k] = I.bmax[k]; }
#pragma unroll
  for (int k = 0; k < 16; k++) { r.inst_inv[k] = I.inv[k]; r.inst_inv_t[k] = I.inv_t[k]; }
  return r;
}

struct Counters { uint32_t nodes, leaves, voxels, finder; };

}  // namespace dev
}  // namespace lrt
