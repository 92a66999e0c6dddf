/*
 * Shared scalar/vector helpers of the CPU oracle (TEST INFRASTRUCTURE ONLY):
 * restated LiteMath conventions and raytrace_common.h primitives used by both
 * the ray-query oracle (lrt_oracle.c) and the differentiable-render oracle
 * (lrt_oracle_dr.c).  Compiled with -ffp-contract=off.
 */
#ifndef LRT_ORACLE_MATH_H
#define LRT_ORACLE_MATH_H
#include <math.h>
#include <stdint.h>

typedef struct { float x, y, z; } f3;
typedef struct { float x, y; } f2;

static inline f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline f3 add3(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f3 mul3(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline f3 scl3(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
static inline f3 mul3s(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline f3 cross3(f3 a, f3 b) {
  return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* LiteMath normalize(u) = u / length(u), length = sqrt(dot(u,u)) (restated convention). */
static inline f3 normalize3(f3 a) { float l = sqrtf(dot3(a, a)); return mk3(a.x / l, a.y / l, a.z / l); }
static inline float fminf_(float a, float b) { return (b < a) ? b : a; }  /* std::min */
static inline float fmaxf_(float a, float b) { return (a < b) ? b : a; }  /* std::max */
/* LiteMath sign (restated convention): -1 for negative, +1 otherwise.  Never 0,
 * which SafeInverse needs to avoid its division by zero (raytrace_common.h:59-67). */
static inline float signf_(float a) { return a < 0.0f ? -1.0f : 1.0f; }
static inline float clampf_(float x, float lo, float hi) { return fminf_(fmaxf_(x, lo), hi); }

/* LiteMath float4x4 (row-major here: m[r*4+c]) times float4; sum in column order. */
static inline f3 matmul4x3(const float m[16], f3 v) {   /* raytrace_common.h:84-92, w=1 */
  return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 1.0f,
             m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 1.0f,
             m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 1.0f);
}
static inline f3 matmul3x3(const float m[16], f3 v) {   /* raytrace_common.h:84-87, w=0 */
  return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * 0.0f,
             m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * 0.0f,
             m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * 0.0f);
}

/* ---------------- raytrace_common.h ---------------- */
#define LEAF_BIT 0x80000000u
#define START_MASK 0x00FFFFFFu
#define SIZE_MASK 0x7F000000u
static inline uint32_t extract_start(uint32_t v) { return v & START_MASK; }
static inline uint32_t extract_count(uint32_t v) { return (v & SIZE_MASK) >> 24; }
static inline uint32_t pack_offset_size(uint32_t start, uint32_t size) {   /* raytrace_common.h:52-55 */
  return LEAF_BIT | ((size << 24) & SIZE_MASK) | (start & START_MASK);
}

/* SafeInverse, raytrace_common.h:59-67 */
static inline f3 safe_inverse(f3 d) {
  const float ooeps = 1.0e-36f;
  f3 r;
  r.x = 1.0f / (fabsf(d.x) > ooeps ? d.x : fabsf(ooeps) * signf_(d.x));
  r.y = 1.0f / (fabsf(d.y) > ooeps ? d.y : fabsf(ooeps) * signf_(d.y));
  r.z = 1.0f / (fabsf(d.z) > ooeps ? d.z : fabsf(ooeps) * signf_(d.z));
  return r;
}

/* RayBoxIntersection2, raytrace_common.h:69-82 */
static inline f2 ray_box2(f3 o, f3 inv, f3 bmin, f3 bmax) {
  const float lo = inv.x * (bmin.x - o.x), hi = inv.x * (bmax.x - o.x);
  const float lo1 = inv.y * (bmin.y - o.y), hi1 = inv.y * (bmax.y - o.y);
  const float lo2 = inv.z * (bmin.z - o.z), hi2 = inv.z * (bmax.z - o.z);
  const float tmin = fmaxf_(fminf_(lo, hi), fminf_(lo1, hi1));
  const float tmax = fminf_(fmaxf_(lo, hi), fmaxf_(lo1, hi1));
  f2 r; r.x = fmaxf_(tmin, fminf_(lo2, hi2)); r.y = fminf_(tmax, fmaxf_(lo2, hi2));
  return r;
}

/* eval_dist_trilinear, BVH/BVH2Common.cpp:62-72 */
static inline float eval_trilinear(const float v[8], f3 dp) {
  return (1 - dp.x) * (1 - dp.y) * (1 - dp.z) * v[0] +
         (1 - dp.x) * (1 - dp.y) * (dp.z) * v[1] +
         (1 - dp.x) * (dp.y) * (1 - dp.z) * v[2] +
         (1 - dp.x) * (dp.y) * (dp.z) * v[3] +
         (dp.x) * (1 - dp.y) * (1 - dp.z) * v[4] +
         (dp.x) * (1 - dp.y) * (dp.z) * v[5] +
         (dp.x) * (dp.y) * (1 - dp.z) * v[6] +
         (dp.x) * (dp.y) * (dp.z) * v[7];
}
#endif
