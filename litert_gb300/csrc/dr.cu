// Differentiable SDF render on the GPU: the forward + adjoint of
// MultiRendererDR::RenderDR (diff_render/MultiRendererDR.cpp:578-750) over an
// indexed SBS, with the per-ray gradient core of dr::BVHDR
// (diff_render/BVH2DR.cpp).
//
//  * dr_pixel_kernel     CastRayWithGrad (:1084-1294): one thread per pixel.  The
//                        forward march finds the first hit; the adjoint recomputes
//                        what it needs from the hit voxel (finite-difference
//                        dt/dvalues, smoothed normal over the 8 neighbour voxels)
//                        instead of storing a payload, and scatters
//                        dLoss/dColour x PD into dLoss/dP with warp-aggregated
//                        atomics.  spp > 1 re-traces each sample in a second pass.
//  * dr_border_detect    the 3x3 border-pixel test (:609-685), compacted with a
//                        warp ballot.
//  * dr_border_kernel    CastBorderRay + CalculateBorderRayDerivatives
//                        (:1319-1499): one warp per border pixel, border_spp rays.
//  * dr_adam_kernel      OptimizeStepAdam (:828-853).
//
// Arithmetic keeps the reference's operation order (compiled with --fmad=false,
// IEEE division and square root), so per-pixel colours and per-ray partial
// derivatives equal the CPU restatement bit for bit; only the order in which
// atomics sum the gradient differs.
#include "dr_internal.h"
#include "trace_common.cuh"

namespace lrt {
namespace drk {
using namespace lrt::dev;

enum : uint32_t { F_DCOLOR = 1, F_DDIFFUSE = 2, F_DNORM = 4, F_BORDER = 8, F_DDIST = 16, F_BORDER_EARLY = 32 };
enum : uint32_t { R_DIFFUSE = 0, R_LAMBERT = 1, R_MASK = 2, R_LINEAR_DEPTH = 3, R_NORMAL = 4 };

struct M3 {
  float3 r0, r1, r2;
};
__device__ __forceinline__ float3 mv(const M3 &m, float3 v) { return f3(dot(m.r0, v), dot(m.r1, v), dot(m.r2, v)); }
__device__ __forceinline__ float3 divs(float3 a, float s) { return f3(a.x / s, a.y / s, a.z / s); }
__device__ __forceinline__ float len3(float3 a) { return sqrtf(dot(a, a)); }

// ---- trilinear helpers, diff_render/BVH2DR.cpp:200-612 ----
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
__device__ __forceinline__ void tri_w(float o[8], float3 dp) {
  o[0] = (1 - dp.x) * (1 - dp.y) * (1 - dp.z); o[1] = (1 - dp.x) * (1 - dp.y) * (dp.z);
  o[2] = (1 - dp.x) * (dp.y) * (1 - dp.z);     o[3] = (1 - dp.x) * (dp.y) * (dp.z);
  o[4] = (dp.x) * (1 - dp.y) * (1 - dp.z);     o[5] = (dp.x) * (1 - dp.y) * (dp.z);
  o[6] = (dp.x) * (dp.y) * (1 - dp.z);         o[7] = (dp.x) * (dp.y) * (dp.z);
}
__device__ __forceinline__ float3 tri3(const float3 c[8], float3 dp) {
  float w[8];
  tri_w(w, dp);
  float3 r = scl(w[0], c[0]);
#pragma unroll
  for (int i = 1; i < 8; i++) r = add(r, scl(w[i], c[i]));
  return r;
}
__device__ __forceinline__ M3 tri3_ddp(const float3 c[8], float3 dp) {
  const float wx[8] = {-(1 - dp.y) * (1 - dp.z), -(1 - dp.y) * (dp.z), -(dp.y) * (1 - dp.z), -(dp.y) * (dp.z),
                       (1 - dp.y) * (1 - dp.z), (1 - dp.y) * (dp.z), (dp.y) * (1 - dp.z), (dp.y) * (dp.z)};
  const float wy[8] = {-(1 - dp.x) * (1 - dp.z), -(1 - dp.x) * (dp.z), (1 - dp.x) * (1 - dp.z), (1 - dp.x) * (dp.z),
                       -(dp.x) * (1 - dp.z), -(dp.x) * (dp.z), (dp.x) * (1 - dp.z), (dp.x) * (dp.z)};
  const float wz[8] = {-(1 - dp.x) * (1 - dp.y), (1 - dp.x) * (1 - dp.y), -(1 - dp.x) * (dp.y), (1 - dp.x) * (dp.y),
                       -(dp.x) * (1 - dp.y), (dp.x) * (1 - dp.y), -(dp.x) * (dp.y), (dp.x) * (dp.y)};
  float3 cx = scl(wx[0], c[0]), cy = scl(wy[0], c[0]), cz = scl(wz[0], c[0]);
#pragma unroll
  for (int i = 1; i < 8; i++) {
    cx = add(cx, scl(wx[i], c[i]));
    cy = add(cy, scl(wy[i], c[i]));
    cz = add(cz, scl(wz[i], c[i]));
  }
  return M3{f3(cx.x, cy.x, cz.x), f3(cx.y, cy.y, cz.y), f3(cx.z, cy.z, cz.z)};
}
// normalize_diff: b is formed in double as the reference's 1.0/(a*sqrt(a)) is
__device__ __forceinline__ M3 nrm_diff(float3 v) {
  const float a = dot(v, v);
  const float b = (float)(1.0 / ((double)a * sqrt((double)a)));
  return M3{scl(b, f3(v.y * v.y + v.z * v.z, -v.x * v.y, -v.x * v.z)),
            scl(b, f3(-v.x * v.y, v.x * v.x + v.z * v.z, -v.y * v.z)),
            scl(b, f3(-v.x * v.z, -v.y * v.z, v.x * v.x + v.y * v.y))};
}
__device__ __forceinline__ M3 tri_ddp_ddp(const float v[8], float3 dp) {
  const float dxdy = (1 - dp.z) * v[0] + (dp.z) * v[1] - (1 - dp.z) * v[2] - (dp.z) * v[3] - (1 - dp.z) * v[4] -
                     (dp.z) * v[5] + (1 - dp.z) * v[6] + (dp.z) * v[7];
  const float dxdz = (1 - dp.y) * v[0] - (1 - dp.y) * v[1] + (dp.y) * v[2] - (dp.y) * v[3] - (1 - dp.y) * v[4] +
                     (1 - dp.y) * v[5] - (dp.y) * v[6] + (dp.y) * v[7];
  const float dydz = (1 - dp.x) * v[0] - (1 - dp.x) * v[1] - (1 - dp.x) * v[2] + (1 - dp.x) * v[3] + (dp.x) * v[4] -
                     (dp.x) * v[5] - (dp.x) * v[6] + (dp.x) * v[7];
  return M3{f3(0, dxdy, dxdz), f3(dxdy, 0, dydz), f3(dxdz, dydz, 0)};
}
// column j of eval_dist_trilinear_ddp_dvalues (a 3x8 matrix)
__device__ __forceinline__ float3 ddp_dvalue(float3 dp, int j) {
  const float ax = (j & 4) ? dp.x : (1 - dp.x), ay = (j & 2) ? dp.y : (1 - dp.y), az = (j & 1) ? dp.z : (1 - dp.z);
  const float sx = (j & 4) ? 1.0f : -1.0f, sy = (j & 2) ? 1.0f : -1.0f, sz = (j & 1) ? 1.0f : -1.0f;
  // entries are +-(a*b): the sign is exact, the product is formed in the reference's order
  return f3(sx * (ay * az), sy * (ax * az), sz * (ax * ay));
}
__device__ __forceinline__ float step01(float e0, float e1, float x) { return clampf((x - e0) / (e1 - e0), 0.0f, 1.0f); }
__device__ __forceinline__ float3 dp_to_nmq(float3 dp, float beta) {
  return f3(dp.x < 0.5f ? step01(-beta, beta, dp.x) : step01(-beta, beta, dp.x - 1.0f),
            dp.y < 0.5f ? step01(-beta, beta, dp.y) : step01(-beta, beta, dp.y - 1.0f),
            dp.z < 0.5f ? step01(-beta, beta, dp.z) : step01(-beta, beta, dp.z - 1.0f));
}

// ---- border relaxation bookkeeping (RayDiffPayload subset) ----
struct Relax {
  float t, sdf;            // missed_hit.t, .sdf
  uint32_t cvb;            // missed_hit.check_vox_border
  float ct, csdf;          // missed_hit_candidate.t, .sdf
  float3 color, normal;    // missed_hit.color, .normal
  uint32_t idx[8];         // missed_indices
  float dth[8];            // missed_dSDF_dtheta
  // Early skipping (border integral only).  A border sample contributes only when
  // its final sdf is below relax_eps, so a voxel whose corner values all exceed
  // min(sdf, skip_t) + margin may be skipped before the walk has met a local
  // minimum (skip_t = relax_eps; +inf restores the reference's walk exactly).
  // The skipped voxels hold no value below skip_t, so until the first update
  // below skip_t both walks' running minima are >= skip_t, an update below skip_t
  // from a voxel's interior or exit happens in both walks alike, and from then on
  // the walks are in the same state.  What can differ is a voxel-entry update
  // (check_vox_border), which depends on the previous voxel's outcome.  flags:
  //   bit 0  re-walk needed: an entry update below skip_t while the two walks'
  //          check_vox_border may differ, or a final candidate below skip_t while
  //          the running minimum is not;
  //   bit 1  the record's indices / dSDF/dtheta / colour / normal were written
  //          after sdf fell below skip_t (else they may be an older voxel's);
  //   bit 2  no voxel of the current brick has been intersected or skipped yet;
  //   bit 3  the walks have diverged (a voxel was skipped that only skip_t skips);
  //   bit 4  check_vox_border may differ between the walks.  It cannot after a
  //          voxel both walks intersected whose exit is inside the surface,
  //          below skip_t, or with the distance still falling there; inside a
  //          brick the next voxel's entry value is that face's value up to
  //          rounding, so after a skipped voxel or an exit above skip_t it lies
  //          above skip_t - margin: bit 0 is set only at a brick's first voxel or
  //          for an entry value within the margin below skip_t.
  // The caller re-walks with skip_t = +inf unless bit 0 is clear and either
  // sdf >= skip_t or bit 1 is set.
  float skip_t;
  uint32_t flags;
};

// BVHDR::Intersect, NEWTON branch (diff_render/BVH2DR.cpp:623-1073).  Returns t in
// voxel units on a hit, else qFar + 1e-6.
template <bool BORDER>
__device__ float intersect(const float values[8], float d, float qFar, float3 start_q, float3 dir, Relax *rl,
                          float band = 0.0f) {
  const float EPS = 1e-6f, SDF_EPS = 1e-7f;
  const float d_inv = 1.0f / d;
  float t = 0.0f;
  bool hit = false;
  if (BORDER) rl->csdf = 1000.f;
  const float start_dist = trilinear(values, start_q);
  if (start_dist <= SDF_EPS) return t;
  const float s000 = values[0] * d_inv, s001 = values[1] * d_inv, s010 = values[2] * d_inv, s011 = values[3] * d_inv;
  const float s100 = values[4] * d_inv, s101 = values[5] * d_inv, s110 = values[6] * d_inv, s111 = values[7] * d_inv;
  const float a = s101 - s001;
  const float k0 = s000, k1 = s100 - s000, k2 = s010 - s000, k3 = s110 - s010 - k1, k4 = k0 - s001, k5 = k1 - a;
  const float k6 = k2 - (s011 - s001), k7 = k3 - (s111 - s011 - a);
  const float3 o = start_q, d3 = dir;
  const float m0 = o.x * o.y, m1 = d3.x * d3.y, m2 = o.x * d3.y + o.y * d3.x;
  const float m3 = k5 * o.z - k1, m4 = k6 * o.z - k2, m5 = k7 * o.z - k3;
  const float c0 = (k4 * o.z - k0) + o.x * m3 + o.y * m4 + m0 * m5;
  const float c1 = d3.x * m3 + d3.y * m4 + m2 * m5 + d3.z * (k4 + k5 * o.x + k6 * o.y + k7 * m0);
  const float c2 = m1 * m5 + d3.z * (k5 * d3.x + k6 * d3.y + k7 * m2);
  const float c3 = k7 * m1 * d3.z;
  const float aa = 3 * c3, b = 2 * c2, c = c1;
  const float t0 = 0;
  float t1 = qFar, t2 = qFar;
  const float t3 = qFar;
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
  const float sdf0 = c0;
  const float sdf1 = (c0 + t1 * (c1 + t1 * (c2 + t1 * c3)));
  const float sdf2 = (c0 + t2 * (c1 + t2 * (c2 + t2 * c3)));
  const float sdf3 = (c0 + t3 * (c1 + t3 * (c2 + t3 * c3)));
  const bool s0 = sdf0 > 0, s1 = sdf1 > 0, s2 = sdf2 > 0, s3 = sdf3 > 0;
  float nwt_min = t0, nwt_max = t0;
  if (s0 != s1) { nwt_min = t0; nwt_max = t1; }
  else if (s1 != s2) { nwt_min = t1; nwt_max = t2; }
  else if (s2 != s3) { nwt_min = t2; nwt_max = t3; }
  if (nwt_min < nwt_max) {
    float rtn = 0.5f * (nwt_min + nwt_max);
    float f = 1000;
    for (unsigned it = 0; it < 10 && fabsf(f) >= SDF_EPS; it++) {
      f = c0 + rtn * (c1 + rtn * (c2 + rtn * c3));
      const float df = c1 + rtn * (2 * c2 + rtn * 3 * c3);
      const float dx = f / (df + signf(df) * 1e-9f);
      rtn -= dx;
    }
    t = rtn;
    hit = (t >= 0 && t <= qFar && fabsf(f) < SDF_EPS);
  }
  if (BORDER) {
    float t_min = qFar + EPS;
    if (fabsf(aa) > EPS) {
      // with D < 0 the reference's roots are NaN, so t_min is NaN and nothing below
      // updates; that case is taken without evaluating them
      if (D >= 0.0f) {
        const float root1 = -0.5f * (b + sqrtf(D)) / aa, root2 = -0.5f * (b - sqrtf(D)) / aa;
        t_min = (signf(aa) > 0) == (root1 < root2) ? root1 : root2;
      } else {
        t_min = __int_as_float(0x7fffffff);
      }
    } else if (b < -EPS) {
      t_min = -c / b;
    }
    const float sdf_min = (c0 + t_min * (c1 + t_min * (c2 + t_min * c3)));
    if ((rl->flags & 16u) && c1 <= 0 && sdf0 < 0.f && rl->sdf >= rl->skip_t) {
      const float v = -sdf0 * d;
      if (v < rl->skip_t && ((rl->flags & 4u) || v >= rl->skip_t - band)) rl->flags |= 1u;
    }
    if (rl->cvb == 1) {
      if (c1 <= 0) {
        if (sdf0 < 0.f && -sdf0 * d < rl->sdf) { rl->t = t0; rl->sdf = -sdf0 * d; }
      }
      rl->cvb = 0;
    }
    if (t_min >= 0 && t_min <= qFar && sdf_min < 0.f && -sdf_min * d < rl->sdf) {
      rl->t = t_min;
      rl->sdf = -sdf_min * d;
    }
    const float dexit = c1 + qFar * (2 * c2 + qFar * 3 * c3);
    if (sdf3 < 0.f && -sdf3 * d < rl->sdf && dexit >= 0.f) {
      rl->cvb = 1;
      rl->ct = qFar;
      rl->csdf = -sdf3 * d;
    }
    // bit 4 for the next voxel: known equal unless the walks have diverged and this
    // exit is outside, not below skip_t and not falling
    const bool known = !(rl->flags & 8u) || !(sdf3 < 0.f) || dexit < 0.f || -sdf3 * d < rl->skip_t;
    rl->flags = (rl->flags & ~(4u | 16u)) | (known ? 0u : 16u);
  }
  return hit ? t : qFar + EPS;
}

// dIntersect_dValues (:1075-1090): central differences, delta 1e-3, on the
// caller's array (the +d, -2d, +d residue stays in it as in the reference)
__device__ void dintersect(float values[8], float d, float qFar, float3 start_q, float3 dir, float out[8]) {
  const float delta = 0.001f;
#pragma unroll 1
  for (int i = 0; i < 8; i++) {
    values[i] += delta;
    const float d1 = intersect<false>(values, d, qFar, start_q, dir, nullptr);
    values[i] -= 2 * delta;
    const float d2 = intersect<false>(values, d, qFar, start_q, dir, nullptr);
    values[i] += delta;
    out[i] = (d1 - d2) / (2 * delta);
  }
}

// brick geometry of a node (OctreeBrickIntersectWithGrad :1142-1160)
struct Brick {
  float sz, d, scale;
  float3 bmin, bmax;
  uint32_t data_offset;
};
__device__ __forceinline__ Brick brick_of(const DevScene &s, uint32_t node) {
  const uint4 nd = __ldg(&s.nodes[node]);
  Brick b;
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF), pz = float(nd.y >> 16);
  b.sz = float(nd.y & 0x0000FFFF);
  const float sz_inv = 2.0f / b.sz, bs = float(s.brick_size);
  b.d = 2.0f / (b.sz * bs);
  b.bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(px, py, pz)));
  b.bmax = add(b.bmin, scl(sz_inv, f3(1, 1, 1)));
  b.scale = 0.5f * b.sz * bs;
  b.data_offset = nd.z;
  return b;
}

__device__ __forceinline__ uint32_t vid(uint32_t x, uint32_t y, uint32_t z, uint32_t v) { return x * v * v + y * v + z; }

// the 8 corner values of a voxel from the per-brick gathered copy of the
// parameters (one load each instead of index-then-value)
__device__ __forceinline__ void load_vals(const DevScene &s, uint32_t node, float3 vox, float values[8]) {
  const uint32_t vx = (uint32_t)vox.x, vy = (uint32_t)vox.y, vz = (uint32_t)vox.z;
  const float *b = s.bvals + (size_t)node * (s.v_size * s.v_size * s.v_size);
#pragma unroll
  for (int i = 0; i < 8; i++) values[i] = __ldg(&b[vid(vx + ((i & 4) >> 2), vy + ((i & 2) >> 1), vz + (i & 1), s.v_size)]);
}
// their parameter indices (load_distance_values_with_indices, diff_render/BVH2DR.cpp:1092-1106)
__device__ __forceinline__ void load_idx(const DevScene &s, uint32_t off, float3 vox, uint32_t idx[8]) {
  const uint32_t vx = (uint32_t)vox.x, vy = (uint32_t)vox.y, vz = (uint32_t)vox.z;
#pragma unroll
  for (int i = 0; i < 8; i++)
    idx[i] = __ldg(&s.values[off + vid(vx + ((i & 4) >> 2), vy + ((i & 2) >> 1), vz + (i & 1), s.v_size)]);
}

__device__ __forceinline__ void load_colors(const DevScene &s, uint32_t t_off, float3 c[8]) {
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t j = __ldg(&s.values[t_off + i]);
    c[i] = f3(__ldg(&s.P[j]), __ldg(&s.P[j + 1]), __ldg(&s.P[j + 2]));
  }
}

// The first hit of a ray (what the adjoint recomputes from).
struct HitRec {
  float t;            // tReal (ray units)
  uint32_t prim;      // brick id, kNoIndex for a miss
  float tl, qFar;     // t and far plane in voxel units
  float3 start_q, vox;
  float3 pos, dir;    // the ray in object space
};

// voxel walk of one brick (OctreeBrickIntersectWithGrad :1160-1240, 1605-1608),
// bounded at 8*brick_size+16 steps where the reference's loop is unbounded
//
// Skips (exact): where every corner value v of a voxel (or brick) satisfies
// min v > skip_margin(max |v|), the voxel's cubic has no root on the segment
// even after rounding, so the finder cannot report a hit; and in border mode
// no point of the segment can bring the relaxation SDF below min v, so the
// only effects of the reference's Intersect call are its resets of the
// candidate and of check_vox_border, which are applied here.  The margin
// bounds the rounding of the cubic's coefficients and of Horner's evaluation
// on [0, qFar] (qFar <= sqrt 3) with a wide safety factor.
__device__ __forceinline__ float skip_margin(float maxabs) { return 2e-3f * maxabs + 1e-6f; }

// by_t: only skip_t skips this voxel (the reference's walk intersects it)
template <bool BORDER>
__device__ __forceinline__ void skipped_intersect(Relax *rl, bool by_t) {
  if (BORDER) {
    rl->csdf = 1000.f;
    if (rl->cvb == 1) rl->cvb = 0;
    uint32_t f = rl->flags & ~4u;
    if (by_t) f |= 8u;
    f = (f & ~16u) | ((f & 8u) ? 16u : 0u);
    rl->flags = f;
  }
}

template <bool BORDER>
__device__ bool brick_visit(const DevScene &s, uint32_t node, float3 pos, float3 dir, float3 inv, float tNear,
                            HitRec &hr, Relax *rl) {
  const Brick B = brick_of(s, node);
  float2 bnf = ray_box(pos, inv, B.bmin.x, B.bmin.y, B.bmin.z, B.bmax.x, B.bmax.y, B.bmax.z);
  const float bs = float(s.brick_size);
  const uint32_t max_steps = walk_step_bound(s.brick_size, bnf.y - bnf.x);
  if (!(bnf.x < bnf.y)) return false;
  if (BORDER) rl->flags |= 4u;
  {
    const float2 bb = __ldg(&s.brick_bounds[node]);   // min v, max |v| over the brick
    const float thr = (BORDER ? fminf(rl->sdf, rl->skip_t) : 0.0f) + skip_margin(bb.y);
    if (bb.x > thr) {
      if (!BORDER) return false;
      // border mode: the walk would call Intersect at least once if its first voxel does
      const float3 lp = scr(sub(add(pos, scl(bnf.x, dir)), B.bmin), B.scale);
      const float3 vox = f3(floorf(clampf(lp.x, 1e-6f, bs - 1e-6f)), floorf(clampf(lp.y, 1e-6f, bs - 1e-6f)),
                            floorf(clampf(lp.z, 1e-6f, bs - 1e-6f)));
      const float3 min_pos = add(B.bmin, scl(B.d, vox));
      const float3 max_pos = add(min_pos, scl(B.d, f3(1, 1, 1)));
      const float2 fnf = ray_box(pos, inv, min_pos.x, min_pos.y, min_pos.z, max_pos.x, max_pos.y, max_pos.z);
      if (tNear < fnf.x) {
        skipped_intersect<BORDER>(rl, !(bb.x > rl->sdf + skip_margin(bb.y)));
        return false;
      }
    }
  }
  // Two nested loops: the inner one steps through voxels (applying the skips)
  // until one needs Intersect or the brick ends; Intersect runs after it.  A
  // lane's sequence of voxels is the single loop's, but the lanes of a warp that
  // reach an intersected voxel after different numbers of steps run it together.
  uint32_t step = 0;
  for (;;) {
    bool cand = false;
    float3 vox, min_pos;
    float2 fnf;
    float values[8], vmax = 0.0f;
    while (bnf.x < bnf.y && step < max_steps) {
      const float3 hit_pos = add(pos, scl(bnf.x, dir));
      const float3 lp = scr(sub(hit_pos, B.bmin), B.scale);
      vox = f3(floorf(clampf(lp.x, 1e-6f, bs - 1e-6f)), floorf(clampf(lp.y, 1e-6f, bs - 1e-6f)),
               floorf(clampf(lp.z, 1e-6f, bs - 1e-6f)));
      min_pos = add(B.bmin, scl(B.d, vox));
      const float3 max_pos = add(min_pos, scl(B.d, f3(1, 1, 1)));
      fnf = ray_box(pos, inv, min_pos.x, min_pos.y, min_pos.z, max_pos.x, max_pos.y, max_pos.z);
      step++;
      // the voxel's min v and max |v| over its 8 corners (dr_brick_bounds_kernel
      // folds them in the corner order of load_vals); its corners are loaded only
      // for the voxel that goes to Intersect
      const uint32_t bsz = s.brick_size;
      const float2 vb = __ldg(&s.vbounds[(size_t)node * (bsz * bsz * bsz) +
                                         (uint32_t(vox.x) * bsz + uint32_t(vox.y)) * bsz + uint32_t(vox.z)]);
      const float vmin = vb.x;
      vmax = vb.y;
      if (tNear < fnf.x) {
        if (!(vmin > (BORDER ? fminf(rl->sdf, rl->skip_t) : 0.0f) + skip_margin(vmax))) {
          load_vals(s, node, vox, values);
          cand = true;
          break;
        }
        skipped_intersect<BORDER>(rl, BORDER && !(vmin > rl->sdf + skip_margin(vmax)));
      }
      bnf.x += mx(0.0f, fnf.y - bnf.x) + 1e-6f;
    }
    if (!cand) return false;
    {
      const float3 start_q = scr(sub(add(pos, scl(fnf.x, dir)), min_pos), B.scale);
      const float qFar = (fnf.y - fnf.x) * B.scale;
      const float prev = BORDER ? rl->sdf : 0.0f;
      const float t = intersect<BORDER>(values, B.d, qFar, start_q, dir, rl, skip_margin(vmax));
      const float tReal = fnf.x + B.d * t;
      if (BORDER) {
        if (rl->sdf < prev && rl->t < t) {
          const float mt = rl->t;
          rl->t = fnf.x + B.d * rl->t;
          const float3 q_ast = add(start_q, scl(mt, dir));
          const float3 y_ast = add(pos, scl(fnf.x + (B.d * mt), dir));
          const float3 dp_ast = scr(sub(y_ast, B.bmin), 0.5f * B.sz);
          float3 g = scr(tri_diff(values, q_ast), 1 / B.d);
          const float3 mult = f3(fabsf(q_ast.x - 0.5f) > 0.5f - 1e-5f ? 0.0f : 1.0f,
                                 fabsf(q_ast.y - 0.5f) > 0.5f - 1e-5f ? 0.0f : 1.0f,
                                 fabsf(q_ast.z - 0.5f) > 0.5f - 1e-5f ? 0.0f : 1.0f);
          g = mul(g, mult);
          const float gl = len3(g);
          if (gl > 1e-9f) {
            float w[8];
            tri_w(w, q_ast);
#pragma unroll
            for (int i = 0; i < 8; i++) rl->dth[i] = -w[i] / gl;
            float3 cols[8];
            load_colors(s, B.data_offset + s.v_size * s.v_size * s.v_size, cols);
            rl->color = tri3(cols, dp_ast);
            rl->normal = divs(g, gl);
            load_idx(s, B.data_offset, vox, rl->idx);
            if (rl->sdf < rl->skip_t) rl->flags |= 2u;
          }
        }
      }
      if (t <= qFar && tReal < hr.t) {
        hr.t = tReal;
        hr.prim = node;
        hr.tl = t;
        hr.qFar = qFar;
        hr.start_q = start_q;
        hr.vox = vox;
        return true;
      }
    }
    bnf.x += mx(0.0f, fnf.y - bnf.x) + 1e-6f;
  }
}

// BVH2TraverseF32WithGrad (:106-167) with stopOnFirstHit; leaves hold one brick,
// tNearSdf = max(tNear, 0.1) (:178-179)
template <bool BORDER>
__device__ void traverse(const DevScene &s, float3 pos, float3 dir, float tNear, HitRec &hr, Relax *rl) {
  uint32_t stack[kStack];
  int top = 0;
  uint32_t left = 0;
  const float3 inv = safe_inverse(dir);
  const float tNearSdf = mx(tNear, 0.1f);
  // a tree visits each pair at most once per ray; more visits mean a malformed BVH
  uint32_t visits = 0;
  const uint32_t max_visits = s.n_pairs + 1;
  while (top >= 0 && hr.prim == kNoIndex) {
    while (top >= 0 && ((left & 0x80000000u) == 0)) {
      if (++visits > max_visits) {
        atomicOr(s.status, kStatusTraversalBound);
        return;
      }
      const float4 a0 = __ldg(&s.pairs[4 * left + 0]), a1 = __ldg(&s.pairs[4 * left + 1]);
      const float4 b0 = __ldg(&s.pairs[4 * left + 2]), b1 = __ldg(&s.pairs[4 * left + 3]);
      const uint32_t n0 = __float_as_uint(a0.w), n1 = __float_as_uint(b0.w);
      const float2 tm0 = ray_box(pos, inv, a0.x, a0.y, a0.z, a1.x, a1.y, a1.z);
      const float2 tm1 = ray_box(pos, inv, b0.x, b0.y, b0.z, b1.x, b1.y, b1.z);
      const bool h0 = (tm0.x <= tm0.y) && (tm0.y >= tNear) && (tm0.x <= hr.t);
      const bool h1 = (tm1.x <= tm1.y) && (tm1.y >= tNear) && (tm1.x <= hr.t);
      left = h0 ? n0 : n1;
      if (h0 && h1) {
        left = (tm0.x <= tm1.x) ? n0 : n1;
        if (top >= kStack) {
          atomicOr(s.status, kStatusStackOverflow);
          top = -1;
          break;
        }
        stack[top] = (tm0.x <= tm1.x) ? n1 : n0;
        top++;
      }
      if (!h0 && !h1) {
        top--;
        left = stack[top > 0 ? top : 0];
      }
    }
    if (top >= 0 && left != 0xFFFFFFFFu) brick_visit<BORDER>(s, left & 0x00FFFFFFu, pos, dir, inv, tNearSdf, hr, rl);
    top--;
    left = stack[top > 0 ? top : 0];
  }
}

// RayQuery_NearestHitWithGrad (:12-102): TLAS leaf box of the single instance,
// ray to object space, BLAS traversal, candidate merge of the relaxation point
template <bool BORDER>
__device__ void query(const DevScene &s, float3 P, float3 D, float tfar, HitRec &hr, Relax *rl,
                      float skip_t = __builtin_huge_valf()) {
  hr.t = tfar;
  hr.prim = kNoIndex;
  if (BORDER) {
    rl->skip_t = skip_t; rl->flags = 0;
    rl->t = tfar; rl->sdf = 1000.0f; rl->cvb = 1;
    rl->ct = tfar; rl->csdf = 1000.0f;
    rl->color = f3(0, 0, 0); rl->normal = f3(1, 0, 0);
#pragma unroll
    for (int i = 0; i < 8; i++) { rl->idx[i] = kNoIndex; rl->dth[i] = 0.0f; }
  }
  const float3 inv = safe_inverse(D);
  const float2 bh = ray_box(P, inv, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0], s.inst_bmax[1],
                            s.inst_bmax[2]);
  if ((bh.x <= bh.y) && (bh.y > 0.0f) && (bh.x < hr.t)) {
    hr.pos = matmul4x3(s.inst_inv, P);
    hr.dir = matmul3x3(s.inst_inv, D);
    traverse<BORDER>(s, hr.pos, hr.dir, 0.0f, hr, rl);
  }
  if (BORDER && rl->csdf < rl->sdf) {   // missed_hit = missed_hit_candidate (whole struct)
    if (rl->csdf < rl->skip_t && rl->sdf >= rl->skip_t) rl->flags |= 1u;
    rl->t = rl->ct; rl->sdf = rl->csdf; rl->cvb = 1;
    rl->color = f3(0, 0, 0); rl->normal = f3(1, 0, 0);
  }
}

// A border sample's query: the walk with early skipping below relax_eps, and the
// reference's own walk again where the skipping could have changed the record
// (Relax::flags); the record is the reference walk's in either case.
__device__ __forceinline__ void border_query(const DevScene &s, float3 P, float3 D, float eps, HitRec &hr, Relax &rl,
                                             float tfar = 1e9f) {
  float skip_t = eps;
#pragma unroll 1
  for (int pass = 0; pass < 2; pass++) {
    query<true>(s, P, D, tfar, hr, &rl, skip_t);
    if (!(rl.flags & 1u) && !(rl.sdf < eps && !(rl.flags & 2u))) break;
    skip_t = __builtin_huge_valf();
  }
}

// Neighbour voxel i of the 2x2x2 block around the hit (OctreeBrickIntersectWithGrad
// :1339-1365): its node (kInvalidIdx if absent), voxel position and offset.
struct Nbr {
  uint32_t node;
  float3 nvox, dvox;
};
__device__ __forceinline__ Nbr neighbour(const DevScene &s, uint32_t node, uint32_t data_offset, float3 vox, float3 dp,
                                         int i) {
  const int ibs = (int)s.brick_size;
  const int vx = (int)(dp.x < 0.5f ? vox.x - 1 : vox.x) + ((i & 4) >> 2);
  const int vy = (int)(dp.y < 0.5f ? vox.y - 1 : vox.y) + ((i & 2) >> 1);
  const int vz = (int)(dp.z < 0.5f ? vox.z - 1 : vox.z) + (i & 1);
  const int bx = vx >= 0 ? (vx < ibs ? 0 : 1) : -1, by = vy >= 0 ? (vy < ibs ? 0 : 1) : -1;
  const int bz = vz >= 0 ? (vz < ibs ? 0 : 1) : -1;
  const uint32_t nid = 9 * (bx + 1) + 3 * (by + 1) + (bz + 1);
  Nbr n;
  const float3 fv = f3(float(vx), float(vy), float(vz));
  n.dvox = sub(fv, vox);
  if (nid == 13) {
    n.node = node;
    n.nvox = fv;
  } else {
    n.node = __ldg(&s.values[data_offset + s.v_size * s.v_size * s.v_size + 8 + nid]);
    n.nvox = sub(fv, scl(float(s.brick_size), f3(float(bx), float(by), float(bz))));
  }
  return n;
}

// Shading state of a hit: colour inputs, normal and what the adjoint reuses.
struct Shade {
  float3 color, normal;     // CRT_HitDR color / normal
  float3 dp;                // hit point in voxel units (IN layout smoothing)
  float3 dpb;               // hit point in brick units (colour interpolation)
  float3 nrm[8];            // neighbour-voxel normals (IN layout)
  float3 nmq;
  float3 tr3;
  uint32_t k;               // slot of the hit voxel among the 8 neighbours
};

// hit colour and normal (OctreeBrickIntersectWithGrad :1300-1460 without the
// derivative terms, and :1489-1497).  fd_residue: the ray also asks for
// position derivatives, so the reference computes the flat normal after
// dIntersect_dValues left its +d, -2d, +d rounding residue in the values.
__device__ void shade_hit(const DevScene &s, const HitRec &hr, Shade &sh, bool fd_residue) {
  const Brick B = brick_of(s, hr.prim);
  const float3 dp = add(hr.start_q, scl(hr.tl, hr.dir));
  sh.dp = dp;
  sh.k = (dp.x < 0.5f ? 4 : 0) + (dp.y < 0.5f ? 2 : 0) + (dp.z < 0.5f ? 1 : 0);
  if (s.need_normal) {
    if (s.layout_in) {
      sh.nmq = dp_to_nmq(dp, 0.5f);
#pragma unroll 1
      for (int i = 0; i < 8; i++) {
        sh.nrm[i] = f3(0, 0, 0);
        const Nbr n = neighbour(s, hr.prim, B.data_offset, hr.vox, dp, i);
        if (n.node != kInvalidIdx) {
          float vn[8];
          load_vals(s, n.node, n.nvox, vn);
          sh.nrm[i] = normalize(tri_diff(vn, sub(dp, n.dvox)));
        }
      }
      sh.tr3 = tri3(sh.nrm, sh.nmq);
      sh.normal = normalize(sh.tr3);
    } else {
      float values[8];
      load_vals(s, hr.prim, hr.vox, values);
      if (fd_residue) {
        const float delta = 0.001f;
#pragma unroll
        for (int i = 0; i < 8; i++) {
          values[i] += delta;
          values[i] -= 2 * delta;
          values[i] += delta;
        }
      }
      sh.normal = normalize(tri_diff(values, dp));
    }
  } else {
    sh.normal = f3(1, 0, 0);
  }
  const float3 pos = add(hr.pos, scl(hr.t, hr.dir));
  sh.dpb = scr(sub(pos, B.bmin), 0.5f * B.sz);
  float3 cols[8];
  load_colors(s, B.data_offset + s.v_size * s.v_size * s.v_size, cols);
  sh.color = tri3(cols, sh.dpb);
}

// CalculateColorWithGrad (diff_render/MultiRendererDR.cpp:902-979)
__device__ float3 color_grad(const DevPreset &p, float t, float3 hcolor, float3 hnormal, M3 &dCdD, M3 &dCdN) {
  const float3 z = f3(0, 0, 0);
  float3 c = f3(1, 0, 1);
  switch (p.render_mode) {
    case R_DIFFUSE:
      c = hcolor;
      dCdD = M3{f3(1, 0, 0), f3(0, 1, 0), f3(0, 0, 1)};
      dCdN = M3{z, z, z};
      break;
    case R_LAMBERT:
      c = z;
      dCdD = M3{z, z, z};
      dCdN = M3{z, z, z};
      for (uint32_t i = 0; i < p.n_lights; i++) {
        const float3 lc = f3(p.light_col[i][0], p.light_col[i][1], p.light_col[i][2]);
        if (p.light_type[i] == 0) {
          const float3 sp = f3(p.light_dir[i][0], p.light_dir[i][1], p.light_dir[i][2]);
          const float q = mx(0.0f, dot(hnormal, sp));
          c = add(c, scr(mul(lc, hcolor), q));
          if (q > 0.0f) {
            dCdD.r0 = add(dCdD.r0, f3(lc.x * q, 0, 0));
            dCdD.r1 = add(dCdD.r1, f3(0, lc.y * q, 0));
            dCdD.r2 = add(dCdD.r2, f3(0, 0, lc.z * q));
            dCdN.r0 = add(dCdN.r0, scl(lc.x * hcolor.x, sp));
            dCdN.r1 = add(dCdN.r1, scl(lc.y * hcolor.y, sp));
            dCdN.r2 = add(dCdN.r2, scl(lc.z * hcolor.z, sp));
          }
        } else {
          c = add(c, mul(lc, hcolor));
          dCdD.r0 = add(dCdD.r0, f3(lc.x, 0, 0));
          dCdD.r1 = add(dCdD.r1, f3(0, lc.y, 0));
          dCdD.r2 = add(dCdD.r2, f3(0, 0, lc.z));
        }
      }
      break;
    case R_MASK:
      c = f3(1, 1, 1);
      dCdD = M3{z, z, z};
      dCdN = M3{z, z, z};
      break;
    case R_LINEAR_DEPTH: {
      const float d = (t - 0.1f) / (10.0f - 0.1f);
      c = f3(d, d, d);
    } break;
    case R_NORMAL:
      c = hnormal;
      dCdD = M3{z, z, z};
      dCdN = M3{f3(1, 0, 0), f3(0, 1, 0), f3(0, 0, 1)};
      break;
    default: break;
  }
  return c;
}

// Gradient scatter.  With warp aggregation every lane of the warp must call it
// (converged); lanes adding to the same index are summed through shared memory
// and one lane issues the global atomic.
__device__ __forceinline__ void scatter(const DevPreset &p, float *grad, float *ws, uint32_t idx, float v, bool valid) {
  if (!p.agg) {
    if (valid) atomicAdd(grad + idx, v);
    return;
  }
  const int lane = threadIdx.x & 31;
  const uint32_t key = valid ? idx : 0xFFFFFFFFu;
  const unsigned peers = __match_any_sync(0xFFFFFFFFu, key);
  const int leader = __ffs(peers) - 1;
  if (peers == (1u << lane)) {              // no peer: direct
    if (valid) atomicAdd(grad + idx, v);
    return;
  }
  if (lane == leader) ws[lane] = 0.0f;
  __syncwarp(peers);
  if (valid) atomicAdd(&ws[leader], v);
  __syncwarp(peers);
  if (valid && lane == leader) atomicAdd(grad + idx, ws[lane]);
  __syncwarp(peers);
}

// The distance/normal/diffuse PDs of one hit sample, scattered as
// dot(dL, dCdD*dDiffuse + dCdN*dNorm) * g_mult (CastRayWithGrad :1181-1271).
// Every lane of the warp calls this (act false for lanes without a hit).
__device__ void scatter_hit_pds(const DevScene &s, const DevPreset &p, const HitRec &hr, const Shade &sh, float3 dL,
                                const M3 &dCdD, const M3 &dCdN, bool act, float *ws) {
  const uint32_t flags = p.flags;
  const float gm = p.g_mult;
  Brick B;
  float values[8] = {0, 0, 0, 0, 0, 0, 0, 0}, dt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t mi[8] = {kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex};
  if (act) {
    B = brick_of(s, hr.prim);
    load_vals(s, hr.prim, hr.vox, values);
    load_idx(s, B.data_offset, hr.vox, mi);
  }
  // colour PDs (:1500-1510, 1217-1225)
  if (flags & F_DCOLOR) {
    const uint32_t t_off = act ? B.data_offset + s.v_size * s.v_size * s.v_size : 0;
#pragma unroll 1
    for (int i = 0; i < 8; i++) {
      float3 diff = f3(0, 0, 0);
      uint32_t ci = kNoIndex;
      if (act) {
        const float3 q = f3(float((i & 4) >> 2), float((i & 2) >> 1), float(i & 1));
        const float3 one = f3(1, 1, 1);
        const float3 lq = add(mul(q, sh.dpb), mul(sub(one, q), sub(one, sh.dpb)));
        const float val = lq.x * lq.y * lq.z;
        ci = __ldg(&s.values[t_off + i]);
        diff = mul(dL, mv(dCdD, f3(val, val, val)));
      }
      const bool ok = act && ci != kNoIndex;
      scatter(p, s.grad, ws, ci + 0, diff.x * gm, ok);
      scatter(p, s.grad, ws, ci + 1, diff.y * gm, ok);
      scatter(p, s.grad, ws, ci + 2, diff.z * gm, ok);
    }
  }
  if (!(flags & (F_DDIFFUSE | F_DNORM | F_DDIST))) return;
  if (act) dintersect(values, B.d, hr.qFar, hr.start_q, hr.dir, dt);
  if (flags & F_DDIST) {   // depth input: dFinalColor = float3(d*dt)/(z_far - z_near)
#pragma unroll 1
    for (int j = 0; j < 8; j++) {
      float v = 0.0f;
      if (act) {
        const float q = B.d * dt[j];
        const float3 fc = divs(f3(q, q, q), 10.0f - 0.1f);
        v = dot(dL, fc) * gm;
      }
      scatter(p, s.grad, ws, mi[j], v, act && mi[j] != kNoIndex);
    }
    return;
  }
  // main-voxel slots: dDiffuse, dNorm accumulated in the reference's order
  float3 acc[8];
#pragma unroll
  for (int j = 0; j < 8; j++) acc[j] = f3(0, 0, 0);
  const bool dnorm = (flags & F_DNORM) && s.need_normal;
  if (dnorm && s.layout_in) {
    float dtri[8];
    tri_w(dtri, sh.nmq);
    const M3 Mf = act ? nrm_diff(sh.tr3) : M3{};
#pragma unroll 1
    for (int i = 0; i < 8; i++) {
      float vn[8];
      uint32_t in_[8] = {kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex, kNoIndex};
      bool valid = false;
      M3 Mi, D2;
      float3 ndp = f3(0, 0, 0);
      if (act) {
        const Nbr n = neighbour(s, hr.prim, B.data_offset, hr.vox, sh.dp, i);
        valid = n.node != kInvalidIdx;
        if (valid) {
          load_vals(s, n.node, n.nvox, vn);
          load_idx(s, __ldg(&s.nodes[n.node]).z, n.nvox, in_);
          ndp = sub(sh.dp, n.dvox);
          const float3 g = tri_diff(vn, ndp);
          Mi = nrm_diff(g);
          D2 = tri_ddp_ddp(vn, ndp);
        }
      }
      const bool own = valid && i == (int)sh.k;
      const bool final_i = valid && len3(sh.nrm[i]) > 0.5f;
#pragma unroll 1
      for (int j = 0; j < 8; j++) {
        float v = 0.0f;
        if (valid) {
          const float3 term = scl(dtri[i], mv(Mi, ddp_dvalue(ndp, j)));
          if (own) {
            acc[j] = add(acc[j], term);
          } else {
            const float3 dn = final_i ? mv(Mf, term) : term;
            const float3 fc = add(mv(dCdD, f3(0, 0, 0)), mv(dCdN, dn));
            v = dot(dL, fc) * gm;
          }
        }
        scatter(p, s.grad, ws, in_[j], v, valid && !own && in_[j] != kNoIndex);
      }
      if (valid) {
        const float3 t1 = mv(D2, hr.dir);
#pragma unroll
        for (int j = 0; j < 8; j++)
          acc[j] = add(acc[j], scl(dtri[i], mv(Mi, f3(t1.x * dt[j], t1.y * dt[j], t1.z * dt[j]))));
      }
    }
    if (act) {
      const M3 dT = tri3_ddp(sh.nrm, sh.nmq);
      const float3 dnmq = f3(1, 1, 1);
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j] = add(acc[j], mv(dT, mul(dnmq, scr(hr.dir, dt[j]))));
      if (len3(sh.nrm[sh.k]) > 0.5f) {
#pragma unroll
        for (int j = 0; j < 8; j++) acc[j] = mv(Mf, acc[j]);
      }
    }
  } else if (dnorm && act) {   // flat normal of the hit voxel (:1460-1487)
    const M3 M = nrm_diff(tri_diff(values, sh.dp));
    const M3 D2 = tri_ddp_ddp(values, sh.dp);
    const float3 t1 = mv(D2, hr.dir);
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const float3 c = ddp_dvalue(sh.dp, j);
      acc[j] = mv(M, f3(c.x + t1.x * dt[j], c.y + t1.y * dt[j], c.z + t1.z * dt[j]));
    }
  }
  M3 dL1;
  if (act && (flags & F_DDIFFUSE)) {
    float3 cols[8];
    load_colors(s, B.data_offset + s.v_size * s.v_size * s.v_size, cols);
    dL1 = tri3_ddp(cols, sh.dpb);
  }
#pragma unroll 1
  for (int j = 0; j < 8; j++) {
    float v = 0.0f;
    if (act) {
      float3 ddf = f3(0, 0, 0);
      if (flags & F_DDIFFUSE) {
        const float hs = 0.5f * B.sz;
        ddf = mv(dL1, f3(hs * hr.dir.x * dt[j], hs * hr.dir.y * dt[j], hs * hr.dir.z * dt[j]));
      }
      const float3 fc = add(mv(dCdD, ddf), mv(dCdN, acc[j]));
      v = dot(dL, fc) * gm;
    }
    scatter(p, s.grad, ws, mi[j], v, act && mi[j] != kNoIndex);
  }
}

// t_samples_to_threshold (diff_render/MultiRendererDR.cpp:995-1061)
__device__ float t_threshold(const float *samples, uint32_t count, float dv, uint32_t dcount) {
  float dmin = samples[0], dmax = samples[0];
  for (uint32_t i = 1; i < count; i++) { dmin = mn(dmin, samples[i]); dmax = mx(dmax, samples[i]); }
  if (dcount > 0) { dmin = mn(dmin, dv); dmax = mx(dmax, dv); }
  const float diff = mx(1e-9f, dmax - dmin);
  uint32_t g[10];
#pragma unroll
  for (int i = 0; i < 10; i++) g[i] = 0;
  for (uint32_t i = 0; i <= count; i++) {
    const float b = ((i < count ? samples[i] : dv) - dmin) / diff * 10;
    const int bi = b >= 9.0f ? 9 : (b <= 0.0f ? 0 : (int)b);
    g[bi] += i < count ? 1u : dcount;
  }
  int max_len = 0, max_start = -1, start = -1;
  for (int i = 1; i < 10; i++) {
    if (start != -1) {
      if (g[i] != 0) {
        const int l = i - start;
        if (l > max_len) { max_len = l; max_start = start; }
        start = -1;
      }
    } else if (g[i] == 0) {
      start = i;
    }
  }
  if (max_len > 4) return dmin + diff * (max_start + 0.5f * max_len) / 10;
  return 0.0f;
}

// pixel tile: a block of 128 threads covers 16x8 pixels, each warp 8x4
__global__ void __launch_bounds__(128) dr_pixel_kernel(DevScene s, DevPreset p, DevView v) {
  __shared__ float ws_all[4][32];
  float *ws = ws_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t x = blockIdx.x * 16 + (w & 1) * 8 + (lane & 7);
  const uint32_t y = blockIdx.y * 8 + (w >> 1) * 4 + (lane >> 3);
  // a pixel outside the ray-casting mask is not cast (CastRayWithGrad :1097-1100):
  // no image, depth, loss or gradient; its mask entry stays 0
  const bool in = x < v.width && y < v.height && (!v.cast_mask || v.cast_mask[(size_t)y * v.width + x]);
  const uint32_t spp = p.spp;
  float3 res = f3(0, 0, 0);
  uint32_t hit_count = 0;
  float samples[kMaxSpp];
  HitRec hr;
  Shade sh;
  M3 dCdD{}, dCdN{};
  bool hit1 = false;
  if (in) {
    for (uint32_t i = 0; i < spp; i++) {
      const float2 d = rand2(x, y, i, p.seed);
      float3 P, D;
      eye_ray(x, y, v.width, v.height, d.x, d.y, v.proj_inv, v.wv_inv, P, D);
      query<false>(s, P, D, 1e9f, hr, nullptr);
      if (hr.prim == kNoIndex) continue;
      shade_hit(s, hr, sh, (p.flags & (F_DDIFFUSE | F_DNORM | F_DDIST)) != 0);
      dCdD = M3{f3(1, 0, 0), f3(0, 1, 0), f3(0, 0, 1)};
      dCdN = M3{f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0)};
      const float3 c = color_grad(p, hr.t, sh.color, sh.normal, dCdD, dCdN);
      res = add(res, divs(c, float(spp)));
      samples[hit_count] = hr.t;
      hit_count++;
    }
  }
  float3 dL = f3(0, 0, 0);
  double loss = 0.0;
  if (in) {
    const size_t px = (size_t)y * v.width + x;
    if (v.cast_mask) v.cast_mask[px] = hit_count > 0 ? 1 : 0;   // process_mask -> masks[image] (:443-448, :1164-1167)
    const float4 cm = make_float4(res.x, res.y, res.z, float(hit_count) / float(spp));
    v.img[px] = cm;
    v.depth[px] = hit_count == 0 ? 0.0f : t_threshold(samples, hit_count, 1e9f, spp - hit_count);
    const float4 rf = __ldg(&v.ref[px]);
    float lg[4];
    const float dd[4] = {cm.x - rf.x, cm.y - rf.y, cm.z - rf.z, cm.w - rf.w};
    float l;
    if (p.loss_fn == 0) {
      l = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2] + dd[3] * dd[3];
#pragma unroll
      for (int k = 0; k < 4; k++) lg[k] = 2.0f * dd[k];
    } else {
      l = fabsf(dd[0]) + fabsf(dd[1]) + fabsf(dd[2]) + fabsf(dd[3]);
#pragma unroll
      for (int k = 0; k < 4; k++) lg[k] = dd[k] < 0 ? -1.0f : 1.0f;
    }
    loss = (double)l;
    dL = divs(scr(f3(lg[0], lg[1], lg[2]), 1.0f), float(spp));
    hit1 = hit_count > 0;
  }
  // pixel losses: warp sum then one double atomic per warp
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) loss += __shfl_down_sync(0xFFFFFFFFu, loss, o);
  if (lane == 0) atomicAdd(v.loss, loss);
  if (!(p.flags & (F_DCOLOR | F_DDIFFUSE | F_DNORM | F_DDIST))) return;
  if (spp == 1) {
    // the single sample's hit record and shading are still live: no re-trace
    M3 a = dCdD, b = dCdN;
    scatter_hit_pds(s, p, hr, sh, dL, a, b, hit1, ws);
    return;
  }
  // spp > 1: re-trace every sample, recompute its shading, scatter its PDs
  for (uint32_t i = 0; i < spp; i++) {
    bool act = false;
    if (in && hit1) {
      const float2 d = rand2(x, y, i, p.seed);
      float3 P, D;
      eye_ray(x, y, v.width, v.height, d.x, d.y, v.proj_inv, v.wv_inv, P, D);
      query<false>(s, P, D, 1e9f, hr, nullptr);
      act = hr.prim != kNoIndex;
      if (act) {
        shade_hit(s, hr, sh, true);
        dCdD = M3{f3(1, 0, 0), f3(0, 1, 0), f3(0, 0, 1)};
        dCdN = M3{f3(0, 0, 0), f3(0, 0, 0), f3(0, 0, 0)};
        color_grad(p, hr.t, sh.color, sh.normal, dCdD, dCdN);
      }
    }
    scatter_hit_pds(s, p, hr, sh, dL, dCdD, dCdN, act, ws);
  }
}

// border pixels (RenderDR :609-685): 3x3 alpha difference or depth threshold
__global__ void dr_border_detect_kernel(DevPreset p, DevView v) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t N = v.width * v.height;
  bool is_border = false;
  if (i < N) {
    const uint32_t x = i % v.width, y = i / v.width;
    const float d0 = v.img[i].w;
    float max_diff = 0.0f, max_thr = 0.0f;
    if (x >= 1 && x < v.width - 1 && y >= 1 && y < v.height - 1)
      for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++) {
          const size_t q = (size_t)(y + dy) * v.width + x + dx;
          max_diff = mx(max_diff, fabsf(d0 - v.img[q].w));
          max_thr = mx(max_thr, v.depth[q]);
        }
    is_border = p.render_mode == R_MASK ? max_diff > 0 : (max_diff > 0 || max_thr > 0);
    v.border_mask[i] = is_border ? 1 : 0;
  }
  const unsigned b = __ballot_sync(0xFFFFFFFFu, is_border);
  const int lane = threadIdx.x & 31;
  uint32_t base = 0;
  if (lane == 0 && b) base = atomicAdd(v.border_count, __popc(b));
  base = __shfl_sync(0xFFFFFFFFu, base, 0);
  if (is_border) v.border_list[base + __popc(b & ((1u << lane) - 1))] = i;
}

// CalculateColor (:855-900)
__device__ __forceinline__ float3 color_plain(const DevPreset &p, float t, float3 c, float3 n) {
  M3 a, b;
  return color_grad(p, t, c, n, a, b);
}

// SVM_fit (:1518-1546) on rows (x, y, 1) * label, scaled in place by etha
__device__ float4 svm_fit(float *xs, float *ys, float *zs, uint32_t N) {
  const float etha = 0.01f, alpha = 0.1f;
  const int epochs = 200;
  for (uint32_t i = 0; i < N; i++) { xs[i] = xs[i] * etha; ys[i] = ys[i] * etha; zs[i] = zs[i] * etha; }
  uint32_t errors = N;
  float w0 = -1.0f, w1 = 1.0f, w2 = 0.0f;
  const float mult = 1.0f - etha * alpha / float(epochs);
  for (int e = 0; e < epochs && errors > 0; e++) {
    errors = 0;
    for (uint32_t j = 0; j < N; j++) {
      const float margin = w0 * xs[j] + w1 * ys[j] + w2 * zs[j];
      w0 = w0 * mult; w1 = w1 * mult; w2 = w2 * mult;
      if (margin < 0) {
        w0 = w0 + xs[j]; w1 = w1 + ys[j]; w2 = w2 + zs[j];
        errors++;
      }
    }
  }
  return make_float4(w0, w1, w2, float(errors) / float(N));
}

__device__ __forceinline__ uint32_t out_code(float x, float y) {   // ComputeOutCode (:1552-1578)
  uint32_t c = 0;
  if (x < 0.0f) c |= 1u; else if (x > 1.0f) c |= 2u;
  if (y < 0.0f) c |= 4u; else if (y > 1.0f) c |= 8u;
  return c;
}

// CohenSutherlandLineClip (:1580-1649) against [0,1]^2.  Each pass moves one end
// onto a window edge, after which that end's code loses the bit it was moved
// for; four passes settle every segment, eight bound the loop.
__device__ bool line_clip(float &x0, float &y0, float &x1, float &y1) {
  uint32_t c0 = out_code(x0, y0), c1 = out_code(x1, y1);
  for (int it = 0; it < 8; it++) {
    if (!(c0 | c1)) return true;
    if (c0 & c1) return false;
    float x = -1, y = -1;
    const uint32_t co = c1 > c0 ? c1 : c0;
    if (co & 8u) { x = x0 + (x1 - x0) * (1.0f - y0) / (y1 - y0); y = 1.0f; }
    else if (co & 4u) { x = x0 + (x1 - x0) * (0.0f - y0) / (y1 - y0); y = 0.0f; }
    else if (co & 2u) { y = y0 + (y1 - y0) * (1.0f - x0) / (x1 - x0); x = 1.0f; }
    else if (co & 1u) { y = y0 + (y1 - y0) * (0.0f - x0) / (x1 - x0); x = 0.0f; }
    if (co == c0) { x0 = x; y0 = y; c0 = out_code(x0, y0); }
    else { x1 = x; y1 = y; c1 = out_code(x1, y1); }
  }
  return false;
}

__device__ __forceinline__ float2 w2s(const float pv[16], float3 q) {   // TransformWorldToScreenSpace (:1296-1301)
  float r[4];
  const float q4[4] = {q.x, q.y, q.z, 1.0f};
  mat_vec4(pv, q4, r);
  return make_float2(0.5f * (r[0] / r[3] + 1.0f), 1.0f - 0.5f * (r[1] / r[3] + 1.0f));
}

// The SVM stage of CastBorderRaySVM (:1651-1816) for every border pixel: a warp
// casts the svm_spp classification rays, then one lane labels them by the depth
// threshold, fits the SVM and derives the pixel's sampling line.
__global__ void __launch_bounds__(128) dr_svm_kernel(DevScene s, DevPreset p, DevView v) {
  __shared__ float sh_t[4][kMaxSvm], sh_x[4][kMaxSvm], sh_y[4][kMaxSvm], sh_z[4][kMaxSvm];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  float *ts = sh_t[wl], *xs = sh_x[wl], *ys = sh_y[wl], *zs = sh_z[wl];
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t nb = *v.border_count;
  const uint32_t W = v.width, H = v.height, N = p.svm_spp, sq = p.svm_sqrt;
  const float isq = 1.0f / float(sq);
  for (uint32_t b = warp; b < nb; b += n_warps) {
    const uint32_t pix = v.border_list[b];
    const uint32_t x = pix % W, y = pix / W;
    for (uint32_t k = lane; k < N; k += 32) {
      const float2 rnd = rand2(x, y, k, p.seed);
      const float dx = isq * (float(k / sq) + rnd.x), dy = isq * (float(k % sq) + rnd.y);
      float3 P, D;
      eye_ray(x, y, W, H, dx, dy, v.proj_inv, v.wv_inv, P, D);
      HitRec hr;
      query<false>(s, P, D, 1e9f, hr, nullptr);
      ts[k] = hr.t;
      xs[k] = dx;
      ys[k] = dy;
    }
    __syncwarp();
    if (lane == 0) {
      SvmLine L{};
      // closest classification hit (first of equal t), from its recomputed ray
      float closest_t = 1e6f;
      uint32_t ck = N;
      for (uint32_t k = 0; k < N; k++)
        if (ts[k] < closest_t) { closest_t = ts[k]; ck = k; }
      float3 closest = f3(1e6f, 1e6f, 1e6f);
      if (ck < N) {
        float3 P, D;
        eye_ray(x, y, W, H, xs[ck], ys[ck], v.proj_inv, v.wv_inv, P, D);
        closest = add(P, scl(ts[ck], D));
      }
      const float thr = t_threshold(ts, N, 0.0f, 0u);
      uint32_t type0 = 0;
      for (uint32_t k = 0; k < N; k++) {
        const float lab = ts[k] <= thr ? -1.0f : 1.0f;
        type0 += ts[k] <= thr ? 1u : 0u;
        xs[k] *= lab; ys[k] *= lab; zs[k] = lab;   // (x, y, 1) * label
      }
      bool keep = !(type0 == N || type0 == 0);
      if (keep) {
        const float4 Wt = svm_fit(xs, ys, zs, N);
        const float err = Wt.w;
        const float f0 = float(type0) / float(N);
        const float rare = mn(f0, 1.0f - f0);
        float p0x = 0, p0y = 0, p1x = 0, p1y = 0, rx = 0, ry = 0, nx = 0, ny = 0, radius = 0, area = 0;
        bool force = false;
        if (err > 0.05f || 2 * err > rare) {
          force = true;
          area = 1.0f;
        } else {
          if (fabsf(Wt.y) > 1e-6f && fabsf(Wt.x) > 1e-6f) {
            p0x = 0.0f; p0y = -Wt.z / Wt.y;
            p1x = 1.0f; p1y = (-Wt.z - Wt.x) / Wt.y;
            const float rY = p1y - p0y;
            if (p0y < -1e-6f || p0y > 1 + 1e-6f) {
              const float k1 = -p0y / rY, k2 = (1 - p0y) / rY, k = (fabsf(k1) < fabsf(k2)) ? k1 : k2;
              p0x = p0x + k * 1.0f; p0y = p0y + k * rY;
            }
            if (p1y < -1e-6f || p1y > 1 + 1e-6f) {
              const float k1 = -p1y / rY, k2 = (1 - p1y) / rY, k = (fabsf(k1) < fabsf(k2)) ? k1 : k2;
              p1x = p1x + k * 1.0f; p1y = p1y + k * rY;
            }
          } else if (fabsf(Wt.x) > 1e-6f) {
            p0x = -Wt.z / Wt.x; p0y = 0.0f;
            p1x = -Wt.z / Wt.x; p1y = 1.0f;
          } else {
            force = true;
          }
          keep = line_clip(p0x, p0y, p1x, p1y);
          if (keep) {
            const float2 a = w2s(v.pv, closest);
            const float2 c = w2s(v.pv, add(closest, scl(p.relax_eps, f3(v.up[0], v.up[1], v.up[2]))));
            const float ddx = c.x - a.x, ddy = c.y - a.y;
            const float thick = sqrtf(ddx * ddx + ddy * ddy) * float(W > H ? W : H);
            radius = mx(0.15f, thick) + 2.0f * err;
            rx = p1x - p0x; ry = p1y - p0y;
            float l = sqrtf(rx * rx + ry * ry);
            const float ux = rx / l, uy = ry / l;
            p0x = p0x - radius * ux; p0y = p0y - radius * uy;
            p1x = p1x + radius * ux; p1y = p1y + radius * uy;
            rx = p1x - p0x; ry = p1y - p0y;
            l = sqrtf(ry * ry + rx * rx);
            nx = -ry / l; ny = rx / l;
            area = 2 * radius * sqrtf(rx * rx + ry * ry);
            keep = force || !(area < 0.005f);
          }
        }
        if (keep) {
          const float area_mult = mn(1.0f, 0.05f + 2.0f * area);
          uint32_t cnt = (uint32_t)(area_mult * float(p.border_spp - N));
          if (cnt < 1u) cnt = 1u;
          L.count = cnt;
          L.force = force ? 1u : 0u;
          L.p0x = p0x; L.p0y = p0y; L.rx = rx; L.ry = ry; L.nx = nx; L.ny = ny;
          L.radius = radius;
          L.pdf = force ? 1.0f / float(cnt) : area / float(cnt);
        }
      }
      v.svm[b] = L;
    }
    __syncwarp();
  }
}

// CastBorderRay / CastBorderRaySVM + CalculateBorderRayDerivatives
// (:1319-1499, :1816-1869): a warp per (border pixel, 32 of its samples),
// grid-stride over the compacted list.  SVM: the samples of the pixel's line
// (dr_svm_kernel), sample index svm_spp + j; the reference's urand() stream is
// replaced by rand2 of the sample index (the oracle draws the same).
template <bool SVM>
__global__ void __launch_bounds__(128, 4) dr_border_kernel(DevScene s, DevPreset p, DevView v) {
  __shared__ float ws_all[4][32];
  float *ws = ws_all[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t nb = *v.border_count;
  const uint32_t W = v.width, H = v.height;
  // work item = (border pixel, chunk of 32 samples): a pixel's samples spread over
  // several warps so that the few border pixels still fill the GPU
  const uint32_t n_max = SVM ? max(1u, p.border_spp - p.svm_spp) : p.border_spp;   // a line's count is at most this
  const uint32_t chunks = (n_max + 31) / 32;
  for (uint32_t item = warp; item < nb * chunks; item += n_warps) {
    const uint32_t bi = item / chunks;
    const uint32_t pix = v.border_list[bi];
    const uint32_t x = pix % W, y = pix / W;
    {
      const uint32_t sid = (item % chunks) * 32 + lane;
      HitRec hr;
      Relax rl;
      bool br = false;
      float3 P = f3(0, 0, 0), D = f3(0, 0, 0);
      float pdf = 1.0f / float(p.border_spp);
      if (SVM) {
        const SvmLine L = v.svm[bi];
        pdf = L.pdf;
        if (sid < L.count) {
          const float2 u = rand2(x, y, p.svm_spp + sid, p.seed);
          float2 d = u;
          if (!L.force) {
            const float a = u.x, br_ = (u.y * 2.0f - 1.0f) * L.radius;
            d = make_float2((L.p0x + a * L.rx) + br_ * L.nx, (L.p0y + a * L.ry) + br_ * L.ny);
          }
          if (d.x > 0 && d.x < 1 && d.y > 0 && d.y < 1) {
            eye_ray(x, y, W, H, d.x, d.y, v.proj_inv, v.wv_inv, P, D);
            border_query(s, P, D, p.relax_eps, hr, rl);
            br = rl.sdf < p.relax_eps;
          }
        }
      } else if (sid < p.border_spp) {
        const float2 d = rand2(x, y, sid, p.seed);
        eye_ray(x, y, W, H, d.x, d.y, v.proj_inv, v.wv_inv, P, D);
        border_query(s, P, D, p.relax_eps, hr, rl);
        br = rl.sdf < p.relax_eps;
      }
      float cd[4] = {0, 0, 0, 0};
      if (br) {
        const bool miss = hr.prim == kNoIndex;
        if (p.input_type == 0) {
          const float3 fin = color_plain(p, rl.t, rl.color, rl.normal);
          float3 fout = f3(0, 0, 0);
          if (!miss) {
            Shade sh;
            shade_hit(s, hr, sh, false);
            fout = color_plain(p, hr.t, sh.color, sh.normal);
          }
          const float3 dd = sub(fin, fout);
          cd[0] = dd.x; cd[1] = dd.y; cd[2] = dd.z; cd[3] = miss ? 1.0f : 0.0f;
        } else {
          const float din = (rl.t - 0.1f) / (10.0f - 0.1f), dout = miss ? 0.0f : (hr.t - 0.1f) / (10.0f - 0.1f);
          cd[0] = cd[1] = cd[2] = din - dout;
          cd[3] = miss ? 1.0f : 0.0f;
        }
      }
#pragma unroll 1
      for (int j = 0; j < 8; j++) {
        float diff = 0.0f;
        bool ok = br && rl.idx[j] != kNoIndex;
        if (ok) {
          const float bd = mx(0.0f, rl.sdf);
          const float3 ys = add(P, scl(rl.t, D));
          const float3 xs = sub(ys, scl(bd, rl.normal));
          float r[4];
          const float pv4[4] = {xs.x, xs.y, xs.z, 1.0f};
          mat_vec4(v.pv, pv4, r);
          const float sx = 0.5f * (r[0] / r[3] + 1.0f), sy = 1.0f - 0.5f * (r[1] / r[3] + 1.0f);
          const float fx = sx * float(W), fy = sy * float(H);
          // the reference converts to unsigned unchecked; projections outside the
          // image (an out-of-bounds read there) are skipped
          ok = fx >= 0.0f && fx < float(W) && fy >= 0.0f && fy < float(H);
          if (ok) {
            const uint32_t xp = (uint32_t)fx, yp = (uint32_t)fy;
            ok = xp < W && yp < H;
            if (ok) {
              const float4 o = v.img[(size_t)yp * W + xp], rf = __ldg(&v.ref[(size_t)yp * W + xp]);
              const float dd[4] = {o.x - rf.x, o.y - rf.y, o.z - rf.z, o.w - rf.w};
              float lg[4];
#pragma unroll
              for (int k = 0; k < 4; k++) lg[k] = p.loss_fn == 0 ? 2.0f * dd[k] : (dd[k] < 0 ? -1.0f : 1.0f);
              const float dtp = lg[0] * cd[0] + lg[1] * cd[1] + lg[2] * cd[2] + lg[3] * cd[3];
              diff = pdf * (1.0f / p.relax_eps) * dtp * rl.dth[j] * p.g_mult;
            }
          }
        }
        scatter(p, s.grad, ws, ok ? rl.idx[j] : kNoIndex, diff, ok);
      }
    }
  }
}

// OptimizeStepAdam (:828-853) after the batch division (:475-476), in the
// reference's arithmetic: the bias corrections 1 - beta^(iter+1) are doubles
// (pow of a float and an unsigned), V and S are divided by them in double and
// rounded to float, the update lr * Vh / (sqrt(Sh) + eps) is float with a float
// square root, and the result is clamped to +-1000 (LiteMath::clamp).  Given the
// same gradient, the parameters and moments equal the reference's bit for bit.
__global__ void dr_adam_kernel(float *x, float *V, float *S, const float *g, uint32_t n, float batch, float lr,
                               float b1, float b2, float eps, double c1, double c2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i] / batch;
    const float Vi = b1 * V[i] + (1 - b1) * gi;
    V[i] = Vi;
    const float Vh = float(double(Vi) / c1);
    const float Si = b2 * S[i] + (1 - b2) * gi * gi;
    S[i] = Si;
    const float Sh = float(double(Si) / c2);
    x[i] = clampf(x[i] - lr * Vh / (sqrtf(Sh) + eps), -1000.0f, 1000.0f);
  }
}

// RayQuery_NearestHitWithGrad on a batch of rays (diff_render/BVH2DR.cpp:12-102):
// the hit (t, primId, colour, normal) and the border relaxation point (t, sdf,
// colour, normal, indices, dSDF/dtheta), 32 words per ray
__global__ void dr_query_kernel(DevScene s, uint32_t flags, float relax_eps, const float4 *pos, const float4 *dir,
                                uint32_t n, uint32_t *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 P4 = pos[i], D4 = dir[i];
  const float3 P = f3(P4.x, P4.y, P4.z), D = f3(D4.x, D4.y, D4.z);
  // the reference's ray query takes tFar from dir.w (a non-positive w asks for any-hit: its magnitude)
  const float tfar = D4.w <= 0.0f ? -D4.w : D4.w;
  HitRec hr;
  Relax rl;
  if (flags & F_BORDER_EARLY) {   // the border integral's walk (early skipping below relax_eps)
    border_query(s, P, D, relax_eps, hr, rl, tfar);
  } else if (flags & F_BORDER) {
    query<true>(s, P, D, tfar, hr, &rl);
  } else {
    query<false>(s, P, D, tfar, hr, nullptr);
    rl.t = tfar; rl.sdf = 1000.0f;
    rl.color = f3(0, 0, 0); rl.normal = f3(1, 0, 0);
#pragma unroll
    for (int k = 0; k < 8; k++) { rl.idx[k] = kNoIndex; rl.dth[k] = 0.0f; }
  }
  uint32_t *o = out + 32 * (size_t)i;
  float3 hc = f3(0, 0, 0), hn = f3(1, 0, 0);
  float ht = tfar;
  if (hr.prim != kNoIndex) {
    Shade sh;
    shade_hit(s, hr, sh, (flags & (F_DDIFFUSE | F_DNORM | F_DDIST)) != 0);
    hc = sh.color;
    hn = sh.normal;
    ht = hr.t;
  }
  o[0] = __float_as_uint(ht);
  o[1] = hr.prim;
  o[2] = __float_as_uint(hc.x); o[3] = __float_as_uint(hc.y); o[4] = __float_as_uint(hc.z);
  o[5] = __float_as_uint(hn.x); o[6] = __float_as_uint(hn.y); o[7] = __float_as_uint(hn.z);
  o[8] = __float_as_uint(rl.t); o[9] = __float_as_uint(rl.sdf);
  o[10] = __float_as_uint(rl.color.x); o[11] = __float_as_uint(rl.color.y); o[12] = __float_as_uint(rl.color.z);
  o[13] = __float_as_uint(rl.normal.x); o[14] = __float_as_uint(rl.normal.y); o[15] = __float_as_uint(rl.normal.z);
#pragma unroll
  for (int k = 0; k < 8; k++) { o[16 + k] = rl.idx[k]; o[24 + k] = __float_as_uint(rl.dth[k]); }
}

void launch_query(const DevScene &s, uint32_t flags, float relax_eps, const float4 *pos, const float4 *dir, uint32_t n,
                  uint32_t *out, cudaStream_t st) {
  dr_query_kernel<<<(n + 127) / 128, 128, 0, st>>>(s, flags, relax_eps, pos, dir, n, out);
}

// per brick: its distance values gathered from the parameters (a float copy in
// the brick's own order) with their min v and max |v| (one warp per brick), and
// per voxel the min and max |.| of its 8 corner values, folded in the walks'
// corner order (what brick_visit tests before it loads a voxel's corners);
// refreshed whenever the parameters change
__global__ void dr_brick_bounds_kernel(const uint4 *nodes, const uint32_t *values, const float *P, uint32_t n_nodes,
                                       uint32_t v3, float2 *out, float *bvals, float2 *vbounds, uint32_t bsz,
                                       uint32_t v_size) {
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= n_nodes) return;
  const uint32_t off = __ldg(&nodes[warp]).z;
  float mn_ = 3.0e38f, mx_ = 0.0f;
  for (uint32_t k = lane; k < v3; k += 32) {
    const float v = __ldg(&P[__ldg(&values[off + k])]);
    bvals[(size_t)warp * v3 + k] = v;
    mn_ = fminf(mn_, v);
    mx_ = fmaxf(mx_, fabsf(v));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn_ = fminf(mn_, __shfl_xor_sync(0xFFFFFFFFu, mn_, o));
    mx_ = fmaxf(mx_, __shfl_xor_sync(0xFFFFFFFFu, mx_, o));
  }
  if (lane == 0) out[warp] = make_float2(mn_, mx_);
  __syncwarp();   // the warp's gathered values, for the per-voxel bounds
  const float *b = bvals + (size_t)warp * v3;
  const uint32_t b3 = bsz * bsz * bsz;
  for (uint32_t k = lane; k < b3; k += 32) {
    const uint32_t x = k / (bsz * bsz), y = (k / bsz) % bsz, z = k % bsz;
    float vmin = b[vid(x, y, z, v_size)], vmax = fabsf(vmin);
#pragma unroll
    for (int i = 1; i < 8; i++) {
      const float v = b[vid(x + ((i & 4) >> 2), y + ((i & 2) >> 1), z + (i & 1), v_size)];
      vmin = fminf(vmin, v);
      vmax = fmaxf(vmax, fabsf(v));
    }
    vbounds[(size_t)warp * b3 + k] = make_float2(vmin, vmax);
  }
}

void launch_brick_bounds(const DevScene &s, uint32_t n_nodes, float2 *out, cudaStream_t st) {
  const uint32_t v3 = s.v_size * s.v_size * s.v_size;
  dr_brick_bounds_kernel<<<(n_nodes + 7) / 8, 256, 0, st>>>(s.nodes, s.values, s.P, n_nodes, v3, out,
                                                             const_cast<float *>(s.bvals),
                                                             const_cast<float2 *>(s.vbounds), s.brick_size, s.v_size);
}

__global__ void dr_scale_kernel(float *g, uint32_t n, float s) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) g[i] *= s;
}

void launch_pixels(const DevScene &s, const DevPreset &p, const DevView &v, cudaStream_t st) {
  const dim3 grid((v.width + 15) / 16, (v.height + 7) / 8);
  dr_pixel_kernel<<<grid, 128, 0, st>>>(s, p, v);
}

void launch_border_detect(const DevPreset &p, const DevView &v, cudaStream_t st) {
  const uint32_t n = v.width * v.height;
  dr_border_detect_kernel<<<(n + 255) / 256, 256, 0, st>>>(p, v);
}

void launch_border(const DevScene &s, const DevPreset &p, const DevView &v, uint32_t max_pixels, int n_sm,
                   cudaStream_t st) {
  // warps take (border pixel, 32-sample chunk) items; enough resident warps to cover
  // the SMs, grid-stride beyond
  const uint32_t chunks = (p.border_spp + 31) / 32;
  uint32_t blocks = uint32_t((uint64_t(max_pixels) * chunks + 3) / 4 > 0xFFFFFFFFull ? 0xFFFFFFFFu
                                                                                     : (uint64_t(max_pixels) * chunks + 3) / 4);
  const uint32_t cap = (uint32_t)n_sm * 16;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  if (p.svm) dr_border_kernel<true><<<blocks, 128, 0, st>>>(s, p, v);
  else dr_border_kernel<false><<<blocks, 128, 0, st>>>(s, p, v);
}

void launch_svm_lines(const DevScene &s, const DevPreset &p, const DevView &v, uint32_t max_pixels, int n_sm,
                      cudaStream_t st) {
  uint32_t blocks = (max_pixels + 3) / 4;   // a warp per border pixel, grid-stride beyond the cap
  const uint32_t cap = (uint32_t)n_sm * 8;
  if (blocks > cap) blocks = cap;
  if (blocks == 0) blocks = 1;
  dr_svm_kernel<<<blocks, 128, 0, st>>>(s, p, v);
}

// Regularization (diff_render/MultiRendererDR.cpp:1933-2055): one thread per brick
// value (brick_size + 1 per axis, the reference's v_size), its in-brick neighbours
__global__ void dr_regularize_kernel(DevScene s, uint32_t n_nodes, float lambda, float power) {
  const uint32_t v = s.brick_size + 1, v3 = v * v * v;
  const uint64_t gid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (gid >= uint64_t(n_nodes) * v3) return;
  const uint32_t node = uint32_t(gid / v3), r = uint32_t(gid % v3);
  const uint32_t i0 = r / (v * v), j0 = (r / v) % v, k0 = r % v;
  const uint32_t idx = s.nodes[node].z + r;
  const uint32_t own = __ldg(&s.values[idx]);
  const float pv = __ldg(&s.P[own]);
  const bool has[6] = {i0 > 0, i0 < v - 1, j0 > 0, j0 < v - 1, k0 > 0, k0 < v - 1};
  const int step[6] = {-int(v * v), int(v * v), -int(v), int(v), -1, 1};
  float acc = 0.0f;
  bool first = true;
#pragma unroll
  for (int n = 0; n < 6; n++) {
    if (!has[n]) continue;
    float d = pv - __ldg(&s.P[__ldg(&s.values[int64_t(idx) + step[n]])]);
    const float sgn_d = d > 0.0f ? 1.0f : -1.0f;
    d = fabsf(d);
    const float c = lambda * power * sgn_d * powf(d, power - 1);
    acc = first ? c : acc + c;
    first = false;
  }
  if (!first) atomicAdd(&s.grad[own], acc);
}

// SolveEikonal (:2058-2120), f = 1
__device__ float solve_eikonal(float m0, float m1, float m2, float h) {
  float m[3] = {m0, m1, m2}, t;
  if (m[0] > m[1]) { t = m[0]; m[0] = m[1]; m[1] = t; }
  if (m[0] > m[2]) { t = m[0]; m[0] = m[2]; m[2] = t; }
  if (m[1] > m[2]) { t = m[1]; m[1] = m[2]; m[2] = t; }
  float dist_new = m[0] + h;
  if (dist_new > m[1]) {
    const float h_2 = h * h;
    float m_sum = m[0] + m[1], c_2 = (m[0] - m[1]) * (m[0] - m[1]);
    dist_new = (m_sum + sqrtf(2 * h_2 - c_2)) * 0.5f;
    if (dist_new > m[2]) {
      const float one_third = 1.f / 3;
      m_sum += m[2];
      c_2 = 3.f * (m[0] * m[0] + m[1] * m[1] + m[2] * m[2] - h_2);
      dist_new = (m_sum + sqrtf(m_sum * m_sum - c_2)) * one_third;
    }
  }
  return dist_new;
}

constexpr float kRedistBig = 99999.f;

// Redistance initialisation (:2170-2227): frozen surface nodes keep their values
__global__ void dr_redist_init_kernel(const float *dist, uint32_t n, float *b0, float *b1, uint8_t *frozen) {
  const uint64_t li = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t N = uint64_t(n) * n * n;
  if (li >= N) return;
  const int ix[3] = {int(li / (uint64_t(n) * n)), int((li / n) % n), int(li % n)};
  const int64_t off[3] = {int64_t(n) * n, int64_t(n), 1};
  bool fr = false;
  float v0 = kRedistBig;
  const float dv = dist[li];
  if (dv == 0.f) { fr = true; v0 = 0.f; }
  if (!fr)
    for (int dim = 0; dim < 3; dim++)
      for (int sg = -1; sg < 2; sg += 2) {
        const int q = ix[dim] + sg;
        if (q >= 0 && q < int(n) && dist[int64_t(li) + sg * off[dim]] * dv < 0) { v0 = dv; fr = true; }
      }
  b0[li] = v0;
  b1[li] = v0;
  frozen[li] = fr ? 1 : 0;
}

// One Jacobi update of all nodes (each iteration of the reference reads only the
// previous iteration's array, so its 8 sweep orderings compute these values)
__global__ void dr_redist_step_kernel(const float *old, float *nw, const uint8_t *frozen, uint32_t n, float h) {
  const uint64_t li = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t N = uint64_t(n) * n * n;
  if (li >= N) return;
  const float ov = old[li];
  if (frozen[li]) { nw[li] = ov; return; }
  const int ix[3] = {int(li / (uint64_t(n) * n)), int((li / n) % n), int(li % n)};
  const int64_t off[3] = {int64_t(n) * n, int64_t(n), 1};
  float am[3] = {kRedistBig, kRedistBig, kRedistBig};
#pragma unroll
  for (int dim = 0; dim < 3; dim++) {
    if (ix[dim] > 0 && ix[dim] < int(n) - 1) {
      am[dim] = old[int64_t(li) - off[dim]];
      const float tmp = old[int64_t(li) + off[dim]];
      if (fabsf(tmp) < fabsf(am[dim])) am[dim] = tmp;
    } else if (ix[dim] > 0 && ix[dim] == int(n) - 1) {
      am[dim] = old[int64_t(li) - off[dim]];
    } else if (ix[dim] == 0 && ix[dim] < int(n) - 1) {
      am[dim] = old[int64_t(li) + off[dim]];
    }
  }
  float r = ov;
  if (am[0] < kRedistBig || am[1] < kRedistBig || am[2] < kRedistBig) {
    if (am[0] >= 0.f && am[1] >= 0.f && am[2] >= 0.f) {
      const float e = solve_eikonal(am[0], am[1], am[2], h);
      r = e < ov ? e : ov;                              // std::min
    } else {
      for (int k = 0; k < 3; k++) if (am[k] < 0.f) am[k] = -am[k];
      const float e = -solve_eikonal(am[0], am[1], am[2], h), o = -fabsf(ov);
      r = e < o ? o : e;                                // std::max
    }
  }
  nw[li] = r;
}

void launch_regularize(const DevScene &s, uint32_t n_nodes, float lambda, float power, cudaStream_t st) {
  const uint64_t total = uint64_t(n_nodes) * (s.brick_size + 1) * (s.brick_size + 1) * (s.brick_size + 1);
  if (total == 0) return;
  dr_regularize_kernel<<<unsigned((total + 255) / 256), 256, 0, st>>>(s, n_nodes, lambda, power);
}

cudaError_t launch_redistance(float *dist, uint32_t n, float h, uint32_t n_iters, cudaStream_t st) {
  const uint64_t N = uint64_t(n) * n * n;
  if (N == 0) return cudaSuccess;
  float *b[2] = {nullptr, nullptr};
  uint8_t *frozen = nullptr;
  cudaError_t e = cudaMallocAsync(&b[0], N * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&b[1], N * 4, st);
  if (e == cudaSuccess) e = cudaMallocAsync(&frozen, N, st);
  const unsigned grid = unsigned((N + 255) / 256);
  if (e == cudaSuccess) {
    dr_redist_init_kernel<<<grid, 256, 0, st>>>(dist, n, b[0], b[1], frozen);
    int cur = 0;
    for (uint32_t it = 0; it < n_iters; it++) {
      dr_redist_step_kernel<<<grid, 256, 0, st>>>(b[1 - cur], b[cur], frozen, n, h);
      cur = 1 - cur;
    }
    e = cudaMemcpyAsync(dist, b[1 - cur], N * 4, cudaMemcpyDeviceToDevice, st);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  for (float *p : b)
    if (p) cudaFreeAsync(p, st);
  if (frozen) cudaFreeAsync(frozen, st);
  return e;
}

void launch_adam(float *x, float *V, float *S, const float *g, uint32_t n, float batch, float lr, float b1, float b2,
                 float eps, double c1, double c2, cudaStream_t st) {
  dr_adam_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(x, V, S, g, n, batch, lr, b1, b2,
                                                                                  eps, c1, c2);
}

void launch_scale(float *g, uint32_t n, float s, cudaStream_t st) {
  dr_scale_kernel<<<(n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096, 256, 0, st>>>(g, n, s);
}

}  // namespace drk
}  // namespace lrt
