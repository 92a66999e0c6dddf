/*
 * Differentiable-render per-ray core of the CPU oracle — TEST INFRASTRUCTURE ONLY.
 *
 * Restates diff_render/BVH2DR.cpp (dr::BVHDR) for the indexed SBS layouts
 * (SDF_SBS_NODE_LAYOUT_ID32F_IRGB32F and _IN) with the NEWTON finder, which
 * MultiRendererDR::OptimizeFixedStructure forces
 * (diff_render/MultiRendererDR.cpp:324-326).  This file is included twice by
 * lrt_oracle_dr.c: with R = float (the oracle proper, bit-exact against the
 * reference compiled in place) and with R = double (a double-precision forward
 * used only for central finite-difference checks of the gradient).  SFX(name)
 * gives each instantiation its own names.  In the double instantiation the
 * Newton solve runs to a tighter tolerance so that finite differences of the
 * hit distance see the root, not the stopping rule.
 *
 * Required macros: R, SFX(n), RSQRT(x), RABS(x), RFLOOR(x), NEWTON_EPS, NEWTON_ITERS.
 */

typedef struct { R x, y, z; } SFX(v3);
typedef struct { SFX(v3) row[3]; } SFX(m3);
typedef struct { R x, y; } SFX(v2);
#define V3 SFX(v3)
#define M3 SFX(m3)
#define V2 SFX(v2)

static inline V3 SFX(mk)(R x, R y, R z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline V3 SFX(add)(V3 a, V3 b) { return SFX(mk)(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 SFX(sub)(V3 a, V3 b) { return SFX(mk)(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 SFX(mul)(V3 a, V3 b) { return SFX(mk)(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 SFX(scl)(R s, V3 a) { return SFX(mk)(s * a.x, s * a.y, s * a.z); }     /* s * v */
static inline V3 SFX(muls)(V3 a, R s) { return SFX(mk)(a.x * s, a.y * s, a.z * s); }    /* v * s */
static inline V3 SFX(divs)(V3 a, R s) { return SFX(mk)(a.x / s, a.y / s, a.z / s); }    /* v / s */
static inline R SFX(dot)(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline R SFX(len)(V3 a) { return RSQRT(SFX(dot)(a, a)); }
static inline V3 SFX(nrm)(V3 a) { return SFX(divs)(a, SFX(len)(a)); }                 /* LiteMath normalize */
static inline R SFX(mn)(R a, R b) { return (b < a) ? b : a; }                          /* std::min */
static inline R SFX(mx)(R a, R b) { return (a < b) ? b : a; }                          /* std::max */
static inline R SFX(sgn)(R a) { return a < 0 ? (R)-1 : (R)1; }                         /* LiteMath sign */
static inline R SFX(clampr)(R u, R a, R b) { return SFX(mn)(SFX(mx)(a, u), b); }
static inline V3 SFX(mv)(M3 m, V3 v) {                                                 /* float3x3 * float3 */
  return SFX(mk)(SFX(dot)(m.row[0], v), SFX(dot)(m.row[1], v), SFX(dot)(m.row[2], v));
}
static inline M3 SFX(rows)(V3 a, V3 b, V3 c) { M3 m; m.row[0] = a; m.row[1] = b; m.row[2] = c; return m; }
static inline M3 SFX(cols)(V3 a, V3 b, V3 c) {
  return SFX(rows)(SFX(mk)(a.x, b.x, c.x), SFX(mk)(a.y, b.y, c.y), SFX(mk)(a.z, b.z, c.z));
}

static inline V3 SFX(safe_inv)(V3 d) {                       /* SafeInverse, raytrace_common.h:59-67 */
  const R ooeps = (R)1.0e-36f;
  return SFX(mk)((R)1 / (RABS(d.x) > ooeps ? d.x : RABS(ooeps) * SFX(sgn)(d.x)),
                 (R)1 / (RABS(d.y) > ooeps ? d.y : RABS(ooeps) * SFX(sgn)(d.y)),
                 (R)1 / (RABS(d.z) > ooeps ? d.z : RABS(ooeps) * SFX(sgn)(d.z)));
}
static inline V2 SFX(box)(V3 o, V3 inv, V3 bmin, V3 bmax) {  /* RayBoxIntersection2, raytrace_common.h:69-82 */
  const R lo = inv.x * (bmin.x - o.x), hi = inv.x * (bmax.x - o.x);
  const R lo1 = inv.y * (bmin.y - o.y), hi1 = inv.y * (bmax.y - o.y);
  const R lo2 = inv.z * (bmin.z - o.z), hi2 = inv.z * (bmax.z - o.z);
  const R tmin = SFX(mx)(SFX(mn)(lo, hi), SFX(mn)(lo1, hi1));
  const R tmax = SFX(mn)(SFX(mx)(lo, hi), SFX(mx)(lo1, hi1));
  V2 r; r.x = SFX(mx)(tmin, SFX(mn)(lo2, hi2)); r.y = SFX(mn)(tmax, SFX(mx)(lo2, hi2));
  return r;
}

/* ---- trilinear helpers, diff_render/BVH2DR.cpp:200-612 and BVH/BVH2Common.cpp:62-72 ---- */
static inline R SFX(tri)(const R v[8], V3 dp) {
  return (1 - dp.x) * (1 - dp.y) * (1 - dp.z) * v[0] + (1 - dp.x) * (1 - dp.y) * (dp.z) * v[1] +
         (1 - dp.x) * (dp.y) * (1 - dp.z) * v[2] + (1 - dp.x) * (dp.y) * (dp.z) * v[3] +
         (dp.x) * (1 - dp.y) * (1 - dp.z) * v[4] + (dp.x) * (1 - dp.y) * (dp.z) * v[5] +
         (dp.x) * (dp.y) * (1 - dp.z) * v[6] + (dp.x) * (dp.y) * (dp.z) * v[7];
}
/* eval_dist_trilinear_diff (:200-229); a + -(b) == a - b exactly in IEEE arithmetic */
static V3 SFX(tri_diff)(const R v[8], V3 dp) {
  R dx = -(1 - dp.y) * (1 - dp.z) * v[0] - (1 - dp.y) * (dp.z) * v[1] - (dp.y) * (1 - dp.z) * v[2] -
         (dp.y) * (dp.z) * v[3] + (1 - dp.y) * (1 - dp.z) * v[4] + (1 - dp.y) * (dp.z) * v[5] +
         (dp.y) * (1 - dp.z) * v[6] + (dp.y) * (dp.z) * v[7];
  R dy = -(1 - dp.x) * (1 - dp.z) * v[0] - (1 - dp.x) * (dp.z) * v[1] + (1 - dp.x) * (1 - dp.z) * v[2] +
         (1 - dp.x) * (dp.z) * v[3] - (dp.x) * (1 - dp.z) * v[4] - (dp.x) * (dp.z) * v[5] +
         (dp.x) * (1 - dp.z) * v[6] + (dp.x) * (dp.z) * v[7];
  R dz = -(1 - dp.x) * (1 - dp.y) * v[0] + (1 - dp.x) * (1 - dp.y) * v[1] - (1 - dp.x) * (dp.y) * v[2] +
         (1 - dp.x) * (dp.y) * v[3] - (dp.x) * (1 - dp.y) * v[4] + (dp.x) * (1 - dp.y) * v[5] -
         (dp.x) * (dp.y) * v[6] + (dp.x) * (dp.y) * v[7];
  return SFX(mk)(dx, dy, dz);
}
/* eval_dist_trilinear_d_dtheta (:231-241) */
static void SFX(tri_dtheta)(R o[8], V3 dp) {
  o[0] = (1 - dp.x) * (1 - dp.y) * (1 - dp.z); o[1] = (1 - dp.x) * (1 - dp.y) * (dp.z);
  o[2] = (1 - dp.x) * (dp.y) * (1 - dp.z);     o[3] = (1 - dp.x) * (dp.y) * (dp.z);
  o[4] = (dp.x) * (1 - dp.y) * (1 - dp.z);     o[5] = (dp.x) * (1 - dp.y) * (dp.z);
  o[6] = (dp.x) * (dp.y) * (1 - dp.z);         o[7] = (dp.x) * (dp.y) * (dp.z);
}
/* eval_color_trilinear (:243-253): weights times float3 corners, summed per component */
static V3 SFX(tri3)(const V3 c[8], V3 dp) {
  R w[8];
  SFX(tri_dtheta)(w, dp);
  V3 r = SFX(scl)(w[0], c[0]);
  for (int i = 1; i < 8; i++) r = SFX(add)(r, SFX(scl)(w[i], c[i]));
  return r;
}
/* eval_color_trilinear_ddp (:255-331): columns d/ddp.x, d/ddp.y, d/ddp.z */
static M3 SFX(tri3_ddp)(const V3 c[8], V3 dp) {
  const R wx[8] = {-(1 - dp.y) * (1 - dp.z), -(1 - dp.y) * (dp.z), -(dp.y) * (1 - dp.z), -(dp.y) * (dp.z),
                   (1 - dp.y) * (1 - dp.z), (1 - dp.y) * (dp.z), (dp.y) * (1 - dp.z), (dp.y) * (dp.z)};
  const R wy[8] = {-(1 - dp.x) * (1 - dp.z), -(1 - dp.x) * (dp.z), (1 - dp.x) * (1 - dp.z), (1 - dp.x) * (dp.z),
                   -(dp.x) * (1 - dp.z), -(dp.x) * (dp.z), (dp.x) * (1 - dp.z), (dp.x) * (dp.z)};
  const R wz[8] = {-(1 - dp.x) * (1 - dp.y), (1 - dp.x) * (1 - dp.y), -(1 - dp.x) * (dp.y), (1 - dp.x) * (dp.y),
                   -(dp.x) * (1 - dp.y), (dp.x) * (1 - dp.y), -(dp.x) * (dp.y), (dp.x) * (dp.y)};
  V3 cx = SFX(scl)(wx[0], c[0]), cy = SFX(scl)(wy[0], c[0]), cz = SFX(scl)(wz[0], c[0]);
  for (int i = 1; i < 8; i++) {
    cx = SFX(add)(cx, SFX(scl)(wx[i], c[i]));
    cy = SFX(add)(cy, SFX(scl)(wy[i], c[i]));
    cz = SFX(add)(cz, SFX(scl)(wz[i], c[i]));
  }
  return SFX(cols)(cx, cy, cz);
}
/* normalize_diff (:333-392): rows d(n_x)/dv, d(n_y)/dv, d(n_z)/dv; b is formed in double as
 * the reference's 1.0/(a*sqrt(a)) is */
static M3 SFX(nrm_diff)(V3 v) {
  R a = SFX(dot)(v, v);
  R b = (R)(1.0 / ((double)a * sqrt((double)a)));
  V3 dx = SFX(scl)(b, SFX(mk)(v.y * v.y + v.z * v.z, -v.x * v.y, -v.x * v.z));
  V3 dy = SFX(scl)(b, SFX(mk)(-v.x * v.y, v.x * v.x + v.z * v.z, -v.y * v.z));
  V3 dz = SFX(scl)(b, SFX(mk)(-v.x * v.z, -v.y * v.z, v.x * v.x + v.y * v.y));
  return SFX(rows)(dx, dy, dz);
}
/* eval_dist_trilinear_ddp_ddp (:394-523) */
static M3 SFX(tri_ddp_ddp)(const R v[8], V3 dp) {
  R dxdy = (1 - dp.z) * v[0] + (dp.z) * v[1] - (1 - dp.z) * v[2] - (dp.z) * v[3] - (1 - dp.z) * v[4] -
           (dp.z) * v[5] + (1 - dp.z) * v[6] + (dp.z) * v[7];
  R dxdz = (1 - dp.y) * v[0] - (1 - dp.y) * v[1] + (dp.y) * v[2] - (dp.y) * v[3] - (1 - dp.y) * v[4] +
           (1 - dp.y) * v[5] - (dp.y) * v[6] + (dp.y) * v[7];
  R dydz = (1 - dp.x) * v[0] - (1 - dp.x) * v[1] - (1 - dp.x) * v[2] + (1 - dp.x) * v[3] + (dp.x) * v[4] -
           (dp.x) * v[5] - (dp.x) * v[6] + (dp.x) * v[7];
  return SFX(rows)(SFX(mk)(0, dxdy, dxdz), SFX(mk)(dxdy, 0, dydz), SFX(mk)(dxdz, dydz, 0));
}
/* eval_dist_trilinear_ddp_dvalues (:525-601): 3x8, row-major */
static void SFX(tri_ddp_dvalues)(V3 dp, R o[24]) {
  o[0] = -(1 - dp.y) * (1 - dp.z); o[1] = -(1 - dp.y) * (dp.z); o[2] = -(dp.y) * (1 - dp.z); o[3] = -(dp.y) * (dp.z);
  o[4] = (1 - dp.y) * (1 - dp.z);  o[5] = (1 - dp.y) * (dp.z);  o[6] = (dp.y) * (1 - dp.z);  o[7] = (dp.y) * (dp.z);
  o[8] = -(1 - dp.x) * (1 - dp.z); o[9] = -(1 - dp.x) * (dp.z); o[10] = (1 - dp.x) * (1 - dp.z); o[11] = (1 - dp.x) * (dp.z);
  o[12] = -(dp.x) * (1 - dp.z);    o[13] = -(dp.x) * (dp.z);    o[14] = (dp.x) * (1 - dp.z);     o[15] = (dp.x) * (dp.z);
  o[16] = -(1 - dp.x) * (1 - dp.y); o[17] = (1 - dp.x) * (1 - dp.y); o[18] = -(1 - dp.x) * (dp.y); o[19] = (1 - dp.x) * (dp.y);
  o[20] = -(dp.x) * (1 - dp.y);     o[21] = (dp.x) * (1 - dp.y);     o[22] = -(dp.x) * (dp.y);     o[23] = (dp.x) * (dp.y);
}
/* step (:603-608) and dp_to_nmq (:1108-1115) */
static inline R SFX(step01)(R e0, R e1, R x) { return SFX(clampr)((x - e0) / (e1 - e0), (R)0.0, (R)1.0); }
static V3 SFX(dp_to_nmq)(V3 dp, R beta) {
  return SFX(mk)(dp.x < (R)0.5f ? SFX(step01)(-beta, beta, dp.x) : SFX(step01)(-beta, beta, dp.x - (R)1.0f),
                 dp.y < (R)0.5f ? SFX(step01)(-beta, beta, dp.y) : SFX(step01)(-beta, beta, dp.y - (R)1.0f),
                 dp.z < (R)0.5f ? SFX(step01)(-beta, beta, dp.z) : SFX(step01)(-beta, beta, dp.z - (R)1.0f));
}

/* ---- CRT_HitDR / RayDiffPayload, diff_render/DR_common.h:47-72 ---- */
typedef struct {
  R t; uint32_t primId, instId, geomId; V3 color; R sdf; V3 normal; uint32_t check_vox_border;
} SFX(hitdr);
typedef struct {
  SFX(hitdr) missed_hit, missed_hit_candidate;
  uint32_t missed_indices[8]; R missed_dSDF_dtheta[8];
  uint32_t dc_index[8]; R dc_value[8];                       /* dDiffuse_dSc */
  V3 dd_diffuse[64]; uint32_t dd_index[64]; V3 dd_norm[64]; R dd_dist[64];   /* dDiffuseNormal_dSd */
} SFX(payload);

typedef struct {
  const orc_dr_scene *s;
  const R *P;                /* values_f, the parameters */
} SFX(ctx);

/* BVHDR::Intersect, NEWTON branch with the border-relaxation bookkeeping
 * (diff_render/BVH2DR.cpp:623-1073).  Returns t (voxel units) on a hit, else qFar + EPS. */
static R SFX(intersect)(uint32_t flags, V3 ray_dir, const R values[8], R d, R qNear, R qFar, V3 start_q,
                        SFX(payload) *pl) {
  const R EPS = (R)1e-6f, SDF_EPS = (R)NEWTON_EPS;
  R d_inv = (R)1.0f / d;
  R t = qNear;
  int hit = 0;
  if (pl) pl->missed_hit_candidate.sdf = (R)1000.f;
  R start_dist = SFX(tri)(values, SFX(add)(start_q, SFX(scl)(t, ray_dir)));
  if (start_dist <= SDF_EPS) {
    hit = 1;
  } else {
    R s000 = values[0] * d_inv, s001 = values[1] * d_inv, s010 = values[2] * d_inv, s011 = values[3] * d_inv;
    R s100 = values[4] * d_inv, s101 = values[5] * d_inv, s110 = values[6] * d_inv, s111 = values[7] * d_inv;
    R a = s101 - s001;
    R k0 = s000, k1 = s100 - s000, k2 = s010 - s000, k3 = s110 - s010 - k1, k4 = k0 - s001, k5 = k1 - a;
    R k6 = k2 - (s011 - s001), k7 = k3 - (s111 - s011 - a);
    V3 o = start_q, d3 = ray_dir;
    R m0 = o.x * o.y, m1 = d3.x * d3.y, m2 = o.x * d3.y + o.y * d3.x;
    R m3 = k5 * o.z - k1, m4 = k6 * o.z - k2, m5 = k7 * o.z - k3;
    R c0 = (k4 * o.z - k0) + o.x * m3 + o.y * m4 + m0 * m5;
    R c1 = d3.x * m3 + d3.y * m4 + m2 * m5 + d3.z * (k4 + k5 * o.x + k6 * o.y + k7 * m0);
    R c2 = m1 * m5 + d3.z * (k5 * d3.x + k6 * d3.y + k7 * m2);
    R c3 = k7 * m1 * d3.z;
    R aa = 3 * c3, b = 2 * c2, c = c1;
    R t0 = 0, t1 = qFar, t2 = qFar, t3 = qFar;
    R D = b * b - 4 * aa * c;
    if (D >= 0) {
      R q = (R)-0.5f * (b + SFX(sgn)(b) * RSQRT(D));
      t1 = RABS(aa) > EPS ? q / aa : t0;
      t2 = RABS(q) > EPS ? c / q : qFar;
      R tmp = SFX(mn)(t1, t2);
      t2 = SFX(mx)(t1, t2);
      t1 = tmp;
      t1 = SFX(clampr)(t1, t0, t3);
      t2 = SFX(clampr)(t2, t0, t3);
    }
    R sdf0 = c0;
    R sdf1 = (c0 + t1 * (c1 + t1 * (c2 + t1 * c3)));
    R sdf2 = (c0 + t2 * (c1 + t2 * (c2 + t2 * c3)));
    R sdf3 = (c0 + t3 * (c1 + t3 * (c2 + t3 * c3)));
    int s0 = sdf0 > 0, s1 = sdf1 > 0, s2 = sdf2 > 0, s3 = sdf3 > 0;
    R nwt_min = t0, nwt_max = t0;
    if (s0 != s1) { nwt_min = t0; nwt_max = t1; }
    else if (s1 != s2) { nwt_min = t1; nwt_max = t2; }
    else if (s2 != s3) { nwt_min = t2; nwt_max = t3; }
    if (nwt_min < nwt_max) {
      unsigned it = 0;
      R rtn = (R)0.5f * (nwt_min + nwt_max);
      R f = 1000;
      while (it < NEWTON_ITERS && RABS(f) >= SDF_EPS) {
        f = c0 + rtn * (c1 + rtn * (c2 + rtn * c3));
        R df = c1 + rtn * (2 * c2 + rtn * 3 * c3);
        R dx = f / (df + SFX(sgn)(df) * (R)1e-9f);
        rtn -= dx;
        it++;
      }
      t = rtn;
      hit = (t >= 0 && t <= qFar && RABS(f) < SDF_EPS);
    } else {
      hit = 0;
    }
    if (pl && (flags & ORC_DR_RAY_FLAG_BORDER)) {
      R t_min = qFar + EPS;
      if (RABS(aa) > EPS) {
        R root1 = (R)-0.5f * (b + RSQRT(D)) / aa, root2 = (R)-0.5f * (b - RSQRT(D)) / aa;
        t_min = (SFX(sgn)(aa) > 0) == (root1 < root2) ? root1 : root2;
      } else if (b < -EPS) {
        t_min = -c / b;
      }
      R sdf_min = (c0 + t_min * (c1 + t_min * (c2 + t_min * c3)));
      if (pl->missed_hit.check_vox_border == 1) {
        if (c1 <= 0) {
          if (sdf0 < (R)0.f && -sdf0 * d < pl->missed_hit.sdf) { pl->missed_hit.t = t0; pl->missed_hit.sdf = -sdf0 * d; }
        }
        pl->missed_hit.check_vox_border = 0;
      }
      if (t_min >= 0 && t_min <= qFar && sdf_min < (R)0.f && -sdf_min * d < pl->missed_hit.sdf) {
        pl->missed_hit.t = t_min;
        pl->missed_hit.sdf = -sdf_min * d;
      }
      if (sdf3 < (R)0.f && -sdf3 * d < pl->missed_hit.sdf && (c1 + qFar * (2 * c2 + qFar * 3 * c3)) >= (R)0.f) {
        pl->missed_hit.check_vox_border = 1;
        pl->missed_hit_candidate.t = qFar;
        pl->missed_hit_candidate.sdf = -sdf3 * d;
      }
    }
  }
  return hit ? t : qFar + EPS;
}

/* dIntersect_dValues (:1075-1090): central differences with delta 1e-3 on the
 * caller's values array, which keeps the rounding residue of +d, -2d, +d. */
static void SFX(dintersect)(uint32_t flags, V3 ray_dir, R values[8], R d, R qNear, R qFar, V3 start_q, R out[8]) {
  const R delta = (R)0.001f;
  for (int i = 0; i < 8; i++) {
    values[i] += delta;
    R d1 = SFX(intersect)(flags, ray_dir, values, d, qNear, qFar, start_q, 0);
    values[i] -= 2 * delta;
    R d2 = SFX(intersect)(flags, ray_dir, values, d, qNear, qFar, start_q, 0);
    values[i] += delta;
    out[i] = (d1 - d2) / (2 * delta);
  }
}

static inline uint32_t SFX(vid)(uint32_t x, uint32_t y, uint32_t z, uint32_t v) { return x * v * v + y * v + z; }

/* load_distance_values_with_indices (:1092-1106) */
static void SFX(load_vals)(const SFX(ctx) *cx, uint32_t node, V3 vox, uint32_t v_size, R values[8], uint32_t idx[8]) {
  const orc_dr_scene *s = cx->s;
  uint32_t v_off = s->nodes[node].data_offset;
  for (int i = 0; i < 8; i++) {
    uint32_t vId = SFX(vid)((uint32_t)vox.x + ((i & 4) >> 2), (uint32_t)vox.y + ((i & 2) >> 1), (uint32_t)vox.z + (i & 1), v_size);
    idx[i] = s->values[v_off + vId];
    values[i] = cx->P[idx[i]];
  }
}

static void SFX(colors)(const SFX(ctx) *cx, uint32_t t_off, V3 c[8]) {
  for (int i = 0; i < 8; i++) {
    uint32_t j = cx->s->values[t_off + i];
    c[i] = SFX(mk)(cx->P[j + 0], cx->P[j + 1], cx->P[j + 2]);
  }
}

/* OctreeBrickIntersectWithGrad (:1130-1610) */
static void SFX(brick_grad)(const SFX(ctx) *cx, uint32_t type, uint32_t flags, V3 ray_pos, V3 ray_dir, R tNear,
                            uint32_t instId, uint32_t geomId, uint32_t bvhNodeId, SFX(payload) *pl, SFX(hitdr) *hit) {
  const orc_dr_scene *s = cx->s;
  const orc_sbs_header *h = &s->hdr;
  const int layout_in = (h->aux_data & 0xFF000000u) == ORC_SBS_LAYOUT_ID32F_IRGB32F_IN;
  R values[8];
  uint32_t primId = bvhNodeId, nodeId = primId;
  uint32_t v_size = h->brick_size + 2 * h->brick_pad + 1;
  const orc_sbs_node *nd = &s->nodes[nodeId];
  R px = (R)(float)(nd->pos_xy >> 16), py = (R)(float)(nd->pos_xy & 0x0000FFFF);
  R pz = (R)(float)(nd->pos_z_lod_size >> 16), sz = (R)(float)(nd->pos_z_lod_size & 0x0000FFFF);
  R sz_inv = (R)2.0f / sz;
  R bs = (R)(float)h->brick_size;
  R d = (R)2.0f / (sz * bs);
  V3 bmin = SFX(add)(SFX(mk)(-1, -1, -1), SFX(scl)(sz_inv, SFX(mk)(px, py, pz)));
  V3 bmax = SFX(add)(bmin, SFX(scl)(sz_inv, SFX(mk)(1, 1, 1)));
  V2 bnf = SFX(box)(ray_pos, SFX(safe_inv)(ray_dir), bmin, bmax);
  R old_t = hit->t;
  const R scale = (R)0.5f * sz * bs;
  /* bounded voxel walk: the reference's loop has no bound; orc_walk_step_bound
   * covers every walk it finishes (see brick_intersect in lrt_oracle.c) */
  const uint32_t max_steps = orc_walk_step_bound(h->brick_size, (float)(bnf.y - bnf.x));
  for (uint32_t step = 0; bnf.x < bnf.y && hit->t == old_t && step < max_steps; step++) {
    V3 hit_pos = SFX(add)(ray_pos, SFX(scl)(bnf.x, ray_dir));
    V3 local_pos = SFX(muls)(SFX(sub)(hit_pos, bmin), scale);
    V3 vox = SFX(mk)(RFLOOR(SFX(clampr)(local_pos.x, (R)1e-6f, bs - (R)1e-6f)),
                     RFLOOR(SFX(clampr)(local_pos.y, (R)1e-6f, bs - (R)1e-6f)),
                     RFLOOR(SFX(clampr)(local_pos.z, (R)1e-6f, bs - (R)1e-6f)));
    V3 min_pos = SFX(add)(bmin, SFX(scl)(d, vox));
    V3 max_pos = SFX(add)(min_pos, SFX(scl)(d, SFX(mk)(1, 1, 1)));
    uint32_t mi[8];
    SFX(load_vals)(cx, nodeId, vox, v_size, values, mi);
    V2 fnf = SFX(box)(ray_pos, SFX(safe_inv)(ray_dir), min_pos, max_pos);
    if (tNear < fnf.x) {
      V3 start_pos = SFX(add)(ray_pos, SFX(scl)(fnf.x, ray_dir));
      V3 start_q = SFX(muls)(SFX(sub)(start_pos, min_pos), scale);
      R qFar = (fnf.y - fnf.x) * scale;
      R prev_sdf = pl->missed_hit.sdf;
      R t = SFX(intersect)(flags, ray_dir, values, d, 0, qFar, start_q, pl);
      R tReal = fnf.x + d * t;
      if (flags & ORC_DR_RAY_FLAG_BORDER) {
        if (pl->missed_hit.sdf < prev_sdf && pl->missed_hit.t < t) {
          R missed_t = pl->missed_hit.t;
          pl->missed_hit.t = fnf.x + d * pl->missed_hit.t;
          V3 q_ast = SFX(add)(start_q, SFX(scl)(missed_t, ray_dir));
          V3 y_ast = SFX(add)(ray_pos, SFX(scl)(fnf.x + (d * missed_t), ray_dir));
          V3 dp_ast = SFX(muls)(SFX(sub)(y_ast, bmin), (R)0.5f * sz);
          V3 g = SFX(muls)(SFX(tri_diff)(values, q_ast), (R)1 / d);
          V3 mult = SFX(mk)(RABS(q_ast.x - (R)0.5f) > (R)0.5f - (R)1e-5f ? 0 : 1,
                            RABS(q_ast.y - (R)0.5f) > (R)0.5f - (R)1e-5f ? 0 : 1,
                            RABS(q_ast.z - (R)0.5f) > (R)0.5f - (R)1e-5f ? 0 : 1);
          g = SFX(mul)(g, mult);
          R glen = SFX(len)(g);
          if (glen > (R)1e-9f) {
            R dv[8];
            SFX(tri_dtheta)(dv, q_ast);
            for (int i = 0; i < 8; i++) pl->missed_dSDF_dtheta[i] = -dv[i] / glen;
            V3 cols[8];
            SFX(colors)(cx, nd->data_offset + v_size * v_size * v_size, cols);
            pl->missed_hit.color = SFX(tri3)(cols, dp_ast);
            pl->missed_hit.normal = SFX(divs)(g, glen);
            for (int i = 0; i < 8; i++) pl->missed_indices[i] = mi[i];
          }
        }
      }
      if (t <= qFar && tReal < hit->t) {
        hit->t = tReal;
        hit->primId = primId;
        hit->instId = instId;
        hit->geomId = geomId | (type << 24);
        unsigned off = 0;
        if (layout_in) {
          V3 p0 = SFX(add)(start_q, SFX(scl)(t, ray_dir));
          off += p0.x < (R)0.5f ? 4 : 0;
          off += p0.y < (R)0.5f ? 2 : 0;
          off += p0.z < (R)0.5f ? 1 : 0;
          off *= 8;
        }
        R dt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (flags & (ORC_DR_RAY_FLAG_DDIFFUSE_DPOS | ORC_DR_RAY_FLAG_DNORM_DPOS | ORC_DR_RAY_FLAG_DDIST_DPOS)) {
          SFX(dintersect)(flags, ray_dir, values, d, 0, qFar, start_q, dt);
          for (int i = 0; i < 8; i++) {
            pl->dd_index[off + i] = mi[i];
            pl->dd_dist[off + i] = d * dt[i];
          }
        }
        if (s->need_normal) {
          if (layout_in) {
            const R beta = (R)0.5f;
            V3 dp = SFX(add)(start_q, SFX(scl)(t, ray_dir));
            V3 normals[8];
            R vn[8], dD1[24], dtri[8];
            uint32_t in_[8];
            V3 nmq = SFX(dp_to_nmq)(dp, beta);
            uint32_t k = off / 8;
            for (int i = 0; i < 8; i++) normals[i] = SFX(mk)(0, 0, 0);
            if (flags & ORC_DR_RAY_FLAG_DNORM_DPOS) SFX(tri_dtheta)(dtri, nmq);
            int vp0x = (int)(dp.x < (R)0.5f ? vox.x - 1 : vox.x);
            int vp0y = (int)(dp.y < (R)0.5f ? vox.y - 1 : vox.y);
            int vp0z = (int)(dp.z < (R)0.5f ? vox.z - 1 : vox.z);
            const int ibs = (int)h->brick_size;
            for (int i = 0; i < 8; i++) {
              int vx = vp0x + ((i & 4) >> 2), vy = vp0y + ((i & 2) >> 1), vz = vp0z + (i & 1);
              int bx = vx >= 0 ? (vx < ibs ? 0 : 1) : -1;
              int by = vy >= 0 ? (vy < ibs ? 0 : 1) : -1;
              int bz = vz >= 0 ? (vz < ibs ? 0 : 1) : -1;
              uint32_t nid = 9 * (bx + 1) + 3 * (by + 1) + (bz + 1);
              V3 dvox = SFX(sub)(SFX(mk)((R)(float)vx, (R)(float)vy, (R)(float)vz), vox);
              uint32_t nnode;
              V3 nvox;
              if (nid == 13) {
                nnode = nodeId;
                nvox = SFX(mk)((R)(float)vx, (R)(float)vy, (R)(float)vz);
              } else {
                nnode = s->values[nd->data_offset + v_size * v_size * v_size + 8 + nid];
                nvox = SFX(sub)(SFX(mk)((R)(float)vx, (R)(float)vy, (R)(float)vz),
                                SFX(scl)(bs, SFX(mk)((R)(float)bx, (R)(float)by, (R)(float)bz)));
              }
              if (nnode != ORC_INVALID_IDX) {
                SFX(load_vals)(cx, nnode, nvox, v_size, vn, in_);
                V3 ndp = SFX(sub)(dp, dvox);
                V3 g = SFX(tri_diff)(vn, ndp);
                normals[i] = SFX(nrm)(g);
                if (flags & ORC_DR_RAY_FLAG_DNORM_DPOS) {
                  for (int j = 0; j < 8; j++) pl->dd_index[8 * i + j] = in_[j];
                  M3 Mi = SFX(nrm_diff)(g);
                  SFX(tri_ddp_dvalues)(ndp, dD1);
                  M3 D2 = SFX(tri_ddp_ddp)(vn, ndp);
                  for (int j = 0; j < 8; j++) {
                    V3 v = SFX(mk)(dD1[j], dD1[8 + j], dD1[16 + j]);
                    pl->dd_norm[8 * i + j] = SFX(add)(pl->dd_norm[8 * i + j], SFX(scl)(dtri[i], SFX(mv)(Mi, v)));
                  }
                  V3 t1 = SFX(mv)(D2, ray_dir);
                  for (int j = 0; j < 8; j++) {
                    V3 v = SFX(mk)(t1.x * dt[j], t1.y * dt[j], t1.z * dt[j]);
                    pl->dd_norm[8 * k + j] = SFX(add)(pl->dd_norm[8 * k + j], SFX(scl)(dtri[i], SFX(mv)(Mi, v)));
                  }
                }
              }
            }
            V3 tr3 = SFX(tri3)(normals, nmq);
            hit->normal = SFX(nrm)(tr3);
            if (flags & ORC_DR_RAY_FLAG_DNORM_DPOS) {
              M3 Mf = SFX(nrm_diff)(tr3);
              M3 dT = SFX(tri3_ddp)(normals, nmq);
              const V3 dnmq = SFX(mk)(1, 1, 1);
              for (int j = 0; j < 8; j++) {
                V3 ddp = SFX(muls)(ray_dir, dt[j]);
                pl->dd_norm[8 * k + j] = SFX(add)(pl->dd_norm[8 * k + j], SFX(mv)(dT, SFX(mul)(dnmq, ddp)));
              }
              for (int i = 0; i < 8; i++)
                if (SFX(len)(normals[i]) > 0.5)
                  for (int j = 0; j < 8; j++) pl->dd_norm[8 * i + j] = SFX(mv)(Mf, pl->dd_norm[8 * i + j]);
            }
          } else {
            V3 p0 = SFX(add)(start_q, SFX(scl)(t, ray_dir));
            V3 g = SFX(tri_diff)(values, p0);
            hit->normal = SFX(nrm)(g);
            if (flags & ORC_DR_RAY_FLAG_DNORM_DPOS) {
              M3 M = SFX(nrm_diff)(g);
              R dD1[24];
              SFX(tri_ddp_dvalues)(p0, dD1);
              M3 D2 = SFX(tri_ddp_ddp)(values, p0);
              V3 t1 = SFX(mv)(D2, ray_dir);
              for (int i = 0; i < 8; i++) {
                dD1[i] += t1.x * dt[i];
                dD1[8 + i] += t1.y * dt[i];
                dD1[16 + i] += t1.z * dt[i];
              }
              for (int i = 0; i < 8; i++)
                pl->dd_norm[off + i] = SFX(mv)(M, SFX(mk)(dD1[i], dD1[8 + i], dD1[16 + i]));
            }
          }
        }
        {
          V3 pos = SFX(add)(ray_pos, SFX(scl)(hit->t, ray_dir));
          V3 dp = SFX(muls)(SFX(sub)(pos, bmin), (R)0.5f * sz);
          uint32_t t_off = nd->data_offset + v_size * v_size * v_size;
          V3 cols[8];
          SFX(colors)(cx, t_off, cols);
          hit->color = SFX(tri3)(cols, dp);
          if (flags & ORC_DR_RAY_FLAG_DDIFFUSE_DCOLOR) {
            for (int i = 0; i < 8; i++) {
              V3 q = SFX(mk)((R)((i & 4) >> 2), (R)((i & 2) >> 1), (R)(i & 1));
              V3 one = SFX(mk)(1, 1, 1);
              V3 lq = SFX(add)(SFX(mul)(q, dp), SFX(mul)(SFX(sub)(one, q), SFX(sub)(one, dp)));
              pl->dc_index[i] = s->values[t_off + i];
              pl->dc_value[i] = lq.x * lq.y * lq.z;
            }
          }
          if (flags & ORC_DR_RAY_FLAG_DDIFFUSE_DPOS) {
            M3 dL = SFX(tri3_ddp)(cols, dp);
            for (int i = 0; i < 8; i++) {
              R hs = (R)0.5f * sz;
              pl->dd_diffuse[off + i] = SFX(mv)(dL, SFX(mk)(hs * ray_dir.x * dt[i], hs * ray_dir.y * dt[i], hs * ray_dir.z * dt[i]));
            }
          }
        }
        break;
      }
    }
    bnf.x += SFX(mx)((R)0.0f, fnf.y - bnf.x) + (R)1e-6f;
  }
}

static void SFX(hit_init)(SFX(hitdr) *h, R tfar) {
  h->t = tfar; h->primId = h->instId = h->geomId = 0xFFFFFFFFu;
  h->color = SFX(mk)(0, 0, 0); h->sdf = (R)1000.0f; h->normal = SFX(mk)(1, 0, 0);
  h->check_vox_border = 0;
}

/* BVH2TraverseF32WithGrad (:106-167), stopOnFirstHit forced on; leaf ->
 * IntersectAllPrimitivesInLeafWithGrad (:171-190) with tNearSdf = max(tNear, 0.1) */
static void SFX(traverse)(const SFX(ctx) *cx, uint32_t flags, V3 ray_pos, V3 ray_dir, R tNear, uint32_t instId,
                          uint32_t geomId, SFX(payload) *pl, SFX(hitdr) *hit) {
  const orc_dr_scene *s = cx->s;
  uint32_t stack[ORC_DR_STACK];
  int top = 0;
  uint32_t left = 0;
  const V3 inv = SFX(safe_inv)(ray_dir);
  const R tNearSdf = SFX(mx)(tNear, (R)0.1f);
  while (top >= 0 && !(hit->primId != 0xFFFFFFFFu)) {
    while (top >= 0 && ((left & 0x80000000u) == 0)) {
      const orc_bvh_pair *fp = &s->pairs[left];
      const uint32_t n0 = fp->l.left_offset, n1 = fp->r.left_offset;
      V2 tm0 = SFX(box)(ray_pos, inv, SFX(mk)(fp->l.bmin[0], fp->l.bmin[1], fp->l.bmin[2]),
                        SFX(mk)(fp->l.bmax[0], fp->l.bmax[1], fp->l.bmax[2]));
      V2 tm1 = SFX(box)(ray_pos, inv, SFX(mk)(fp->r.bmin[0], fp->r.bmin[1], fp->r.bmin[2]),
                        SFX(mk)(fp->r.bmax[0], fp->r.bmax[1], fp->r.bmax[2]));
      const int h0 = (tm0.x <= tm0.y) && (tm0.y >= tNear) && (tm0.x <= hit->t);
      const int h1 = (tm1.x <= tm1.y) && (tm1.y >= tNear) && (tm1.x <= hit->t);
      left = h0 ? n0 : n1;
      if (h0 && h1) {
        left = (tm0.x <= tm1.x) ? n0 : n1;
        if (top >= ORC_DR_STACK) { top = -1; break; }   /* the reference's stack[80] would overflow */
        stack[top] = (tm0.x <= tm1.x) ? n1 : n0;
        top++;
      }
      if (!h0 && !h1) {
        top--;
        left = stack[top > 0 ? top : 0];
      }
    }
    if (top >= 0 && left != 0xFFFFFFFFu) {
      const uint32_t start = left & 0x00FFFFFFu;
      SFX(brick_grad)(cx, ORC_TYPE_SDF_SBS_COL, flags, ray_pos, ray_dir, tNearSdf, instId, geomId, start, pl, hit);
    }
    top--;
    left = stack[top > 0 ? top : 0];
  }
}

/* RayQuery_NearestHitWithGrad (:12-102): payload initialisation, the single
 * instance's TLAS leaf box, ray to object space, BLAS traversal, candidate merge. */
static SFX(hitdr) SFX(query)(const SFX(ctx) *cx, uint32_t flags, const float posn[4], const float dirf[4],
                             SFX(payload) *pl) {
  const orc_dr_scene *s = cx->s;
  R tfar = (R)dirf[3];
  if (tfar <= 0) tfar = -tfar;
  V3 P = SFX(mk)(posn[0], posn[1], posn[2]), Dd = SFX(mk)(dirf[0], dirf[1], dirf[2]);
  const V3 inv = SFX(safe_inv)(Dd);
  SFX(hitdr) hit;
  SFX(hit_init)(&hit, tfar);
  SFX(hit_init)(&pl->missed_hit, tfar);
  pl->missed_hit.check_vox_border = 1;
  pl->missed_hit_candidate = pl->missed_hit;
  for (int i = 0; i < 8; i++) {
    pl->missed_indices[i] = 0xFFFFFFFFu; pl->missed_dSDF_dtheta[i] = 0;
    pl->dc_index[i] = 0xFFFFFFFFu; pl->dc_value[i] = 0;
  }
  for (int i = 0; i < 64; i++) {
    pl->dd_index[i] = 0xFFFFFFFFu;
    pl->dd_diffuse[i] = SFX(mk)(0, 0, 0); pl->dd_norm[i] = SFX(mk)(0, 0, 0); pl->dd_dist[i] = 0;
  }
  V2 bh = SFX(box)(P, inv, SFX(mk)(s->inst_bmin[0], s->inst_bmin[1], s->inst_bmin[2]),
                   SFX(mk)(s->inst_bmax[0], s->inst_bmax[1], s->inst_bmax[2]));
  if ((bh.x <= bh.y) && (bh.y > (R)posn[3]) && (bh.x < hit.t)) {
    const float *m = s->inst_inv;
    V3 rp = SFX(mk)(m[0] * P.x + m[1] * P.y + m[2] * P.z + m[3] * (R)1.0f,
                    m[4] * P.x + m[5] * P.y + m[6] * P.z + m[7] * (R)1.0f,
                    m[8] * P.x + m[9] * P.y + m[10] * P.z + m[11] * (R)1.0f);
    V3 rd = SFX(mk)(m[0] * Dd.x + m[1] * Dd.y + m[2] * Dd.z + m[3] * (R)0.0f,
                    m[4] * Dd.x + m[5] * Dd.y + m[6] * Dd.z + m[7] * (R)0.0f,
                    m[8] * Dd.x + m[9] * Dd.y + m[10] * Dd.z + m[11] * (R)0.0f);
    SFX(traverse)(cx, flags, rp, rd, (R)posn[3], 0, 0, pl, &hit);
  }
  if (pl->missed_hit_candidate.sdf < pl->missed_hit.sdf) pl->missed_hit = pl->missed_hit_candidate;
  return hit;
}

#undef V3
#undef M3
#undef V2
