// Learned proposal for the SBS leaf phase.
//
// A per-(ray, brick) MLP (mlp.cuh) predicts where along the ray's segment
// through a brick the first zero crossing lies.  The proposal is used as a
// jump: if every voxel of the voxel-index box spanned by the segment's entry
// voxel and the predicted voxel (the predicted voxel excepted) is empty in the
// brick's occupancy mask (no corner <= 0, so the reference's walk would run no
// finder there), and the walk's first voxel at the predicted voxel's entry (which
// rounding may put next to it) is the predicted voxel or one of those empty
// voxels, the walk starts at the predicted voxel's entry instead of the
// brick's; from there on it is the reference walk with the reference finder
// (BVH/BVH2Common.cpp:764-984, 437-522), which refines the crossing exactly.
// Otherwise the plain walk runs from the brick entry.  Hits therefore equal the
// plain kernel's bit for bit; the network only decides how much of the walk is
// skipped.
//
// Kernels: triple generation from the plain finder's hits, one training step
// (forward + backward on the tensor cores, Adam by the last block), batched
// inference, and the persistent render kernel with the proposal in its leaf
// phase (the warp evaluates the network for all lanes holding a brick at once).
#include "mlp.cuh"
#include "proposal_internal.h"
#include "tc05.cuh"
#include "traverse.cuh"

namespace lrt {
namespace dev {

using namespace lrt::mlp;

// 16 features of a ray segment through a brick: entry and exit in brick units
// [0,1]^3, the brick's 8 corner values and the segment length in brick edges,
// the smallest corner value.  t0, t1: the segment (ray-box of the brick).
__device__ void brick_features(const DevScene &s, uint32_t brick, float3 rp, float3 rd, float3 inv, float f[16],
                               float &t0, float &t1) {
  const lrt_sbs_header &h = s.sbs_hdr;
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
  const float px = float(nd.x >> 16), py = float(nd.x & 0x0000FFFF), pz = float(nd.y >> 16);
  const float sz = float(nd.y & 0x0000FFFF);
  const float sz_inv = 2.0f / sz;
  const float3 bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(px, py, pz)));
  const float3 bmax = add(bmin, scl(sz_inv, f3(1, 1, 1)));
  const float2 bnf = ray_box(rp, inv, bmin.x, bmin.y, bmin.z, bmax.x, bmax.y, bmax.z);
  t0 = bnf.x;
  t1 = bnf.y;
  const float k = 0.5f * sz;   // 1 / brick edge
  const float3 p0 = scr(sub(add(rp, scl(t0, rd)), bmin), k), p1 = scr(sub(add(rp, scl(t1, rd)), bmin), k);
  f[0] = p0.x; f[1] = p0.y; f[2] = p0.z; f[3] = p1.x; f[4] = p1.y; f[5] = p1.z;
  const GlobalLoader gl(s, nd.z, sz_inv);
  const uint32_t bs = h.brick_size, pad = h.brick_pad, v = bs + 2 * pad + 1;
  float cmin = 3.0e38f;
#pragma unroll
  for (int i = 0; i < 8; i++) {
    const uint32_t vId = (((i & 4) ? bs : 0u) + pad) * v * v + (((i & 2) ? bs : 0u) + pad) * v + (((i & 1) ? bs : 0u) + pad);
    const float c = decode_dx(gl.data, vId, gl.lg, gl.bits, gl.max_val, gl.d_max, gl.mult) * k;
    f[6 + i] = c;
    cmin = fminf(cmin, c);
  }
  f[14] = (t1 - t0) * k;
  f[15] = cmin;
}

// the voxel the reference walk takes for entry distance t (its floor/clamp)
__device__ __forceinline__ int3 walk_voxel(float3 rp, float3 rd, float t, float3 bmin, float scale, float bs) {
  const float3 lp = scr(sub(add(rp, scl(t, rd)), bmin), scale);
  return make_int3(int(floorf(fmn(fmx(lp.x, 1e-6f), bs - 1e-6f))), int(floorf(fmn(fmx(lp.y, 1e-6f), bs - 1e-6f))),
                   int(floorf(fmn(fmx(lp.z, 1e-6f), bs - 1e-6f))));
}

// Where the walk may start given the prediction u (fraction of the segment):
// the predicted voxel's entry distance if every other voxel of the box spanned
// with the entry voxel is empty, else -inf (walk from the brick entry).
__device__ float proposal_start(const DevScene &s, uint32_t brick, float3 rp, float3 rd, float3 inv, float t0,
                                float t1, float u, bool &jumped, uint32_t &skipped) {
  jumped = false;
  skipped = 0;
  const float none = -3.4e38f;
  const uint32_t bsz = s.sbs_hdr.brick_size;
  // z rows of the occupancy mask stay inside one word for power-of-two bricks up to 32
  if (!(u > 0.0f) || !(t1 > t0) || bsz > 32 || (bsz & (bsz - 1)) != 0) return none;
  u = fminf(u, 1.0f);
  const float th = t0 + u * (t1 - t0);
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
  const float sz = float(nd.y & 0x0000FFFF);
  const float sz_inv = 2.0f / sz, bs = float(bsz), d = 2.0f / (sz * bs), scale = 0.5f * sz * bs;
  const float3 bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(float(nd.x >> 16), float(nd.x & 0xFFFF), float(nd.y >> 16))));
  const int3 v0 = walk_voxel(rp, rd, t0, bmin, scale, bs), vh = walk_voxel(rp, rd, th, bmin, scale, bs);
  if (v0.x == vh.x && v0.y == vh.y && v0.z == vh.z) return none;
  const uint32_t *occ = s.occ + size_t(brick) * s.occ_words;
  const int x0 = min(v0.x, vh.x), x1 = max(v0.x, vh.x), y0 = min(v0.y, vh.y), y1 = max(v0.y, vh.y);
  const int z0 = min(v0.z, vh.z), z1 = max(v0.z, vh.z);
  const uint32_t zmask = ((z1 - z0 + 1) >= 32 ? 0xFFFFFFFFu : ((1u << (z1 - z0 + 1)) - 1u)) << z0;
  for (int x = x0; x <= x1; x++)
    for (int y = y0; y <= y1; y++) {
      const uint32_t base = (uint32_t(x) * bsz + uint32_t(y)) * bsz;   // a z row never straddles a word
      uint32_t m = zmask;
      if (x == vh.x && y == vh.y) m &= ~(1u << vh.z);
      if ((__ldg(&occ[base >> 5]) >> (base & 31u)) & m) return none;
    }
  // the predicted voxel's entry: its near planes, as the walk computes them
  const float3 mp = add(bmin, scl(d, f3(float(vh.x), float(vh.y), float(vh.z))));
  const float nx = inv.x * ((inv.x > 0.0f ? mp.x : mp.x + d) - rp.x);
  const float ny = inv.y * ((inv.y > 0.0f ? mp.y : mp.y + d) - rp.y);
  const float nz = inv.z * ((inv.z > 0.0f ? mp.z : mp.z + d) - rp.z);
  const float start = fmx(fmx(nx, ny), nz);
  // the walk's first voxel at that distance, as the walk computes it: on the entry
  // plane, rounding may put it next to the predicted voxel; it must be the predicted
  // voxel or one of the box's (empty) voxels, else no jump
  const int3 w = walk_voxel(rp, rd, fmx(t0, start), bmin, scale, bs);
  const bool w_ok = (w.x == vh.x && w.y == vh.y && w.z == vh.z) ||
                    (w.x >= x0 && w.x <= x1 && w.y >= y0 && w.y <= y1 && w.z >= z0 && w.z <= z1);
  if (!w_ok) return none;
  jumped = true;
  skipped = uint32_t(abs(vh.x - v0.x) + abs(vh.y - v0.y) + abs(vh.z - v0.z));   // voxel faces crossed
  return start;
}

__device__ __forceinline__ uint32_t hash3(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t h = a * 747796405u + 2891336453u;
  h ^= b + 0x9e3779b9u + (h << 6) + (h >> 2);
  h = (h ^ (h >> 16)) * 0x85ebca6bu;
  h ^= c + 0x9e3779b9u + (h << 6) + (h >> 2);
  h = (h ^ (h >> 13)) * 0xc2b2ae35u;
  return h ^ (h >> 16);
}

// ---------------------------------------------------------------- triple generation
// One thread per pixel of the views (regular pixel centres): plain closest-hit
// trace; a hit yields (features of the hit brick's segment, crossing fraction).
// The middle of the first voxel of the ray's walk through `brick` in which the
// walk would run the finder (occupied, entered after tNear), as a distance along
// the ray: the farthest point a jump can be certified to (every voxel before it
// on the walk is empty).  The walk's own arithmetic (brick_intersect); t1 when
// no voxel qualifies.
__device__ float first_finder_voxel(const DevScene &s, uint32_t brick, float3 rp, float3 rd, float3 inv, float tNear,
                                    float t0, float t1) {
  const uint32_t bsz = s.sbs_hdr.brick_size;
  const uint4 nd = __ldg(reinterpret_cast<const uint4 *>(s.bricks) + brick);
  const float sz = float(nd.y & 0x0000FFFF), sz_inv = 2.0f / sz, bs = float(bsz), d = 2.0f / (sz * bs);
  const float scale = 0.5f * sz * bs;
  const float3 bmin = add(f3(-1, -1, -1), scl(sz_inv, f3(float(nd.x >> 16), float(nd.x & 0xFFFF), float(nd.y >> 16))));
  const uint32_t *occ = s.occ + size_t(brick) * s.occ_words;
  const bool posx = inv.x > 0.0f, posy = inv.y > 0.0f, posz = inv.z > 0.0f;
  float t = t0;
  const uint32_t max_steps = walk_step_bound(bsz, t1 - t0);
  for (uint32_t step = 0; t < t1 && step < max_steps; step++) {
    const int3 v = walk_voxel(rp, rd, t, bmin, scale, bs);
    const float3 mp = add(bmin, scl(d, f3(float(v.x), float(v.y), float(v.z))));
    const float ex = fmn(fmn(inv.x * ((posx ? mp.x + d : mp.x) - rp.x), inv.y * ((posy ? mp.y + d : mp.y) - rp.y)),
                         inv.z * ((posz ? mp.z + d : mp.z) - rp.z));
    const uint32_t vid = (uint32_t(v.x) * bsz + uint32_t(v.y)) * bsz + uint32_t(v.z);
    if ((__ldg(&occ[vid >> 5]) >> (vid & 31u)) & 1u) {
      const float en = fmx(fmx(inv.x * ((posx ? mp.x : mp.x + d) - rp.x), inv.y * ((posy ? mp.y : mp.y + d) - rp.y)),
                           inv.z * ((posz ? mp.z : mp.z + d) - rp.z));
      if (tNear < en) return fmn(fmx(0.5f * (en + ex), t0), t1);   // the voxel may reach past the segment
    }
    t += fmx(0.0f, ex - t) + 1e-6f;
  }
  return t1;
}

__global__ void __launch_bounds__(128) gen_triples_kernel(DevScene s, const DevView *views, uint32_t n_views,
                                                          uint64_t total_pix, TripleBuf out, uint32_t target) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= total_pix) return;
  uint32_t v = 0;
  while (v + 1 < n_views && views[v + 1].pix_offset <= i) v++;
  const DevView &V = views[v];
  const uint32_t p = uint32_t(i - V.pix_offset), x = p % V.width, y = p / V.width;
  float3 pos, dir;
  eye_ray(x, y, V.width, V.height, 0.5f, 0.5f, V.proj_inv, V.wv_inv, pos, dir);
  Hit hit;
  Counters cnt = {0, 0, 0, 0};
  trace<LRT_TYPE_SDF_SBS, false, LRT_INTERSECT_NEWTON>(s, pos, 0.0f, dir, 1e9f, hit, cnt);
  if (hit.prim == kMiss) return;
  const float3 rp = matmul4x3(s.inst_inv, pos), rd = matmul3x3(s.inst_inv, dir);
  const float3 inv = safe_inverse(rd);
  float f[16], t0, t1;
  brick_features(s, hit.prim, rp, rd, inv, f, t0, t1);
  if (!(t1 > t0)) return;
  const unsigned long long k = atomicAdd(out.count, 1ull);
  if (k >= out.capacity) return;
  uint4 *dst = reinterpret_cast<uint4 *>(out.feat);
  dst[feat_u4(k, 0)] = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
  dst[feat_u4(k, 1)] =
      make_uint4(pack_bf16(f[8], f[9]), pack_bf16(f[10], f[11]), pack_bf16(f[12], f[13]), pack_bf16(f[14], f[15]));
  // target 0: the crossing's fraction of the segment (t*); 1: the first voxel the
  // walk runs the finder in (where a jump should land)
  const float tt = target ? first_finder_voxel(s, hit.prim, rp, rd, inv, 0.1f, t0, t1) : hit.t;
  out.target[k] = (tt - t0) / (t1 - t0);
}

// ---------------------------------------------------------------- training
__device__ __forceinline__ void load_weights(Weights &W, const MlpState &m) {
  for (int i = threadIdx.x; i < kBfWords; i += blockDim.x) W.w[i] = m.wbf[i];
}

// per-column sums over the 32 rows of the warp's C tiles: lanes g == 0 (0..3)
// end with the totals of columns nt*8 + 2t + j
__device__ __forceinline__ void add_colsums(float p[4][2], float *g_out, int lane) {
#pragma unroll
  for (int nt = 0; nt < 4; nt++)
#pragma unroll
    for (int j = 0; j < 2; j++) {
      float v = p[nt][j];
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 4);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 8);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 16);
      if (lane < 4) atomicAdd(&g_out[nt * 8 + 2 * lane + j], v);
    }
}

// One step over `batch` samples (128 per block): loss, gradient into m.grad;
// with update, the last block to finish applies Adam and clears the gradient.
__global__ void __launch_bounds__(128) mlp_train_kernel(TripleView data, MlpState m, uint32_t batch, uint32_t step,
                                                        uint32_t seed, int random, int update, float lr, float b1,
                                                        float b2, float eps) {
  __shared__ Weights W;
  __shared__ __align__(16) __nv_bfloat16 sx[4][32 * kIn];
  __shared__ __align__(16) __nv_bfloat16 sg[4][32 * kHid];
  __shared__ __align__(16) __nv_bfloat16 sh[4][32 * kHid];
  __shared__ float sy[4][32], sdy[4][32];
  __shared__ float gsum[kParams];
  __shared__ unsigned int last;
  load_weights(W, m);
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) gsum[i] = 0.0f;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
  const uint32_t gid = blockIdx.x * 128 + threadIdx.x;
  const bool valid = gid < batch;
  uint64_t idx = 0;
  if (valid) idx = random ? (uint64_t(hash3(seed, step, gid)) * data.n) >> 32 : uint64_t(gid);
  // the sample's 16 bf16 features into the warp tile (zeros for padding lanes)
  {
    uint4 a = make_uint4(0, 0, 0, 0), b = a;
    if (valid) {
      const uint4 *src = reinterpret_cast<const uint4 *>(data.feat);
      a = src[feat_u4(data.first + idx, 0)];
      b = src[feat_u4(data.first + idx, 1)];
    }
    uint4 *dst = reinterpret_cast<uint4 *>(&sx[w][lane * kIn]);
    dst[0] = a;
    dst[1] = b;
  }
  __syncwarp();
  float h1[2][4][4], h2[2][4][4];
  const float y = forward_warp<true>(W, sx[w], sy[w], lane, h1, h2);
  const float target = valid ? data.target[data.first + idx] : 0.0f;
  const float err = valid ? (y - target) : 0.0f;
  float l = err * err;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
  if (lane == 0 && m.loss) atomicAdd(m.loss, l / float(batch));
  sdy[w][lane] = 2.0f * err / float(batch);
  __syncwarp();
  // ---- layer 3: dW3[k] = sum dy h2[:,k], db3 = sum dy; dh2 = dy W3 (h2 > 0)
  const __nv_bfloat16 *w3 = W.w + kBfW3;
  float p[4][2];
  float dh2[2][4][4];
#pragma unroll
  for (int nt = 0; nt < 4; nt++) { p[nt][0] = p[nt][1] = 0.0f; }
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    const float dlo = sdy[w][mt * 16 + g], dhi = sdy[w][mt * 16 + g + 8];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      const int col = nt * 8 + 2 * t;
      p[nt][0] += dlo * h2[mt][nt][0] + dhi * h2[mt][nt][2];
      p[nt][1] += dlo * h2[mt][nt][1] + dhi * h2[mt][nt][3];
      const float wa = __bfloat162float(w3[col]), wb = __bfloat162float(w3[col + 1]);
      dh2[mt][nt][0] = h2[mt][nt][0] > 0.0f ? dlo * wa : 0.0f;
      dh2[mt][nt][1] = h2[mt][nt][1] > 0.0f ? dlo * wb : 0.0f;
      dh2[mt][nt][2] = h2[mt][nt][2] > 0.0f ? dhi * wa : 0.0f;
      dh2[mt][nt][3] = h2[mt][nt][3] > 0.0f ? dhi * wb : 0.0f;
    }
  }
  add_colsums(p, gsum + kOffW3, lane);
  {
    float v = sdy[w][lane];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    if (lane == 0) atomicAdd(&gsum[kOffB3], v);
  }
  // db2 = column sums of dh2; stage dh2 and h1 (bf16) for the transposed products
#pragma unroll
  for (int nt = 0; nt < 4; nt++) { p[nt][0] = p[nt][1] = 0.0f; }
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      const int col = nt * 8 + 2 * t, r = mt * 16 + g;
      p[nt][0] += dh2[mt][nt][0] + dh2[mt][nt][2];
      p[nt][1] += dh2[mt][nt][1] + dh2[mt][nt][3];
      *reinterpret_cast<uint32_t *>(&sg[w][r * kHid + col]) = pack_bf16(dh2[mt][nt][0], dh2[mt][nt][1]);
      *reinterpret_cast<uint32_t *>(&sg[w][(r + 8) * kHid + col]) = pack_bf16(dh2[mt][nt][2], dh2[mt][nt][3]);
      *reinterpret_cast<uint32_t *>(&sh[w][r * kHid + col]) = pack_bf16(h1[mt][nt][0], h1[mt][nt][1]);
      *reinterpret_cast<uint32_t *>(&sh[w][(r + 8) * kHid + col]) = pack_bf16(h1[mt][nt][2], h1[mt][nt][3]);
    }
  add_colsums(p, gsum + kOffB2, lane);
  __syncwarp();
  // ---- dW2[o][i] = sum_b dh2[b][o] h1[b][i]: A = dh2^T (32 x 32 samples), B = h1
#pragma unroll
  for (int mo = 0; mo < 2; mo++)
#pragma unroll
    for (int ni = 0; ni < 4; ni++) {
      float c[4] = {0, 0, 0, 0};
#pragma unroll
      for (int kb = 0; kb < 2; kb++) {
        uint32_t a[4], b0, b1;
        ld_at(a, sg[w], kHid, mo * 16, kb * 16, lane);
        ld_b_kn(b0, b1, sh[w], kHid, ni * 8, kb * 16, lane);
        mma16816(c, a, b0, b1);
      }
      const int o = mo * 16 + g, i = ni * 8 + 2 * t;
      atomicAdd(&gsum[kOffW2 + o * kHid + i], c[0]);
      atomicAdd(&gsum[kOffW2 + o * kHid + i + 1], c[1]);
      atomicAdd(&gsum[kOffW2 + (o + 8) * kHid + i], c[2]);
      atomicAdd(&gsum[kOffW2 + (o + 8) * kHid + i + 1], c[3]);
    }
  // ---- dh1 = (dh2 W2) (h1 > 0): A = dh2 (C tiles re-packed), B[k=o][n=i] = W2[o][i]
  float dh1[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    uint32_t a[2][4];
    c_to_a(dh2[mt], a);
#pragma unroll
    for (int ni = 0; ni < 4; ni++) {
      float c[4] = {0, 0, 0, 0};
#pragma unroll
      for (int kb = 0; kb < 2; kb++) {
        uint32_t b0, b1;
        ld_b_kn(b0, b1, W.w + kBfW2, kHid, ni * 8, kb * 16, lane);
        mma16816(c, a[kb], b0, b1);
      }
#pragma unroll
      for (int e = 0; e < 4; e++) dh1[mt][ni][e] = h1[mt][ni][e] > 0.0f ? c[e] : 0.0f;
    }
  }
  __syncwarp();
#pragma unroll
  for (int nt = 0; nt < 4; nt++) { p[nt][0] = p[nt][1] = 0.0f; }
#pragma unroll
  for (int mt = 0; mt < 2; mt++)
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      const int col = nt * 8 + 2 * t, r = mt * 16 + g;
      p[nt][0] += dh1[mt][nt][0] + dh1[mt][nt][2];
      p[nt][1] += dh1[mt][nt][1] + dh1[mt][nt][3];
      *reinterpret_cast<uint32_t *>(&sg[w][r * kHid + col]) = pack_bf16(dh1[mt][nt][0], dh1[mt][nt][1]);
      *reinterpret_cast<uint32_t *>(&sg[w][(r + 8) * kHid + col]) = pack_bf16(dh1[mt][nt][2], dh1[mt][nt][3]);
    }
  add_colsums(p, gsum + kOffB1, lane);
  __syncwarp();
  // ---- dW1[i][j] = sum_b dh1[b][i] x[b][j]: A = dh1^T, B = x
#pragma unroll
  for (int mi = 0; mi < 2; mi++)
#pragma unroll
    for (int nj = 0; nj < 2; nj++) {
      float c[4] = {0, 0, 0, 0};
#pragma unroll
      for (int kb = 0; kb < 2; kb++) {
        uint32_t a[4], b0, b1;
        ld_at(a, sg[w], kHid, mi * 16, kb * 16, lane);
        ld_b_kn(b0, b1, sx[w], kIn, nj * 8, kb * 16, lane);
        mma16816(c, a, b0, b1);
      }
      const int i = mi * 16 + g, j = nj * 8 + 2 * t;
      atomicAdd(&gsum[kOffW1 + i * kIn + j], c[0]);
      atomicAdd(&gsum[kOffW1 + i * kIn + j + 1], c[1]);
      atomicAdd(&gsum[kOffW1 + (i + 8) * kIn + j], c[2]);
      atomicAdd(&gsum[kOffW1 + (i + 8) * kIn + j + 1], c[3]);
    }
  __syncthreads();
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) atomicAdd(&m.grad[i], gsum[i]);
  if (!update) return;
  // the last block applies Adam (ticket after a fence that publishes this block's sums)
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = (atomicAdd(m.ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  const float c1 = 1.0f - powf(b1, float(step + 1)), c2 = 1.0f - powf(b2, float(step + 1));
  for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
    const float gi = atomicExch(&m.grad[i], 0.0f);
    const float mi = b1 * m.adam_m[i] + (1.0f - b1) * gi;
    const float vi = b2 * m.adam_v[i] + (1.0f - b2) * gi * gi;
    m.adam_m[i] = mi;
    m.adam_v[i] = vi;
    m.master[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
  __syncthreads();
  // refresh the bf16 image: W1, W2, W3 (row 0 of its 8-row tile), bias blocks
  for (int i = threadIdx.x; i < kBfWords; i += blockDim.x)
    reinterpret_cast<uint16_t *>(m.wbf)[i] = weight_image_word(m.master, i);
  if (threadIdx.x == 0) *m.ticket = 0u;
}

// MLP outputs for n given samples (bf16 features)
__global__ void __launch_bounds__(128) mlp_infer_kernel(TripleView data, MlpState m, float *out) {
  __shared__ Weights W;
  __shared__ __align__(16) __nv_bfloat16 sx[4][32 * kIn];
  __shared__ float sy[4][32];
  load_weights(W, m);
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint64_t gid = uint64_t(blockIdx.x) * 128 + threadIdx.x;
  uint4 a = make_uint4(0, 0, 0, 0), b = a;
  if (gid < data.n) {
    const uint4 *src = reinterpret_cast<const uint4 *>(data.feat);
    a = src[feat_u4(data.first + gid, 0)];
    b = src[feat_u4(data.first + gid, 1)];
  }
  uint4 *dst = reinterpret_cast<uint4 *>(&sx[w][lane * kIn]);
  dst[0] = a;
  dst[1] = b;
  __syncwarp();
  const float y = forward_warp<false>(W, sx[w], sy[w], lane, nullptr, nullptr);
  if (gid < data.n) out[gid] = y;
}

// ---------------------------------------------------------------- 128-sample tiles on tcgen05
// The network on the fifth-generation tensor cores, warp-specialised and
// pipelined.  A persistent CTA of nine warps walks the 128-sample tiles of the
// store that hold the requested window, up to four tiles in flight (one TMEM
// accumulator of 32 columns and one shared-memory hidden buffer each, tile j in
// slot j % 4).  Every layer is its products plus its bias block (three BF16
// terms of the bias against a constant block of ones, mlp_image.h), summed in
// the tensor core, so the epilogue adds no bias.
//   warp 0 (one thread)  loads each tile's 4 KB of features with one bulk copy
//                        (cp.async.bulk) into a ring of three shared-memory
//                        stages -- the store's tile layout is the MMA's
//                        operand layout -- and issues layer 1 (M = 128, N = 32:
//                        K = 16 features, then K = 16 of the bias block) of the
//                        tile loaded two copies earlier, once its slot is free;
//   warps 1-8            two epilogue groups of four warps (even and odd tiles)
//                        working on two tiles at once.  Each warp reads its 32
//                        TMEM lanes (rows) and applies ReLU and BF16 rounding
//                        (one cvt.rn.relu.bf16x2.f32 per pair) into the next
//                        layer's A operand in shared memory; the group's first
//                        thread issues layer 2 (N = 32) and layer 3 (N = 16,
//                        column 0 the output) as soon as its four warps have
//                        written the layer's input; after layer 3 each warp
//                        writes its rows' column 0.
// Every hand-off is an mbarrier, waited on with the blocking try_wait (no CTA
// barrier inside the loop).  Measured with clock64 stamps and ncu, the epilogue
// is what bounds the kernel: with the biases added on the CUDA cores it issued
// about 1,400 warp instructions per tile.  The weights are staged once per CTA
// in the canonical K-major layout.  Waits are bounded by `wait_limit` polls: a
// timeout sets status bit 1 and makes the role leave its loop; the others run
// out the same way, then each issuing thread waits (at most kTcWait polls) for
// everything it issued, the loader for every copy it started, and the TMEM is
// freed.
constexpr uint32_t kTcLbo = 128;         // adjacent core matrices along K (weights, hidden operands)
constexpr uint32_t kTcWait = 1u << 20;   // mbarrier polls of the final drain (up to ~1 us each)
constexpr int kTcStages = 3;             // feature tiles in shared memory
constexpr int kTcAcc = 4;                // tiles in flight (TMEM accumulators, hidden buffers)
constexpr int kTcThreads = 288;
constexpr int kTcBlocksPerSm = 4;        // 4 x 128 TMEM columns
constexpr uint32_t kTcHidBytes = 128 * kHid * 2;
constexpr uint32_t kTcDynSmem = kTcStages * 4096 + kTcAcc * kTcHidBytes;

// ReLU + BF16 of one 32-wide accumulator row (this lane's TMEM lane, read in two
// 16-column halves to keep registers low) into the A operand of the next layer
__device__ __forceinline__ void hidden_to_smem(uint32_t trow, uint8_t *sH, uint32_t row) {
#pragma unroll
  for (int h = 0; h < 32; h += 16) {
    float v[16];
    tc05::tmem_ld16(trow + uint32_t(h), v);
#pragma unroll
    for (int j = 0; j < 16; j += 8) {
      uint4 q;
      q.x = pack_bf16_relu(v[j], v[j + 1]);
      q.y = pack_bf16_relu(v[j + 2], v[j + 3]);
      q.z = pack_bf16_relu(v[j + 4], v[j + 5]);
      q.w = pack_bf16_relu(v[j + 6], v[j + 7]);
      *reinterpret_cast<uint4 *>(sH + tc05::kmajor_offset(row, uint32_t(h + j), kTcLbo, 512)) = q;
    }
  }
}

__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm) mlp_infer_tc_kernel(TripleView data, MlpState m,
                                                                                  float *out, unsigned int *status,
                                                                                  uint32_t wait_limit) {
  extern __shared__ __align__(128) uint8_t tc_dyn[];
  uint8_t *const sX = tc_dyn;                           // kTcStages x 4 KB feature tiles
  uint8_t *const sH = tc_dyn + kTcStages * 4096;        // kTcAcc x hidden operand
  __shared__ __align__(128) uint8_t sW1[kHid * kIn * 2], sB1[kHid * 16 * 2];
  __shared__ __align__(128) uint8_t sW2[kHid * kHid * 2], sB2[kHid * 16 * 2];
  __shared__ __align__(128) uint8_t sW3[16 * kHid * 2], sB3[16 * 16 * 2];
  __shared__ __align__(128) uint8_t sOnes[128 * 16 * 2];
  __shared__ __align__(8) uint64_t full[kTcStages], empty[kTcStages];
  __shared__ __align__(8) uint64_t l1[kTcAcc], l2[kTcAcc], l3[kTcAcc], afree[kTcAcc], fin[3];
  __shared__ uint32_t tmem_slot;
  const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
  const uint64_t t_first = data.first >> 7;
  const uint64_t n_tiles = data.n ? ((data.first + data.n - 1) >> 7) - t_first + 1 : 0;
  const uint32_t my_tiles = blockIdx.x < n_tiles ? uint32_t((n_tiles - 1 - blockIdx.x) / gridDim.x + 1) : 0u;
  // weights (W stored [n][k] is the K-major B operand), bias blocks and the ones
  // block into the canonical layout
  const __nv_bfloat16 zero = __float2bfloat16_rn(0.0f), one = __float2bfloat16_rn(1.0f);
  auto put = [](uint8_t *base, uint32_t r, uint32_t k, uint32_t sbo, __nv_bfloat16 v) {
    *reinterpret_cast<__nv_bfloat16 *>(base + tc05::kmajor_offset(r, k, kTcLbo, sbo)) = v;
  };
  for (uint32_t i = tid; i < kHid * kIn; i += kTcThreads) put(sW1, i / kIn, i % kIn, 256, m.wbf[kBfW1 + i]);
  for (uint32_t i = tid; i < kHid * kHid; i += kTcThreads) put(sW2, i / kHid, i % kHid, 512, m.wbf[kBfW2 + i]);
  for (uint32_t i = tid; i < 16 * kHid; i += kTcThreads)
    put(sW3, i / kHid, i % kHid, 512, i < 8 * kHid ? m.wbf[kBfW3 + i] : zero);
  for (uint32_t i = tid; i < kHid * 16; i += kTcThreads) {
    put(sB1, i / 16, i % 16, 256, m.wbf[kBfB1 + i]);
    put(sB2, i / 16, i % 16, 256, m.wbf[kBfB2 + i]);
  }
  for (uint32_t i = tid; i < 16 * 16; i += kTcThreads) put(sB3, i / 16, i % 16, 256, i < 8 * 16 ? m.wbf[kBfB3 + i] : zero);
  for (uint32_t i = tid; i < 128 * 16; i += kTcThreads) put(sOnes, i / 16, i % 16, 256, (i % 16) < 3 ? one : zero);
  if (tid == 0) {
    for (int i = 0; i < kTcStages; i++) {
      tc05::mbar_init(&full[i], 1);
      tc05::mbar_init(&empty[i], 1);
    }
    for (int a = 0; a < kTcAcc; a++) {
      tc05::mbar_init(&l1[a], 1);
      tc05::mbar_init(&l2[a], 1);
      tc05::mbar_init(&l3[a], 1);
      tc05::mbar_init(&afree[a], 1);
    }
    for (int k = 0; k < 3; k++) tc05::mbar_init(&fin[k], 1);
    tc05::fence_mbar_init();
  }
  if (warp == 0) tc05::tmem_alloc(&tmem_slot, 32 * kTcAcc);
  tc05::fence_proxy_async();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tbase = tmem_slot;
  const uint32_t aOnes = tc05::smem_addr(sOnes);
  auto tile_of = [&](uint32_t j) { return t_first + blockIdx.x + uint64_t(j) * gridDim.x; };
  uint32_t issued = 0, consumed = 0;   // the loader's copies started / read by a layer 1

  if (warp == 0) {
    // ---- loader and layer 1: tile j's copy is started two tiles ahead of its layer 1
    if (lane == 0) {
      constexpr uint32_t kId32 = tc05::idesc_bf16_f32(128, 32);
      // descriptors built once; a stage's feature tile is dX plus its offset in 16-byte units
      const uint64_t dX = tc05::smem_desc(tc05::smem_addr(sX), 2048, 128);
      const uint64_t dW1 = tc05::smem_desc(tc05::smem_addr(sW1), kTcLbo, 256);
      const uint64_t dB1 = tc05::smem_desc(tc05::smem_addr(sB1), kTcLbo, 256);
      const uint64_t dOnes = tc05::smem_desc(aOnes, kTcLbo, 256);
      bool ok = true;
      for (uint32_t j = 0; ok && j < my_tiles + kTcStages - 1; j++) {
        if (j < my_tiles) {
          const uint32_t st = j % kTcStages;
          if (j >= uint32_t(kTcStages) && !tc05::mbar_wait(&empty[st], ((j / kTcStages) - 1) & 1u, wait_limit)) {
            ok = false;
            break;
          }
          tc05::mbar_arrive_expect_tx(&full[st], 4096);
          tc05::bulk_g2s(sX + st * 4096, data.feat + tile_of(j) * 2048, 4096, &full[st]);
          issued = j + 1;
        }
        if (j + 1 >= uint32_t(kTcStages) && j + 1 - kTcStages < my_tiles) {
          const uint32_t jj = j + 1 - kTcStages, a = jj % kTcAcc, st = jj % kTcStages;
          if (jj >= uint32_t(kTcAcc) && !tc05::mbar_wait(&afree[a], ((jj / kTcAcc) - 1) & 1u, wait_limit)) {
            ok = false;
            break;
          }
          if (!tc05::mbar_wait(&full[st], (jj / kTcStages) & 1u, wait_limit)) { ok = false; break; }
          tc05::fence_after_sync();
          tc05::mma_bf16(tbase + a * 32u, dX + uint64_t((st * 4096u) >> 4), dW1, kId32, false);
          tc05::mma_bf16(tbase + a * 32u, dOnes, dB1, kId32, true);
          tc05::mma_commit(&l1[a]);
          tc05::mma_commit(&empty[st]);   // the stage is free once layer 1 has read it
          consumed = jj + 1;
        }
      }
      if (!ok) atomicOr(status, 2u);
      tc05::mma_commit(&fin[0]);
      if (!tc05::mbar_wait(&fin[0], 0, kTcWait)) atomicOr(status, 2u);
    }
  } else {
    // ---- epilogue: group g takes tiles g, g + 2, ...; warp w reads TMEM lanes
    // 32 * (w % 4) .. + 31 (rows of the tile).  The group's first warp waits for
    // each layer's completion barrier and issues the group's layers 2 and 3; the
    // four warps meet on the group's named barrier (id 1 + g), where they sleep.
    constexpr uint32_t kId32 = tc05::idesc_bf16_f32(128, 32), kId16 = tc05::idesc_bf16_f32(128, 16);
    const uint32_t g = (warp - 1) >> 2, q = warp & 3u, row = 32u * q + lane, trow = tbase + ((32u * q) << 16);
    const uint32_t bar = 1u + g;
    const bool leader = ((warp - 1) & 3u) == 0;   // the whole warp waits, its lane 0 issues
    // the layers' shared-memory descriptors, built once (a slot's hidden operand
    // descriptor is dH plus the slot's offset in 16-byte units)
    struct LayerDesc {
      uint64_t w0, w1, bias;
      uint32_t idesc;
    };
    const uint32_t aW2 = tc05::smem_addr(sW2), aW3 = tc05::smem_addr(sW3);
    const LayerDesc d2{tc05::smem_desc(aW2, kTcLbo, 512), tc05::smem_desc(aW2 + 2 * kTcLbo, kTcLbo, 512),
                       tc05::smem_desc(tc05::smem_addr(sB2), kTcLbo, 256), kId32};
    const LayerDesc d3{tc05::smem_desc(aW3, kTcLbo, 512), tc05::smem_desc(aW3 + 2 * kTcLbo, kTcLbo, 512),
                       tc05::smem_desc(tc05::smem_addr(sB3), kTcLbo, 256), kId16};
    const uint64_t dH = tc05::smem_desc(tc05::smem_addr(sH), kTcLbo, 512);
    const uint64_t dOnes = tc05::smem_desc(aOnes, kTcLbo, 256);
    bool failed = false;
    // the leader waits for `done`; false in every warp of the group on a timeout
    auto group_wait = [&](uint64_t *done, uint32_t ph) {
      bool bad = false;
      if (leader) bad = !tc05::mbar_wait(done, ph, wait_limit);
      return !tc05::bar_or(bar, 128, bad);
    };
    for (uint32_t j = g; j < my_tiles && !failed; j += 2) {
      const uint32_t a = j % kTcAcc, ph = (j / kTcAcc) & 1u;
      uint8_t *const hb = sH + a * kTcHidBytes;
#pragma unroll 1
      for (int layer = 1; layer <= 2; layer++) {
        if (!group_wait(layer == 1 ? &l1[a] : &l2[a], ph)) { failed = true; break; }
        tc05::fence_after_sync();
        hidden_to_smem(trow + a * 32u, hb, row);
        tc05::fence_proxy_async();
        tc05::fence_before_sync();
        tc05::bar_sync(bar, 128);   // the tile's 128 rows of this layer's output are in shared memory
        if (leader && lane == 0) {  // the next layer: products of this layer's output, then its bias block
          tc05::fence_after_sync();
          const LayerDesc &L = layer == 1 ? d2 : d3;
          const uint64_t ha = dH + uint64_t((a * kTcHidBytes) >> 4);   // the slot's hidden operand
          const uint32_t d = tbase + a * 32u;
          tc05::mma_bf16(d, ha, L.w0, L.idesc, false);
          tc05::mma_bf16(d, ha + (2 * kTcLbo >> 4), L.w1, L.idesc, true);
          tc05::mma_bf16(d, dOnes, L.bias, L.idesc, true);
          tc05::mma_commit(layer == 1 ? &l2[a] : &l3[a]);
        }
      }
      if (failed || !group_wait(&l3[a], ph)) { failed = true; break; }
      tc05::fence_after_sync();
      const float y = tc05::tmem_ld1(trow + a * 32u);
      const uint64_t gi = tile_of(j) * 128 + row;
      if (gi >= data.first && gi < data.first + data.n) out[gi - data.first] = y;
      tc05::fence_before_sync();
      tc05::bar_sync(bar, 128);     // all four warps have read the slot
      if (leader && lane == 0) tc05::mbar_arrive(&afree[a]);
    }
    if (failed && leader && lane == 0) atomicOr(status, 2u);
    if (leader && lane == 0) {   // every MMA this thread issued has completed before the TMEM is freed
      tc05::mma_commit(&fin[1 + g]);
      if (!tc05::mbar_wait(&fin[1 + g], 0, kTcWait)) atomicOr(status, 2u);
    }
  }
  __syncthreads();
  // copies no layer 1 consumed (after a timeout) land before the CTA exits
  if (warp == 0 && lane == 0)
    for (uint32_t j = consumed; j < issued; j++)
      if (!tc05::mbar_wait(&full[j % kTcStages], (j / kTcStages) & 1u, kTcWait)) atomicOr(status, 2u);
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  if (warp == 0) tc05::tmem_dealloc(tbase, 32 * kTcAcc);
}

// ---------------------------------------------------------------- render with the proposal
// The plain persistent kernel's structure (render_kernel, trace.cu) with the
// leaf phase made warp-synchronous: every lane searches for its next brick,
// then the warp runs the network once for all lanes holding one (the others
// feed zeros), and each such lane walks its brick from the proposed start.
__global__ void __launch_bounds__(128, 4) render_proposal_kernel(DevScene s, RenderLaunch L, MlpState m,
                                                                 unsigned long long *stats) {
  __shared__ Weights W;
  __shared__ __align__(16) __nv_bfloat16 sx[4][32 * kIn];
  __shared__ float sy[4][32];
  load_weights(W, m);
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, wi = threadIdx.x >> 5;
  Counters cnt = {0, 0, 0, 0};
  unsigned long long n_prop = 0, n_jump = 0, n_hit_jump = 0, n_skip = 0;
  for (;;) {
    uint32_t tile = 0;
    if (lane == 0) tile = atomicAdd(L.tile_counter, 1u);
    tile = __shfl_sync(0xffffffffu, tile, 0);
    if (tile >= L.total_tiles) break;
    uint32_t v = 0;
    while (v + 1 < L.n_views && L.views[v + 1].tile_offset <= tile) v++;
    const DevView &V = L.views[v];
    const uint32_t lt = tile - V.tile_offset, lw = V.tile_w_log2;
    const uint32_t x = (lt % V.tiles_x) * (1u << lw) + (lane & ((1u << lw) - 1u));
    const uint32_t y = (lt / V.tiles_x) * (32u >> lw) + (lane >> lw);
    const bool in = x < V.width && y < V.height;
    float3 pos = f3(0, 0, 0), dir = f3(0, 0, 1);
    if (in) eye_ray(x, y, V.width, V.height, 0.5f, 0.5f, V.proj_inv, V.wv_inv, pos, dir);
    Hit hit;
    hit.t = 1e9f;
    hit.prim = kMiss;
    hit.geom = kMiss;
    hit.c0 = 1.0f;
    hit.c1 = hit.c2 = hit.c3 = 0.0f;
    bool active = in;
    if (active) {   // TLAS leaf box of the single instance
      const float3 invw = safe_inverse(dir);
      const float2 bh = ray_box(pos, invw, s.inst_bmin[0], s.inst_bmin[1], s.inst_bmin[2], s.inst_bmax[0],
                                s.inst_bmax[1], s.inst_bmax[2]);
      active = (bh.x <= bh.y) && (bh.y > 0.0f) && (bh.x < hit.t);
    }
    const float3 rp = matmul4x3(s.inst_inv, pos), rd = matmul3x3(s.inst_inv, dir);
    const float3 inv = safe_inverse(rd);
    const float tNearSdf = 0.1f;
    uint2 st[kStackSize];
    int sp = 0;
    if (active) {
      st[0] = make_uint2(0u, __float_as_uint(-3.4e38f));
      sp = 1;
    }
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
        visit_node<false, kStackSize>(s, ref, rp, inv, 0.0f, hit.t, st, sp, cnt);
      }
      if (!__any_sync(0xffffffffu, have_leaf)) break;
      float f[16], t0 = 0.0f, t1 = 0.0f;
#pragma unroll
      for (int k = 0; k < 16; k++) f[k] = 0.0f;
      if (have_leaf) brick_features(s, leaf, rp, rd, inv, f, t0, t1);
      uint4 *dst = reinterpret_cast<uint4 *>(&sx[wi][lane * kIn]);
      dst[0] = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
      dst[1] = make_uint4(pack_bf16(f[8], f[9]), pack_bf16(f[10], f[11]), pack_bf16(f[12], f[13]),
                          pack_bf16(f[14], f[15]));
      __syncwarp();
      const float u = forward_warp<false>(W, sx[wi], sy[wi], lane, nullptr, nullptr);
      if (have_leaf) {
        n_prop++;
        bool jumped = false;
        uint32_t skipped = 0;
        const float start = proposal_start(s, leaf, rp, rd, inv, t0, t1, u, jumped, skipped);
        n_skip += skipped;
        const float before = hit.t;
        brick_intersect<false, false, LRT_INTERSECT_NEWTON>(s, rp, rd, inv, tNearSdf, leaf, hit, cnt, nullptr, start);
        if (jumped) {
          n_jump++;
          if (hit.t < before) n_hit_jump++;
        }
      }
    }
    if (in) {
      const size_t pix = size_t(V.pix_offset) + size_t(y) * V.width + x;
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
    }
  }
  if (stats) {
    atomicAdd(&stats[0], n_prop);
    atomicAdd(&stats[1], n_jump);
    atomicAdd(&stats[2], n_hit_jump);
    atomicAdd(&stats[3], n_skip);
  }
}

}  // namespace dev

cudaError_t launch_gen_triples(const DevScene &s, const DevView *views, uint32_t n_views, uint64_t total_pix,
                               const TripleBuf &out, uint32_t target, cudaStream_t st) {
  const uint64_t blocks = (total_pix + 127) / 128;
  dev::gen_triples_kernel<<<unsigned(blocks), 128, 0, st>>>(s, views, n_views, total_pix, out, target);
  return cudaGetLastError();
}

cudaError_t launch_mlp_step(const TripleView &data, const MlpState &m, uint32_t batch, uint32_t step, uint32_t seed,
                            bool random, bool update, float lr, float b1, float b2, float eps, cudaStream_t st) {
  const uint32_t blocks = (batch + 127) / 128;
  dev::mlp_train_kernel<<<blocks, 128, 0, st>>>(data, m, batch, step, seed, random ? 1 : 0, update ? 1 : 0, lr, b1,
                                                b2, eps);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer(const TripleView &data, const MlpState &m, float *out, cudaStream_t st) {
  const uint64_t blocks = (data.n + 127) / 128;
  dev::mlp_infer_kernel<<<unsigned(blocks), 128, 0, st>>>(data, m, out);
  return cudaGetLastError();
}

cudaError_t launch_mlp_infer_tc(const TripleView &data, const MlpState &m, float *out, unsigned int *status,
                                cudaStream_t st, uint32_t wait_limit) {
  int device = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  if (e != cudaSuccess) return e;
  if (data.n == 0) return cudaSuccess;
  const uint64_t tiles = ((data.first + data.n - 1) >> 7) - (data.first >> 7) + 1;
  uint64_t blocks = uint64_t(sms) * dev::kTcBlocksPerSm;
  if (blocks > tiles) blocks = tiles;
  e = cudaFuncSetAttribute(dev::mlp_infer_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dev::kTcDynSmem));
  if (e != cudaSuccess) return e;
  dev::mlp_infer_tc_kernel<<<unsigned(blocks), dev::kTcThreads, dev::kTcDynSmem, st>>>(data, m, out, status,
                                                                                        wait_limit);
  return cudaGetLastError();
}

cudaError_t launch_render_proposal(const DevScene &s, const RenderLaunch &L, const MlpState &m,
                                   unsigned long long *stats, int num_sms, cudaStream_t st) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dev::render_proposal_kernel, 128, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  uint32_t blocks = uint32_t(num_sms) * uint32_t(per_sm);
  const uint32_t max_blocks = (L.total_tiles + 3) / 4;
  if (blocks > max_blocks) blocks = max_blocks;
  if (blocks == 0) blocks = 1;
  dev::render_proposal_kernel<<<blocks, 128, 0, st>>>(s, L, m, stats);
  return cudaGetLastError();
}

}  // namespace lrt
