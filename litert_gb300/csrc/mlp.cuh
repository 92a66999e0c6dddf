// The per-(ray, brick) proposal network: 16 -> 32 -> 32 -> 1, ReLU, BF16
// weights and activations on the tensor cores (mma.sync m16n8k16, FP32
// accumulation), one warp evaluating 32 samples (two 16-row tiles).
//
// Parameter layout (FP32 master copy, 1633 floats): W1[32][16], b1[32],
// W2[32][32], b2[32], W3[32], b3.  The BF16 copy the kernels read holds W1, W2
// and W3 padded to an 8-row tile (rows 1..7 zero), then each layer's bias as
// an extra 16-wide K block: output n's row holds the bias split into three BF16
// terms (hi, mid, lo; their sum equals the FP32 bias to about 2^-24 of it) and
// zeros.  Multiplied by a constant A block whose first three columns are 1, it
// adds the bias inside the tensor core, after the layer's products, so neither
// engine adds a bias on the CUDA cores.
//
// Fragment layouts (PTX mma.m16n8k16, .row.col, g = lane>>2, t = lane&3):
//   A (16x16): a0 = (g, 2t..2t+1), a1 = (g+8, 2t..), a2 = (g, 2t+8..), a3 = (g+8, 2t+8..)
//   B (16x8):  b0 = (k 2t..2t+1, n g), b1 = (k 2t+8..2t+9, n g)
//   C (16x8):  c0,c1 = (g, 2t..2t+1), c2,c3 = (g+8, 2t..2t+1)
// Two adjacent C tiles (columns 0..7, 8..15) re-packed to BF16 are exactly the
// A fragment of the next layer's 16-wide K block, so layers chain in registers.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#include "mlp_image.h"

namespace lrt {
namespace mlp {

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x (lo) in the low half
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
// ReLU and round-to-nearest-even to BF16 of two floats in one instruction (lo in the low half);
// equal to pack_bf16(fmaxf(lo, 0), fmaxf(hi, 0)) up to the sign of a zero
__device__ __forceinline__ uint32_t pack_bf16_relu(float lo, float hi) {
  uint32_t r;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
  return r;
}

__device__ __forceinline__ void mma16816(float d[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// two 16-bit values at (row, col) and (row, col+1) of a row-major bf16 matrix
__device__ __forceinline__ uint32_t ld_pair(const __nv_bfloat16 *m, int ld, int row, int col) {
  return *reinterpret_cast<const uint32_t *>(m + row * ld + col);
}
// (row, col) and (row+1, col): a column pair (for transposed operands)
__device__ __forceinline__ uint32_t ld_colpair(const __nv_bfloat16 *m, int ld, int row, int col) {
  const uint16_t lo = *reinterpret_cast<const uint16_t *>(m + row * ld + col);
  const uint16_t hi = *reinterpret_cast<const uint16_t *>(m + (row + 1) * ld + col);
  return uint32_t(lo) | (uint32_t(hi) << 16);
}

// A fragment (rows r0..r0+15, K block k0..k0+15) of a row-major [rows][ld] bf16 matrix
__device__ __forceinline__ void ld_a(uint32_t a[4], const __nv_bfloat16 *m, int ld, int r0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  a[0] = ld_pair(m, ld, r0 + g, k0 + 2 * t);
  a[1] = ld_pair(m, ld, r0 + g + 8, k0 + 2 * t);
  a[2] = ld_pair(m, ld, r0 + g, k0 + 2 * t + 8);
  a[3] = ld_pair(m, ld, r0 + g + 8, k0 + 2 * t + 8);
}
// A fragment of the TRANSPOSE of a row-major [K][M] matrix: A[m][k] = m_[k][m]
__device__ __forceinline__ void ld_at(uint32_t a[4], const __nv_bfloat16 *m, int ld, int m0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  a[0] = ld_colpair(m, ld, k0 + 2 * t, m0 + g);
  a[1] = ld_colpair(m, ld, k0 + 2 * t, m0 + g + 8);
  a[2] = ld_colpair(m, ld, k0 + 2 * t + 8, m0 + g);
  a[3] = ld_colpair(m, ld, k0 + 2 * t + 8, m0 + g + 8);
}
// B fragment from W stored [n][k] row-major (B[k][n] = W[n][k]): the weight layout
__device__ __forceinline__ void ld_b_nk(uint32_t &b0, uint32_t &b1, const __nv_bfloat16 *w, int ld, int n0, int k0,
                                        int lane) {
  const int g = lane >> 2, t = lane & 3;
  b0 = ld_pair(w, ld, n0 + g, k0 + 2 * t);
  b1 = ld_pair(w, ld, n0 + g, k0 + 2 * t + 8);
}
// B fragment from a row-major [k][n] matrix (B[k][n] = m[k][n])
__device__ __forceinline__ void ld_b_kn(uint32_t &b0, uint32_t &b1, const __nv_bfloat16 *m, int ld, int n0, int k0,
                                        int lane) {
  const int g = lane >> 2, t = lane & 3;
  b0 = ld_colpair(m, ld, k0 + 2 * t, n0 + g);
  b1 = ld_colpair(m, ld, k0 + 2 * t + 8, n0 + g);
}

// C tiles (16 rows x 32 cols as four n8 tiles) -> A fragments of the two K blocks
__device__ __forceinline__ void c_to_a(const float c[4][4], uint32_t a[2][4]) {
#pragma unroll
  for (int kb = 0; kb < 2; kb++) {
    a[kb][0] = pack_bf16(c[2 * kb][0], c[2 * kb][1]);
    a[kb][1] = pack_bf16(c[2 * kb][2], c[2 * kb][3]);
    a[kb][2] = pack_bf16(c[2 * kb + 1][0], c[2 * kb + 1][1]);
    a[kb][3] = pack_bf16(c[2 * kb + 1][2], c[2 * kb + 1][3]);
  }
}

// The constant A fragment of the bias blocks: columns 0..2 of every row are 1.
__device__ __forceinline__ void ones_a(uint32_t a[4], int lane) {
  const int t = lane & 3;
  const uint32_t v = t == 0 ? 0x3F803F80u : t == 1 ? 0x00003F80u : 0u;   // (1, 1) / (1, 0) / (0, 0)
  a[0] = v;
  a[1] = v;
  a[2] = 0u;
  a[3] = 0u;
}

// Shared-memory weights of a block.
struct Weights {
  __nv_bfloat16 w[kBfWords];
};

// Forward of 32 samples held as a row-major [32][16] bf16 tile `x` (row = lane
// of the sample).  Returns the output of the lane's own sample; h1/h2 (C tiles,
// post-ReLU, FP32) are kept for the backward when requested.
template <bool KEEP>
__device__ __forceinline__ float forward_warp(const Weights &W, const __nv_bfloat16 *x, float *ybuf, int lane,
                                              float h1[2][4][4], float h2[2][4][4]) {
  const int g = lane >> 2, t = lane & 3;
  float out_lo[2], out_hi[2];
  uint32_t a1s[4];
  ones_a(a1s, lane);
#pragma unroll
  for (int mt = 0; mt < 2; mt++) {
    uint32_t a[4];
    ld_a(a, x, kIn, mt * 16, 0, lane);
    // Each layer sums its products from zero, then its bias block (three BF16
    // terms against the constant ones), all in the tensor core, as the tcgen05
    // engine does: both engines round at the same points.
    float c1[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      c1[nt][0] = c1[nt][1] = c1[nt][2] = c1[nt][3] = 0.0f;
      uint32_t b0, b1;
      ld_b_nk(b0, b1, W.w + kBfW1, kIn, nt * 8, 0, lane);
      mma16816(c1[nt], a, b0, b1);
      ld_b_nk(b0, b1, W.w + kBfB1, 16, nt * 8, 0, lane);
      mma16816(c1[nt], a1s, b0, b1);
#pragma unroll
      for (int e = 0; e < 4; e++) c1[nt][e] = fmaxf(c1[nt][e], 0.0f);
    }
    uint32_t a2[2][4];
    c_to_a(c1, a2);
    float c2[4][4];
#pragma unroll
    for (int nt = 0; nt < 4; nt++) {
      c2[nt][0] = c2[nt][1] = c2[nt][2] = c2[nt][3] = 0.0f;
#pragma unroll
      for (int kb = 0; kb < 2; kb++) {
        uint32_t b0, b1;
        ld_b_nk(b0, b1, W.w + kBfW2, kHid, nt * 8, kb * 16, lane);
        mma16816(c2[nt], a2[kb], b0, b1);
      }
      uint32_t b0, b1;
      ld_b_nk(b0, b1, W.w + kBfB2, 16, nt * 8, 0, lane);
      mma16816(c2[nt], a1s, b0, b1);
#pragma unroll
      for (int e = 0; e < 4; e++) c2[nt][e] = fmaxf(c2[nt][e], 0.0f);
    }
    uint32_t a3[2][4];
    c_to_a(c2, a3);
    float c3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int kb = 0; kb < 2; kb++) {
      uint32_t b0, b1;
      ld_b_nk(b0, b1, W.w + kBfW3, kHid, 0, kb * 16, lane);
      mma16816(c3, a3[kb], b0, b1);
    }
    {
      uint32_t b0, b1;
      ld_b_nk(b0, b1, W.w + kBfB3, 16, 0, 0, lane);
      mma16816(c3, a1s, b0, b1);
    }
    out_lo[mt] = c3[0];
    out_hi[mt] = c3[2];
    if (KEEP) {
#pragma unroll
      for (int nt = 0; nt < 4; nt++)
#pragma unroll
        for (int e = 0; e < 4; e++) { h1[mt][nt][e] = c1[nt][e]; h2[mt][nt][e] = c2[nt][e]; }
    }
  }
  // column 0 of the output lives in the t == 0 lanes: rows g and g+8 of each tile
  if (t == 0) {
    ybuf[g] = out_lo[0];
    ybuf[g + 8] = out_hi[0];
    ybuf[16 + g] = out_lo[1];
    ybuf[24 + g] = out_hi[1];
  }
  __syncwarp();
  const float y = ybuf[lane];
  __syncwarp();
  return y;
}

}  // namespace mlp
}  // namespace lrt
