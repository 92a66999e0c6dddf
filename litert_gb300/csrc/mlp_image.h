// The proposal network's sizes, its FP32 parameter layout and the BF16 weight
// image the tensor-core kernels read (host and device; no device code).
#pragma once
#include <cstdint>
#include <cstring>

#ifndef __CUDACC__
#define LRT_HD
#else
#define LRT_HD __host__ __device__
#endif

namespace lrt {
namespace mlp {

constexpr int kIn = 16, kHid = 32;
constexpr int kParams = 1633;
constexpr int kOffW1 = 0, kOffB1 = 512, kOffW2 = 544, kOffB2 = 1568, kOffW3 = 1600, kOffB3 = 1632;
// BF16 weight image: W1 (32x16), W2 (32x32), W3 padded (8x32), bias blocks
// B1 (32x16), B2 (32x16), B3 padded (8x16)
constexpr int kBfW1 = 0, kBfW2 = 512, kBfW3 = 1536, kBfB1 = 1792, kBfB2 = 2304, kBfB3 = 2816, kBfWords = 2944;

// BF16 word of the weight image at index i (0 <= i < kBfWords) from the FP32
// parameters, as bits: the weights rounded to nearest, the biases split
LRT_HD inline uint16_t bf16_bits_rn(float x) {
  uint32_t u;
  memcpy(&u, &x, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return uint16_t(u >> 16);   // inf / NaN kept
  u += 0x7FFFu + ((u >> 16) & 1u);
  return uint16_t(u >> 16);
}
LRT_HD inline float bf16_bits_to_float(uint16_t b) {
  const uint32_t u = uint32_t(b) << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}
// term `part` (0 hi, 1 mid, 2 lo) of b = hi + mid + lo, each BF16; the
// subtractions are exact (each remainder has at most 16 significant bits)
LRT_HD inline uint16_t bias_term(float b, int part) {
  const uint16_t hi = bf16_bits_rn(b);
  const float r1 = b - bf16_bits_to_float(hi);
  const uint16_t mid = bf16_bits_rn(r1);
  const float r2 = r1 - bf16_bits_to_float(mid);
  return part == 0 ? hi : part == 1 ? mid : bf16_bits_rn(r2);
}
LRT_HD inline uint16_t weight_image_word(const float *params, int i) {
  if (i < kBfW2) return bf16_bits_rn(params[kOffW1 + i]);
  if (i < kBfW3) return bf16_bits_rn(params[kOffW2 + (i - kBfW2)]);
  if (i < kBfB1) return i - kBfW3 < kHid ? bf16_bits_rn(params[kOffW3 + (i - kBfW3)]) : uint16_t(0);
  const int blk = i < kBfB2 ? 0 : i < kBfB3 ? 1 : 2;
  const int j = i - (blk == 0 ? kBfB1 : blk == 1 ? kBfB2 : kBfB3), n = j >> 4, k = j & 15;
  if (k >= 3) return 0;
  if (blk == 0) return bias_term(params[kOffB1 + n], k);
  if (blk == 1) return bias_term(params[kOffB2 + n], k);
  return n == 0 ? bias_term(params[kOffB3], k) : uint16_t(0);
}

}  // namespace mlp
}  // namespace lrt
