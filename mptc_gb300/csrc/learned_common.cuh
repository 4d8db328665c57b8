// Learned candidate proposal: a block MLP f (54 -> 128 -> 128 -> 64) and a
// candidate MLP g (32 -> 128 -> 64) whose dot product scores how likely an
// index word is to pass a block's exact error test. Only the top-K scored
// window positions get the exact test; a block none of them passes falls back
// to the exhaustive search, so every accepted block still satisfies the
// reference's acceptance rule (err_diff <= threshold) and the stream stays a
// valid MPTC stream.
//
// Inference (embeddings and window scoring, learned_tc.cuh) and the training
// step's matrix products (gemm_tc_kernel, learned.cuh) both run on the tcgen05
// tensor cores with BF16 operands and FP32 accumulators in tensor memory.
//
// This header holds the sizes and the input features (the same for training
// and inference).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace mptc {

constexpr int kFeatIn = 54, kFeatPad = 64;  // block features, padded K
constexpr int kH1 = 128, kH2 = 128, kEmb = 64;  // hidden widths of f, embedding width
constexpr int kCandIn = 32, kCandH = 128;
constexpr int kMaxBatch = 32;              // streams (jobs) one learned-proposal launch covers
constexpr int kMaxK = 16;                  // proposals per block
constexpr uint16_t kNoProposal = 0xFFFFu;  // empty top-K slot

// Block features, half `half` (columns 32*half .. +31) as 16 packed bf16 pairs:
// 48 pixel channels (p - lo_c) / (hi_c - lo_c) over the block's own channel
// range (0 for a flat channel), the stb endpoints ep1, ep2 as r/31, g/63,
// b/31, zero padding to 64.
template <int HALF>
__device__ __forceinline__ void block_feature_cols(const uint32_t (&w)[12], const uint32_t (&lo)[3],
                                                   const float (&inv)[3], uint32_t e1, uint32_t e2,
                                                   uint32_t (&out)[16]) {
  float f[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const int i = 32 * HALF + j;  // a compile-time column
    float v = 0.f;
    if (i < 48) {
      const uint32_t byte = (w[i >> 2] >> (8 * (i & 3))) & 0xFFu;
      v = (float)(byte - lo[i % 3]) * inv[i % 3];
    } else if (i < 54) {
      const uint32_t ep = i < 51 ? e1 : e2;
      const int ch = (i - 48) % 3;
      v = ch == 0 ? (float)(ep >> 11) * (1.0f / 31.0f)
                  : ch == 1 ? (float)((ep >> 5) & 63) * (1.0f / 63.0f) : (float)(ep & 31) * (1.0f / 31.0f);
    }
    f[j] = v;
  }
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const __nv_bfloat162 b = __floats2bfloat162_rn(f[2 * j], f[2 * j + 1]);
    out[j] = *reinterpret_cast<const uint32_t *>(&b);
  }
}

// The block's 48 pixel bytes as 12 words (rows of 12 bytes; frame rows are a
// multiple of 4 bytes apart).
__device__ __forceinline__ void load_block_words(const uint8_t *__restrict__ rgb, int width, int bx, int by,
                                                 uint32_t (&w)[12]) {
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const uint32_t *p = reinterpret_cast<const uint32_t *>(rgb + ((size_t)(4 * by + r) * width + 4 * bx) * 3);
    w[3 * r] = __ldg(p);
    w[3 * r + 1] = __ldg(p + 1);
    w[3 * r + 2] = __ldg(p + 2);
  }
}

// Feature half `half` from the block's pixel words and stb block.
__device__ __forceinline__ void block_feature_words(const uint32_t (&w)[12], uint64_t stb, int half,
                                                    uint32_t (&out)[16]) {
  uint32_t lo[3] = {255u, 255u, 255u}, hi[3] = {0u, 0u, 0u};
#pragma unroll
  for (int i = 0; i < 48; ++i) {
    const uint32_t v = (w[i >> 2] >> (8 * (i & 3))) & 0xFFu;
    lo[i % 3] = min(lo[i % 3], v);
    hi[i % 3] = max(hi[i % 3], v);
  }
  float inv[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) inv[c] = hi[c] > lo[c] ? 1.0f / (float)(hi[c] - lo[c]) : 0.0f;
  const uint32_t e1 = (uint32_t)(stb & 0xFFFF), e2 = (uint32_t)((stb >> 16) & 0xFFFF);
  if (half)
    block_feature_cols<1>(w, lo, inv, e1, e2, out);
  else
    block_feature_cols<0>(w, lo, inv, e1, e2, out);
}

__device__ __forceinline__ void block_feature_half(const uint8_t *__restrict__ rgb, int width, int bx, int by,
                                                   uint64_t stb, int half, uint32_t (&out)[16]) {
  uint32_t w[12];
  load_block_words(rgb, width, bx, by, w);
  block_feature_words(w, stb, half, out);
}

// Word features, half `half`: the 32 bits of an index word as 0/1 (half 0),
// zero padding (half 1).
__device__ __forceinline__ void word_feature_half(uint32_t word, int half, uint32_t (&out)[16]) {
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const uint32_t b0 = (word >> (2 * j)) & 1u, b1 = (word >> (2 * j + 1)) & 1u;
    // bf16 1.0 = 0x3F80
    out[j] = half ? 0u : (b0 ? 0x3F80u : 0u) | (b1 ? 0x3F800000u : 0u);
  }
}

}  // namespace mptc
