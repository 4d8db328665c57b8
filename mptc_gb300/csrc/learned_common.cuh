// Learned candidate proposal: a block MLP f (54 -> 256 -> 256 -> 64) and a
// candidate MLP g (32 -> 128 -> 64) whose dot product scores how likely an
// index word is to pass a block's exact error test. Only the top-K scored
// window positions get the exact test; a block none of them passes falls back
// to the exhaustive search, so every accepted block still satisfies the
// reference's acceptance rule (err_diff <= threshold) and the stream stays a
// valid MPTC stream.
//
// All matrix products run on the tensor cores through mma.sync m16n8k16 with
// BF16 operands and FP32 accumulation, in forward, backward and scoring.
//
// This header holds the sizes and the tensor-core helpers shared by the
// training kernels (learned.cuh) and the scoring kernels (learned_search.cuh).
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace mptc {

constexpr int kFeatIn = 54, kFeatPad = 64;  // block features, padded K
constexpr int kH1 = 256, kH2 = 256, kEmb = 64;
constexpr int kCandIn = 32, kCandH = 128;

__device__ __forceinline__ uint32_t pack_bf16x2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16_16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

}  // namespace mptc
