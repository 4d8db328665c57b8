// Decoded-block squared error of a frame, the PSNR measure that compares the
// learned proposal's output with the exhaustive search's.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "learned_common.cuh"
#include "search.cuh"

namespace mptc {

// Decoded-stream squared error of a frame's final blocks (what a DXT1 decoder
// shows: RGB565 endpoints expanded, 4-colour if ep1 > ep2, else 3-colour with
// black), summed into *sse (u64). For PSNR comparisons of encoder variants.
__global__ void decoded_sse_kernel(const uint8_t *__restrict__ rgb, int width, int bw, int nblk,
                                   const uint64_t *__restrict__ blocks, unsigned long long *__restrict__ sse) {
  unsigned long long acc = 0;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < nblk; idx += gridDim.x * blockDim.x) {
    const int by = idx / bw, bx = idx - by * bw;
    const uint64_t b = blocks[idx];
    const uint32_t e1 = (uint32_t)(b & 0xFFFF), e2 = (uint32_t)((b >> 16) & 0xFFFF), ix = (uint32_t)(b >> 32);
    int c[4][3];
    const int r1 = (int)(e1 >> 11), g1 = (int)((e1 >> 5) & 63), b1 = (int)(e1 & 31);
    const int r2 = (int)(e2 >> 11), g2 = (int)((e2 >> 5) & 63), b2 = (int)(e2 & 31);
    c[0][0] = (r1 << 3) | (r1 >> 2); c[0][1] = (g1 << 2) | (g1 >> 4); c[0][2] = (b1 << 3) | (b1 >> 2);
    c[1][0] = (r2 << 3) | (r2 >> 2); c[1][1] = (g2 << 2) | (g2 >> 4); c[1][2] = (b2 << 3) | (b2 >> 2);
    for (int k = 0; k < 3; ++k) {
      c[2][k] = e1 > e2 ? (2 * c[0][k] + c[1][k]) / 3 : (c[0][k] + c[1][k]) / 2;
      c[3][k] = e1 > e2 ? (c[0][k] + 2 * c[1][k]) / 3 : 0;
    }
    for (int p = 0; p < 16; ++p) {
      const int s = (ix >> (2 * p)) & 3;
      const uint8_t *px = rgb + ((size_t)(4 * by + p / 4) * width + 4 * bx + p % 4) * 3;
      for (int k = 0; k < 3; ++k) {
        const int d = (int)px[k] - c[s][k];
        acc += (unsigned long long)(d * d);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(sse, acc);
}

}  // namespace mptc
