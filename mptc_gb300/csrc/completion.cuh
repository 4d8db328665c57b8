// Completion words and their bounded waits: the memory-order helpers the
// intra dataflow and the scans use, and the intra wavefront order.
#pragma once
#include <cstdint>

#include "selection.cuh"

namespace mptc {

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Completion words are read and written as single 64-bit words, so
// publishing needs no fence and a waiter needs no second load.
__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t *p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(uint64_t *p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Waits until done[idx] != 0 and returns the word. Gives up after ~1 s, or at
// once when another wait of this launch already gave up (sets kDevTimeout and
// returns 0), so a broken dependency can never hang the GPU: every later wait
// falls through.
__device__ __forceinline__ uint64_t wait_done(const uint64_t *done, size_t idx, uint32_t *status) {
  uint64_t w = ld_relaxed(done + idx);
  if (w) return w;
  const uint64_t t0 = global_ns();
  for (uint32_t it = 0; it < (1u << 24); ++it) {
    if (it >= 256) __nanosleep(64);  // spin first: the awaited block is usually close
    if ((w = ld_relaxed(done + idx)) != 0) return w;
    if ((it & 63u) == 63u) {
      if (ld_acquire(status) & kDevTimeout) return 0;
      if (global_ns() - t0 > 1000000000ull) break;
    }
  }
  atomicOr(status, kDevTimeout);
  return 0;
}

// Wavefront order of the intra dataflow. Block (x, y) reads, in this frame,
// only blocks of rows y-2sa+1 .. y-1 with columns up to x+sa-1 and blocks of
// row y left of x; with t = x + sa*y every such block has a smaller t. Blocks
// are therefore ranked by (t, y): order[rank] = block index. Blocks of equal t
// never read each other.
__global__ void __launch_bounds__(256) wavefront_order_kernel(int bw, int bh, int sa, uint32_t *__restrict__ order) {
  const int n = bw * bh;
  for (int idx = blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += gridDim.x * blockDim.x) {
    const int y = idx / bw, x = idx - y * bw;
    const long long t = (long long)x + (long long)sa * y;
    long long rank = 0;
    for (int yy = 0; yy < bh; ++yy) {  // blocks with t' < t: x' < t - sa*y'
      const long long c = t - (long long)sa * yy;
      if (c <= 0) break;
      rank += c < bw ? c : bw;
    }
    for (int yy = 0; yy < y; ++yy) {  // blocks with t' == t and y' < y
      const long long xp = t - (long long)sa * yy;
      rank += (xp >= 0 && xp < bw);
    }
    order[rank] = (uint32_t)idx;
  }
}

}  // namespace mptc
