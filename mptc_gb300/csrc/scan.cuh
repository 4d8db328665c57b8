// Ordered compactions of a frame: the pending list of an inter frame and the
// unique palette.
#pragma once
#include <cstdint>

#include "completion.cuh"

namespace mptc {

// ------------------------------------------------------ ordered compaction --
// Single-pass ordered compactions (decoupled look-back, Merrill & Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", 2016): a CTA
// per tile of kScanTile blocks takes tiles in order from a zeroed counter,
// counts its tile, publishes the count, adds up its predecessors' published
// counts (or the first inclusive prefix among them) and scatters its items
// at the resulting offset. Tile states are 64-bit words, zeroed per frame:
// 0 = not yet published, kTileAgg | v = the tile's count v, kTilePre | v =
// the count of the tile and all tiles before it. A tile reads only tiles
// taken before it by running CTAs, so the look-back always ends; each wait
// is bounded like wait_done.
constexpr int kScanTile = 1024;  // blocks per tile: 256 threads x 4
constexpr uint64_t kTileAgg = 1ull << 62, kTilePre = 2ull << 62;

// Warp 0 of the CTA owning `tile`: publishes `count` and returns (in every
// lane) the sum of the counts of the tiles before it.
__device__ __forceinline__ uint32_t lookback(uint64_t *state, int tile, uint32_t count, uint32_t *status) {
  const int lane = threadIdx.x & 31;
  if (tile == 0) {
    if (lane == 0) st_relaxed(state, kTilePre | count);
    return 0;
  }
  if (lane == 0) st_relaxed(state + tile, kTileAgg | count);
  uint32_t before = 0;
  for (int j = tile - 1;; j -= 32) {
    const int k = j - lane;  // lane l reads the l-th nearest unread predecessor
    uint64_t v = k >= 0 ? ld_relaxed(state + k) : kTilePre;
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; __any_sync(kFull, v == 0); ++it) {
      if (v == 0) v = ld_relaxed(state + k);
      if ((it & 63u) == 63u && (ld_acquire(status) & kDevTimeout || global_ns() - t0 > 1000000000ull)) {
        atomicOr(status, kDevTimeout);
        v = v ? v : kTilePre;  // give up: the result is flagged invalid
      }
    }
    const unsigned pre = __ballot_sync(kFull, (v >> 62) == 2);
    const int stop = pre ? __ffs(pre) - 1 : 31;  // the nearest inclusive prefix ends the look-back
    before += __reduce_add_sync(kFull, lane <= stop ? (uint32_t)v : 0u);
    if (pre) break;
  }
  if (lane == 0) st_relaxed(state + tile, kTilePre | (before + count));
  return before;
}

// CTA-wide exclusive scan of one count per thread (256 threads); returns the
// thread's offset and the CTA total in `total`. Ends with a barrier.
__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t c, uint32_t *s_warp, uint32_t &total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = c;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t v = __shfl_up_sync(kFull, inc, d);
    if (lane >= d) inc += v;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  uint32_t before = 0;
  total = 0;
#pragma unroll
  for (int w = 0; w < 8; ++w) {
    const uint32_t t = s_warp[w];
    before += w < warp ? t : 0u;
    total += t;
  }
  __syncthreads();  // s_warp is reused by the caller
  return before + inc - c;
}

// Inter frames: the blocks the inter pass left open (done == 0) in wavefront
// order, into pending[0 .. *n_pending); for the fixed-point sweeps each open
// block's first estimate is its stb word (cur[idx]) and the first n_flags
// change flags read (1, 0, 0, ...).
__global__ void __launch_bounds__(256) pending_scan_kernel(const uint32_t *__restrict__ order,
                                                           const uint64_t *__restrict__ done,
                                                           const uint64_t *__restrict__ stb, int n, int ntiles,
                                                           uint64_t *state, uint32_t *claim,
                                                           uint32_t *__restrict__ pending,
                                                           uint32_t *__restrict__ n_pending,
                                                           uint32_t *__restrict__ cur, uint32_t *__restrict__ changed,
                                                           int n_flags, uint32_t *status) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[8], s_before;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(claim, 1u);
  __syncthreads();
  const int tile = s_tile, i0 = tile * kScanTile + 4 * threadIdx.x;
  uint32_t blk[4];
  unsigned open = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + q;
    blk[q] = i < n ? __ldg(order + i) : 0u;
    if (i < n && __ldcg(done + blk[q]) == 0ull) open |= 1u << q;
  }
  uint32_t total;
  uint32_t off = cta_exclusive_scan(__popc(open), s_warp, total);
  if (threadIdx.x < 32) {
    const uint32_t b = lookback(state, tile, total, status);
    if (threadIdx.x == 0) s_before = b;
  }
  __syncthreads();
  off += s_before;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if ((open >> q) & 1u) {
      pending[off++] = blk[q];
      cur[blk[q]] = (uint32_t)(__ldg(stb + blk[q]) >> 32);
    }
  if (tile == ntiles - 1 && threadIdx.x == 0) *n_pending = s_before + total;
  if (tile == 0)
    for (int f = threadIdx.x; f < n_flags; f += blockDim.x) changed[f] = f == 0 ? 1u : 0u;
}

// ----------------------------------------------------------------- unique --
// The unique palette lists the stb interp of every unaccepted block in raster
// order (codec/dxt_image.cpp:953-954), compacted in one pass; the same pass
// counts the frame's inter, intra and unique blocks into stats[0..2].
__global__ void __launch_bounds__(256) unique_scan_kernel(const uint16_t *__restrict__ motion,
                                                          const uint64_t *__restrict__ stb, int nblk, int ntiles,
                                                          uint64_t *state, uint32_t *claim,
                                                          uint32_t *__restrict__ unique,
                                                          uint32_t *__restrict__ n_unique,
                                                          uint32_t *__restrict__ stats, uint32_t *status) {
  __shared__ int s_tile;
  __shared__ uint32_t s_warp[8], s_before;
  if (threadIdx.x == 0) s_tile = (int)atomicAdd(claim, 1u);
  __syncthreads();
  const int tile = s_tile, i0 = tile * kScanTile + 4 * threadIdx.x;
  unsigned uq = 0;
  int ni = 0, na = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int i = i0 + q;
    if (i < nblk) {
      const uint16_t m = motion[i];
      if (m == 0xFFFFu)
        uq |= 1u << q;
      else if (m & 0x80u)
        ++ni;
      else
        ++na;
    }
  }
  uint32_t total;
  uint32_t off = cta_exclusive_scan(__popc(uq), s_warp, total);
  ni = __reduce_add_sync(kFull, ni);
  na = __reduce_add_sync(kFull, na);
  if ((threadIdx.x & 31) == 0) {
    if (ni) atomicAdd(stats + 0, (uint32_t)ni);
    if (na) atomicAdd(stats + 1, (uint32_t)na);
  }
  if (threadIdx.x < 32) {
    const uint32_t b = lookback(state, tile, total, status);
    if (threadIdx.x == 0) {
      s_before = b;
      if (total) atomicAdd(stats + 2, total);
    }
  }
  __syncthreads();
  off += s_before;
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if ((uq >> q) & 1u) unique[off++] = (uint32_t)(__ldg(stb + i0 + q) >> 32);
  if (tile == ntiles - 1 && threadIdx.x == 0) *n_unique = s_before + total;
}

}  // namespace mptc
