// Learned candidate proposal, the search half: window scoring on the
// fifth-generation tensor cores (tcgen05) — block embeddings against the
// TMA-staged embeddings of the previous frame's final blocks, the top-K
// distinct candidates of each block's window kept in registers as the scores
// leave TMEM — then the exact test of the K proposals with the reference's
// selection rule, and the exhaustive search of the blocks none passed.
#pragma once
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

#include "learned_common.cuh"
#include "search.cuh"
#include "tc_sm100.cuh"

namespace mptc {

// ---- window scoring + top-K ------------------------------------------------------
// Tiles of 8 block rows x 16 block columns (M = 128 blocks, one thread and one
// TMEM lane each). The union of their inter windows spans 8 + 2sa - 1 rows and
// 16 + 2sa - 1 <= 32 columns of the previous frame (sa <= 8); it is staged ROWS
// union rows at a time (N = 32 ROWS candidate positions per stage, the
// dictionary slice of a pipeline stage) by a 3-D TMA copy of G viewed as
// [bh][bw][64] bf16, zero-filled outside the frame. The F tile comes by a TMA
// copy of F viewed the same way. Stage s's MMA writes accumulator s % 2, so the
// MMA of stage s+1 and the copy of stage s+2 overlap the reading of stage s.
//
// Each thread then walks its own window in the reference's scan order (rows
// ascending, columns ascending) and keeps the K best scores in registers.
// Equal index words score bit-identically (the same G row against the same F
// row), so a score equal to one already kept is the same word seen before and
// is skipped: the K proposals are K distinct words, each at its first
// position in scan order.
constexpr int kScoreTileW = 16, kScoreTileH = 8, kScoreThreads = 128;

struct ScoreArgs {
  int bw, bh, sa;
  uint16_t *topk;    // n x kMaxK window positions, best first
  uint32_t *status;  // device status word
};

// A launch covers the frames of up to kMaxBatch jobs (the streams of a
// batch, or one): score tiles are numbered across the jobs and CTAs take them
// from one counter. Job j's embeddings are reached through its tensor maps.
struct ScoreBatch {
  int n;
  int tile_end[kMaxBatch];
  ScoreArgs a[kMaxBatch];
  CUtensorMap tmF[kMaxBatch], tmG[kMaxBatch];
  uint32_t *next;  // tile counter (zero before the launch)
};

template <int K>
__device__ __forceinline__ void topk_insert(float (&s)[K], int (&p)[K], float v, int pos) {
  if (!(v > s[K - 1])) return;
#pragma unroll
  for (int j = 0; j < K; ++j)
    if (s[j] == v) return;
  float cv = v;
  int cp = pos;
#pragma unroll
  for (int j = 0; j < K; ++j) {
    if (cv > s[j]) {
      const float ts = s[j];
      const int tp = p[j];
      s[j] = cv;
      p[j] = cp;
      cv = ts;
      cp = tp;
    }
  }
}

// v[j] for a runtime j without indexing the register array (which would put
// it in local memory): a five-level tree of selects.
__device__ __forceinline__ float pick32(const float (&v)[32], int j) {
  float a[16], b[8], c[4], d[2];
#pragma unroll
  for (int i = 0; i < 16; ++i) a[i] = (j & 16) ? v[i + 16] : v[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) b[i] = (j & 8) ? a[i + 8] : a[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) c[i] = (j & 4) ? b[i + 4] : b[i];
#pragma unroll
  for (int i = 0; i < 2; ++i) d[i] = (j & 2) ? c[i + 2] : c[i];
  return (j & 1) ? d[1] : d[0];
}

using tc::kTileBytes;

template <int ROWS>
constexpr size_t score_smem_bytes() {
  return 1024 + kTileBytes + 2 * (size_t)ROWS * 32 * 128 + 128;
}

template <int ROWS, int K>
__global__ void __launch_bounds__(kScoreThreads, 1) score_topk_tc_kernel(const __grid_constant__ ScoreBatch batch) {
  constexpr int N = 32 * ROWS;
  constexpr uint32_t kGBytes = (uint32_t)N * 128u;
  extern __shared__ uint8_t dsm[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(dsm) + 1023) & ~uintptr_t(1023));
  uint8_t *sF = sm;
  uint8_t *sG[2] = {sm + kTileBytes, sm + kTileBytes + kGBytes};
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kTileBytes + 2 * kGBytes);  // F, G0, G1, M0, M1
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 5);
  volatile uint32_t *abort_flag = tslot + 1;
  volatile int *s_tile = reinterpret_cast<volatile int *>(tslot + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  if (tid == 0) {
    for (int i = 0; i < 5; ++i) tc::mbar_init(bar + i, 1);
    *abort_flag = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, 2 * N);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
  const int r = tid >> 4, c = tid & 15;    // this thread's block inside the tile
  const int wr0 = 2 * warp;                // the warp's first tile row; its window rows span wr0 .. wr0 + w2
  const uint32_t idesc = tc::idesc_bf16(128, N);
  // phase parities: bit 0 F, bits 1-2 the G buffers, bits 3-4 the accumulators
  uint32_t phase = 0;
  auto wait = [&](uint64_t *b, int bit) {
    if (!tc::mbar_wait(b, (phase >> bit) & 1u, abort_flag)) *abort_flag = 1;
    phase ^= 1u << bit;
  };
  const int total = batch.tile_end[batch.n - 1];
  for (;;) {
    if (tid == 0) *s_tile = (int)atomicAdd(batch.next, 1u);
    __syncthreads();
    const int gt = *s_tile;
    if (gt >= total || *abort_flag) break;
    int jb = 0;
    while (gt >= batch.tile_end[jb]) ++jb;
    const ScoreArgs &a = batch.a[jb];
    const CUtensorMap *tmF = &batch.tmF[jb], *tmG = &batch.tmG[jb];
    const int tile = gt - (jb ? batch.tile_end[jb - 1] : 0);
    const int sa = a.sa, w2 = 2 * sa, U = kScoreTileH + w2 - 1, nst = (U + ROWS - 1) / ROWS;
    const int tiles_x = (a.bw + kScoreTileW - 1) / kScoreTileW;
    const int ty0 = (tile / tiles_x) * kScoreTileH, tx0 = (tile % tiles_x) * kScoreTileW;
    const int bx = tx0 + c, by = ty0 + r;
    if (tid == 0) {
      tc::mbar_arrive_expect_tx(bar, kTileBytes);
      tc::tma_load_3d(sF, tmF, 0, tx0, ty0, bar);
      for (int s = 0; s < 2 && s < nst; ++s) {
        tc::mbar_arrive_expect_tx(bar + 1 + s, kGBytes);
        tc::tma_load_3d(sG[s], tmG, 0, tx0 - sa, ty0 - sa + s * ROWS, bar + 1 + s);
      }
      wait(bar, 0);
      wait(bar + 1, 1);
      tc::tc_fence_after();
      const uint32_t fa = tc::smem_addr(sF), ga = tc::smem_addr(sG[0]);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(tmem, tc::desc_sw128(fa + 32 * k), tc::desc_sw128(ga + 32 * k), idesc, k > 0);
      tc::mma_commit(bar + 3);
    }
    float ts[K];
    int tp[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
      ts[j] = -3.0e38f;
      tp[j] = -1;
    }
    const bool in_frame = bx < a.bw && by < a.bh;
    // window columns j of the union (relative to the block: j - c in [0, w2))
    // that lie inside the frame: tx0 - sa + j in [0, bw)
    const int jlo = max(c, sa - tx0), jhi = min(c + w2, a.bw - tx0 + sa);
    const uint32_t cols = jhi > jlo ? (0xFFFFFFFFu >> (32 - (jhi - jlo))) << jlo : 0u;
#pragma unroll 1
    for (int s = 0; s < nst; ++s) {
      const int b = s & 1;
      wait(bar + 3 + b, 3 + b);
      tc::tc_fence_after();
      if (tid == 0) {
        if (s + 1 < nst) {
          const int b1 = (s + 1) & 1;
          wait(bar + 1 + b1, 1 + b1);
          tc::tc_fence_after();
          const uint32_t fa = tc::smem_addr(sF), ga = tc::smem_addr(sG[b1]);
#pragma unroll
          for (int k = 0; k < 4; ++k)
            tc::mma_bf16(tmem + (uint32_t)(b1 * N), tc::desc_sw128(fa + 32 * k), tc::desc_sw128(ga + 32 * k), idesc,
                         k > 0);
          tc::mma_commit(bar + 3 + b1);
        }
        if (s + 2 < nst) {  // stage s's MMA is done: its G buffer takes stage s + 2
          tc::mbar_arrive_expect_tx(bar + 1 + b, kGBytes);
          tc::tma_load_3d(sG[b], tmG, 0, tx0 - sa, ty0 - sa + (s + 2) * ROWS, bar + 1 + b);
        }
      }
      // union rows of this stage that meet the warp's window rows
      const int u0 = max(s * ROWS, wr0), u1 = min(s * ROWS + ROWS, wr0 + w2 + 1);
#pragma unroll 1
      for (int ur = u0; ur < u1; ++ur) {
        float v[32];
        tc::tmem_ld32(lane_base + (uint32_t)(b * N + (ur - s * ROWS) * 32), v);
        const int gy = ty0 - sa + ur;
        if (in_frame && ur >= r && ur < r + w2 && gy >= 0 && gy < a.bh) {
          const int prow = (ur - r) * w2 - c;
          // the window's columns scoring above the current K-th best, then
          // the insertions (few once the list is full) in scan order
          const float thr = ts[K - 1];
          uint32_t m = 0;
#pragma unroll
          for (int j = 0; j < 32; ++j) m |= (v[j] > thr ? 1u : 0u) << j;
          m &= cols;
          while (m) {
            const int j = __ffs(m) - 1;
            m &= m - 1;
            topk_insert<K>(ts, tp, pick32(v, j), prow + j);
          }
        }
      }
      tc::tc_fence_before();
      __syncthreads();
    }
    if (in_frame) {
      uint16_t *o = a.topk + ((size_t)by * a.bw + bx) * kMaxK;
#pragma unroll
      for (int j = 0; j < K; ++j) o[j] = tp[j] < 0 ? kNoProposal : (uint16_t)tp[j];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_free(tmem, 2 * N);
  if (tid == 0 && *abort_flag)
    for (int j = 0; j < batch.n; ++j) atomicOr(batch.a[j].status, kDevTimeout);
}

// ---- exact test of the proposals -------------------------------------------------
// A warp tests the K proposals of 32/K blocks at once (lane = block slot x
// proposal). Each proposal is evaluated exactly (refit, snap, validity, error;
// codec/dxt_image.cpp:258-349) and the reference's selection rule
// (codec/dxt_image.cpp:715-774: the first err_diff <= 0 in scan order ends its
// row, a later row's first err_diff < 0 replaces it, otherwise the first
// minimum) runs over the K proposal positions in closed form. A block whose
// selection passes the threshold becomes final with the reference's inter
// motion code; the others are listed for the exhaustive search.
// The frames of up to kMaxBatch jobs per launch: job j owns the block groups
// [group_end[j-1], group_end[j]) (a group: the 32/K blocks of one warp pass).
struct EvalBatch {
  int n;
  int group_end[kMaxBatch];
  SearchParams P[kMaxBatch];
  const uint16_t *topk[kMaxBatch];
  uint32_t *fb_count[kMaxBatch];  // zeroed fallback counter
  uint32_t *fb_list[kMaxBatch];   // room for every block of the frame
};

template <int K, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) learned_eval_kernel(const __grid_constant__ EvalBatch batch) {
  constexpr int BPW = 32 / K;
  __shared__ BlockTab s_tab[WARPS][BPW];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  build_snap_tables(s_snap5, s_snap6);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, slot = lane / K, k = lane % K;
  const int total = batch.group_end[batch.n - 1];
  for (int gg = blockIdx.x * WARPS + warp; gg < total; gg += gridDim.x * WARPS) {
    int jb = 0;
    while (gg >= batch.group_end[jb]) ++jb;
    const SearchParams &P = batch.P[jb];
    const uint16_t *__restrict__ topk = batch.topk[jb];
    const int nblk = P.bw * P.bh, w2 = 2 * P.sa;
    const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
    const int base = (gg - (jb ? batch.group_end[jb - 1] : 0)) * BPW;
    int sumsq = 0;
#pragma unroll
    for (int jj = 0; jj < BPW; ++jj) {
      const int idx = base + jj;
      if (idx < nblk) {
        const int by = idx / P.bw, bx = idx - by * P.bw;
        const int sq = stage_block(s_tab[warp][jj], P.rgb, P.width, bx, by, lane);
        if (jj == slot) sumsq = sq;
      }
    }
    const int idx = base + slot;
    const bool valid = idx < nblk;
    const int by = valid ? idx / P.bw : 0, bx = valid ? idx - by * P.bw : 0;
    const BlockTab &tab = s_tab[warp][slot];
    int e = kInvalid, pos = -1, refit = 0;
    uint32_t cand = 0, eps = 0;
    uint64_t stb = 0;
    if (valid) {
      stb = P.stb[idx];
      const uint16_t p = topk[(size_t)idx * kMaxK + k];
      const int prow = p / w2, pcol = p - prow * w2;
      const int gy = by - P.sa + prow, gx = bx - P.sa + pcol;
      // the scoring kernel lists in-frame window positions only; anything
      // else (a list left from an aborted launch) is ignored, never read
      if (p != kNoProposal && p < w2 * w2 && gy >= 0 && gy < P.bh && gx >= 0 && gx < P.bw) {
        pos = p;
        const size_t nidx = (size_t)gy * P.bw + gx;
        cand = __ldg(prev_hi + 2 * nidx);
        const float4 d = __ldg(P.wdesc + nidx);
        const WeightSums ws{d.x, d.y, d.z, d.w};
        const PixelGroups pg = load_groups(tab);
        e = eval_candidate(tab, pg, s_snap5, s_snap6, cand, ws, (uint32_t)(stb >> 32), P.orig_err[idx], sumsq, eps,
                           refit);
      }
    }
    const int row = pos >= 0 ? pos / w2 : 0;
    // P0: first position with err_diff <= 0
    int k1 = (e != kInvalid && e <= 0) ? pos : 0xFFFF;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k1 = min(k1, __shfl_xor_sync(kFull, k1, o));
    const int r0 = k1 < 0xFFFF ? k1 / w2 : 0x7FFF;
    // the last later row with an err_diff < 0, and its first such position
    int k2 = (e != kInvalid && e < 0 && row > r0) ? (row << 16) | (0xFFFF - pos) : 0;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k2 = max(k2, __shfl_xor_sync(kFull, k2, o));
    // otherwise the first minimum
    int k3 = e != kInvalid ? ((e + 65536) << 12) | pos : 0x7FFFFFFF;
#pragma unroll
    for (int o = K / 2; o > 0; o >>= 1) k3 = min(k3, __shfl_xor_sync(kFull, k3, o));
    int sel = -1, m = kInvalid;
    if (k2 > 0) {
      sel = 0xFFFF - (k2 & 0xFFFF);
      m = 0;
    } else if (k1 < 0xFFFF) {
      sel = k1;
      m = 0;
    } else if (k3 != 0x7FFFFFFF) {
      sel = k3 & 0xFFF;
      m = (k3 >> 12) - 65536;
    }
    const bool accept = sel >= 0 && m <= P.thr;
    if (valid && accept && pos == sel) {
      const uint64_t blk = refit ? ((uint64_t)eps | ((uint64_t)cand << 32)) : stb;
      const int col = sel - row * w2;
      P.final_blk[idx] = blk;
      P.motion[idx] = (uint16_t)((col | 0x80) | ((row | 0x80) << 8));
      P.done[idx] = done_word(blk);
    }
    if (valid && !accept && k == 0) {
      P.done[idx] = 0;
      batch.fb_list[jb][atomicAdd(batch.fb_count[jb], 1u)] = (uint32_t)idx;
    }
    __syncwarp();
  }
}

// The exhaustive inter search (InterBlockSearch, codec/dxt_image.cpp:715-774)
// of the listed blocks, one warp per block.
struct ListBatch {
  int n;
  SearchParams P[kMaxBatch];
  const uint32_t *list[kMaxBatch];
  const uint32_t *count[kMaxBatch];
};

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) inter_list_kernel(const __grid_constant__ ListBatch batch) {
  __shared__ BlockTab s_tab[WARPS];
  __shared__ DedupTab s_dd[WARPS];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  build_snap_tables(s_snap5, s_snap6);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // the jobs' lists one after the other, every warp of the grid on each
  int off = 0;
  for (int jb = 0; jb < batch.n; ++jb) {
  const SearchParams &P = batch.P[jb];
  const uint32_t *__restrict__ list = batch.list[jb];
  const int n = (int)*batch.count[jb];
  const int start = (blockIdx.x * WARPS + warp - off % (gridDim.x * WARPS) + gridDim.x * WARPS) % (gridDim.x * WARPS);
  off += n;
  for (int k = start; k < n; k += gridDim.x * WARPS) {
    const int idx = (int)list[k];
    const int by = idx / P.bw, bx = idx - by * P.bw;
    const int sumsq = stage_block(s_tab[warp], P.rgb, P.width, bx, by, lane);
    const PixelGroups pg = load_groups(s_tab[warp]);
    const uint64_t word = inter_block_search(P, s_tab[warp], s_dd[warp], pg, s_snap5, s_snap6, idx, bx, by,
                                             P.stb[idx], P.orig_err[idx], sumsq, lane);
    if (lane == 0) P.done[idx] = word;
    __syncwarp();
  }
  }
}

// Exact err_diff (the inter search's refit, validity and error of
// codec/dxt_image.cpp:258-349 against the block's own stb error) of C candidate
// index words for each of B listed blocks: err[b * C + c], INT_MAX when the
// refit would swap the endpoints. One warp per block. Labels the training
// examples of the learned proposal with the exhaustive search's own numbers.
constexpr int kErrWarps = 4;
__global__ void __launch_bounds__(kErrWarps * 32) candidate_errors_kernel(
    const uint8_t *__restrict__ rgb, int width, int bw, const uint64_t *__restrict__ stb,
    const uint32_t *__restrict__ blocks, const uint32_t *__restrict__ cands, int B, int C, int *__restrict__ err) {
  __shared__ BlockTab s_tab[kErrWarps];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ float4 s_wk[4];
  build_snap_tables(s_snap5, s_snap6);
  build_weight_table(s_wk);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int b = blockIdx.x * kErrWarps + warp; b < B; b += gridDim.x * kErrWarps) {
    const int idx = (int)blocks[b];
    const int by = idx / bw, bx = idx - by * bw;
    const int sumsq = stage_block(s_tab[warp], rgb, width, bx, by, lane);
    const PixelGroups pg = load_groups(s_tab[warp]);
    const uint64_t sb = stb[idx];
    uint32_t px[16];
    load_block_px(rgb, width, bx, by, px);
    const int orig = block_error_physical(px, sb);
    for (int c = lane; c < C; c += 32) {
      const uint32_t cand = cands[(size_t)b * C + c];
      uint32_t eps = 0;
      int refit = 0;
      err[(size_t)b * C + c] = eval_candidate(s_tab[warp], pg, s_snap5, s_snap6, cand, weight_sums(cand, s_wk),
                                              (uint32_t)(sb >> 32), orig, sumsq, eps, refit);
    }
    __syncwarp();
  }
}

}  // namespace mptc
