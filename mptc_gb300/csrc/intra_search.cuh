// IntraSearch (codec/dxt_image.cpp:652-713): the dataflow over an intra
// frame's blocks and the fixed-point sweeps of an inter frame's open blocks.
#pragma once
#include <cstdint>

#include "completion.cuh"

namespace mptc {

// Per-block cache of evaluated index words for the intra search. Refit and
// error depend only on the block and the word, and a block's causal window
// holds few distinct words (about 33 of 240 positions on the 1080p stream,
// and the word a block waits for last is almost always one of them), so each
// thread first looks its word up: a hit skips the evaluation, which takes the
// refit off the dataflow's critical path and most of the issue load off the
// SMs. Entries: key = word (the block's own word marks an empty bucket, as the
// identity candidate is never evaluated), val = eps << 32 | err_diff written
// once, all ones while the owner is still evaluating (no valid entry has
// eps = 0xFFFFFFFF, since its high half would be q2 < q1 <= 0xFFFF). A thread
// that finds its word still being evaluated, or no free bucket within the
// probe limit, evaluates it itself; results are identical either way.
constexpr int kEvalBuckets = 512;  // power of two, indexed by a 9-bit hash
constexpr int kEvalProbes = 16;
constexpr uint64_t kEvalPending = ~0ull;

template <int NB>
struct EvalCacheN {
  uint32_t key[NB];
  unsigned long long val[NB];
};
using EvalCache = EvalCacheN<kEvalBuckets>;

// Resets a cache with the threads first, first + stride, ... of the CTA.
template <int NB>
__device__ __forceinline__ void eval_cache_reset(EvalCacheN<NB> &c, uint32_t own, int first, int stride) {
  for (int b = first; b < NB; b += stride) {
    c.key[b] = own;
    c.val[b] = kEvalPending;
  }
}

template <int NB>
__device__ __forceinline__ void eval_cache_reset(EvalCacheN<NB> &c, uint32_t own) {
  eval_cache_reset(c, own, threadIdx.x, blockDim.x);
}

// Whether a CTA consults its cache: on content where a window's words are
// all different (noise) lookups never find a repeat and only cost time, so
// after a block in which fewer than a quarter of the threads that looked a word
// up found it already present (evaluated or being evaluated), the cache is
// bypassed for the next 8 blocks, then tried again. All threads update it with
// the same block-wide counts, so it stays CTA-uniform.
struct CacheUse {
  bool on = true;
  int off_left = 0;
  __device__ __forceinline__ void update(int looked, int hits) {
    if (on) {
      if (looked >= 32 && 4 * hits < looked) {
        on = false;
        off_left = 8;
      }
    } else if (--off_left <= 0) {
      on = true;
    }
  }
};

template <int NB>
__device__ __forceinline__ int cached_eval(EvalCacheN<NB> &c, bool use, const BlockTab &tab, const PixelGroups &pg,
                                           const uint8_t *snap5, const uint8_t *snap6, const float4 *wk,
                                           uint32_t cand, uint32_t own, int orig, int sumsq, uint32_t &eps,
                                           int &refit, int &looked, int &hits) {
  constexpr int kBits = NB == 512 ? 9 : NB == 256 ? 8 : NB == 128 ? 7 : 6;
  static_assert(NB == (1 << kBits), "bucket count: a power of two from 64 to 512");
  if (cand == own) {
    eps = 0;
    refit = 0;
    return 0;
  }
  refit = 1;
  uint32_t b = (cand * 2654435761u) >> (32 - kBits);
  int slot = -1;
  for (int probe = 0; use && probe < kEvalProbes; ++probe) {
    const uint32_t k = *(volatile uint32_t *)&c.key[b];
    if (k == cand) {
      const unsigned long long v = *(volatile unsigned long long *)&c.val[b];
      ++looked;
      ++hits;  // the word is a repeat, even if its result is not written yet
      if (v != kEvalPending) {
        eps = (uint32_t)(v >> 32);
        return (int)(uint32_t)v;
      }
      break;  // being evaluated by another thread: evaluate here too
    }
    if (k == own) {
      const uint32_t old = atomicCAS(&c.key[b], own, cand);
      if (old == own) {
        ++looked;
        slot = (int)b;
        break;
      }
      if (old == cand) {
        ++looked;
        ++hits;
        break;
      }
    }
    b = (b + 1) & (NB - 1);
  }
  const WeightSums ws = weight_sums(cand, wk);
  const int e = eval_candidate(tab, pg, snap5, snap6, cand, ws, own, orig, sumsq, eps, refit);
  if (e == kInvalid) eps = 0;
  if (slot >= 0)
    *(volatile unsigned long long *)&c.val[slot] = ((unsigned long long)eps << 32) | (uint32_t)e;
  return e;
}

// Selection and output of one block of the intra search: the CTA reduces
// the threads' statistics, then the thread holding the selected statistic
// writes the final block and motion code (and, when `publish`, the block's
// completion word). Returns the block's completion word in that thread and 0
// in the others. Ends with a barrier.
template <int THREADS>
__device__ __forceinline__ uint64_t publish_intra(const SearchParams &P, const ThreadSel &ts, CtaReduce<THREADS> &red,
                                                  int idx, uint64_t stb, int w2, int tid, bool publish) {
  int m, pick;
  const int sel = cta_select<THREADS>(ts, red, w2, m, pick);
  const bool accept = sel >= 0 && m <= P.thr;
  // the thread whose statistics hold the selected position (its own position,
  // or, in the later sweeps, statistics merged from the first)
  const bool holder = pick == 0   ? ts.le0_pos == sel
                      : pick == 1 ? ts.neg_key >= 0 && 0xFFFF - (ts.neg_key & 0xFFFF) == sel
                                  : ts.min_e == m && ts.min_pos == sel;
  uint64_t out = 0;
  if (accept ? holder : tid == 0) {
    uint16_t code = 0xFFFFu;
    uint64_t blk = stb;
    if (accept) {
      const SelPick &pk = pick == 0 ? ts.le0 : (pick == 1 ? ts.neg : ts.mn);
      const int row = sel / w2, col = sel - row * w2;
      code = (uint16_t)((w2 - 1 - col) | ((w2 - 1 - row) << 8));
      if (pk.refit) blk = (uint64_t)pk.eps | ((uint64_t)pk.cand << 32);
    }
    P.final_blk[idx] = blk;
    P.motion[idx] = code;
    if (publish) st_relaxed(P.done + idx, done_word(blk));  // waiters read only this word
    out = done_word(blk);
  }
  __syncthreads();
  return out;
}

// IntraSearch, codec/dxt_image.cpp:652-713, as a dataflow over the blocks
// still pending after the inter pass, in wavefront order: rows j = by ..
// by-2sa+1 (descending), columns i = bx+sa-1 .. bx-sa (descending), skipping
// j == by && i >= bx; motion (i-bx+sa, j-by+2sa-1). Unaccepted blocks are
// unique: motion (255,255), final = stb block.
// One CTA per block, one window position per thread and round; CTAs claim
// pending blocks one at a time from P.work, so every block a CTA waits on was
// claimed earlier by a running CTA and the dataflow cannot deadlock. At most
// 64 registers per thread: the stream calls run this kernel beside the inter
// kernels of other frames, which then keep more CTAs per SM.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 4) intra_search_kernel(SearchParams P, const uint32_t *__restrict__ pending,
                                                               const uint32_t *__restrict__ n_pending_dev,
                                                               int n_pending_host,
                                                               const uint32_t *__restrict__ run_flag = nullptr) {
  if (run_flag && __ldcg(run_flag) == 0u) return;  // the sweeps below converged
  __shared__ BlockTab s_tab;
  __shared__ EvalCache s_cache;
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ float4 s_wk[4];
  __shared__ int s_red[2 * (THREADS / 32)];
  __shared__ int s_claim, s_sumsq;
  build_snap_tables(s_snap5, s_snap6);
  build_weight_table(s_wk);
  CtaReduce<THREADS> red{s_red, 0};
  CacheUse cache;
  const int tid = threadIdx.x, lane = tid & 31;
  const int n_pend = n_pending_host >= 0 ? n_pending_host : (int)__ldcg(n_pending_dev);
  const int w2 = 2 * P.sa, npos = w2 * w2;
  while (true) {
    if (tid == 0) s_claim = (int)atomicAdd(P.work, 1u);
    __syncthreads();
    const int k = s_claim;
    if (k >= n_pend) break;
    const int idx = (int)__ldcg(pending + k);
    const int by = idx / P.bw, bx = idx - by * P.bw;
    const uint64_t stb = __ldg(P.stb + idx);
    const uint32_t own = (uint32_t)(stb >> 32);
    eval_cache_reset(s_cache, own);
    if (tid < 32) {
      const int sq = stage_block(s_tab, P.rgb, P.width, bx, by, lane);
      if (tid == 0) s_sumsq = sq;
    }
    __syncthreads();
    const int orig = __ldg(P.orig_err + idx);
    const int sumsq = s_sumsq;
    const PixelGroups pg = load_groups(s_tab);
    ThreadSel ts;
    int looked = 0, hits = 0;
    for (int base = 0; base < npos; base += THREADS) {
      const int pos = base + tid;
      const int row = pos / w2, col = pos - row * w2;
      const int j = by - row, i = bx + P.sa - 1 - col;
      if (pos < npos && i >= 0 && j >= 0 && i < P.bw && j < P.bh && !(j == by && i >= bx)) {
        const size_t nidx = (size_t)j * P.bw + i;
        const uint64_t w = wait_done(P.done, nidx, P.status);
        if (w) {
          const uint32_t cand = (uint32_t)w;
          uint32_t eps = 0;
          int refit = 0;
          const int e = cached_eval(s_cache, cache.on, s_tab, pg, s_snap5, s_snap6, s_wk, cand, own, orig, sumsq,
                                    eps, refit, looked, hits);
          ts.add(pos, row, e, cand, eps, refit);
        }
      }
    }
    publish_intra(P, ts, red, idx, stb, w2, tid, true);
    cache.update(__syncthreads_count(looked > 0), __syncthreads_count(hits > 0));
  }
}

// Inter frames: the intra search of the blocks the inter pass left open, as
// a fixed-point iteration instead of a dataflow. Each open block's result
// depends only on the final index words of earlier blocks (causal order), so
// the system x_b = F_b(x_earlier) has exactly one solution, and it is the only
// fixed point. Sweep k evaluates every open block from the estimates of sweep
// k-1 (cur; open blocks start at their stb word, i.e. as if unique, which most
// open blocks on inter frames end up as) and writes its result (final block,
// motion code, next estimate); when no estimate changed, the outputs of that
// sweep are the reference's. A sweep runs only while the previous one changed
// something (changed[k] != 0); if the last sweep still changed something, the
// dataflow kernel recomputes the open blocks exactly. Sweeps have no waits:
// every open block is independent within a sweep.
// Positions whose block is final (done) give the same results in every sweep
// (on the 1080p stream 85% of an open block's positions): the first sweep
// stores each warp's statistics over them (part, for the first part_cap open
// blocks), and the later sweeps evaluate only the positions whose block is
// open, merging the stored statistics in. A later sweep also skips a block
// whose open window blocks all kept the estimates the previous sweep read
// (cur against before): its result, already written, cannot change.
template <int THREADS>
__global__ void __launch_bounds__(THREADS, 3) intra_sweep_kernel(SearchParams P, const uint32_t *__restrict__ pending,
                                                              const uint32_t *__restrict__ n_pending_dev,
                                                              const uint32_t *__restrict__ cur,
                                                              const uint32_t *__restrict__ before,
                                                              uint32_t *__restrict__ next,
                                                              const uint32_t *__restrict__ changed_in,
                                                              uint32_t *__restrict__ changed_out,
                                                              SweepPartial *__restrict__ part, int part_cap,
                                                              bool first) {
  if (__ldcg(changed_in) == 0u) return;
  __shared__ BlockTab s_tab;
  __shared__ EvalCache s_cache;
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ float4 s_wk[4];
  __shared__ int s_red[2 * (THREADS / 32)];
  __shared__ int s_sumsq;
  build_snap_tables(s_snap5, s_snap6);
  build_weight_table(s_wk);
  CtaReduce<THREADS> red{s_red, 0};
  CacheUse cache;
  const int tid = threadIdx.x, lane = tid & 31;
  const int n_pend = (int)__ldcg(n_pending_dev);
  const int w2 = 2 * P.sa, npos = w2 * w2;
  for (int k = blockIdx.x; k < n_pend; k += gridDim.x) {
    const int idx = (int)__ldcg(pending + k);
    const int by = idx / P.bw, bx = idx - by * P.bw;
    if (!first) {  // any open window block with a new estimate?
      bool moved = false;
      for (int pos = tid; pos < npos; pos += THREADS) {
        const int row = pos / w2, col = pos - row * w2;
        const int j = by - row, i = bx + P.sa - 1 - col;
        if (i >= 0 && j >= 0 && i < P.bw && j < P.bh && !(j == by && i >= bx)) {
          const size_t nidx = (size_t)j * P.bw + i;
          if (__ldcg(P.done + nidx) == 0ull && __ldcg(cur + nidx) != __ldcg(before + nidx)) moved = true;
        }
      }
      if (!__syncthreads_or(moved)) {
        if (tid == 0) next[idx] = __ldcg(cur + idx);
        continue;
      }
    }
    const uint64_t stb = __ldg(P.stb + idx);
    const uint32_t own = (uint32_t)(stb >> 32);
    eval_cache_reset(s_cache, own);
    if (tid < 32) {
      const int sq = stage_block(s_tab, P.rgb, P.width, bx, by, lane);
      if (tid == 0) s_sumsq = sq;
    }
    __syncthreads();
    const int orig = __ldg(P.orig_err + idx);
    const int sumsq = s_sumsq;
    const PixelGroups pg = load_groups(s_tab);
    ThreadSel ts, tf;  // all positions; (first sweep) those of final blocks
    int looked = 0, hits = 0;
    const bool stored = k < part_cap;
    SweepPartial *wp = part + ((size_t)k * (THREADS / 32) + (tid >> 5));
    for (int base = 0; base < npos; base += THREADS) {
      const int pos = base + tid;
      const int row = pos / w2, col = pos - row * w2;
      const int j = by - row, i = bx + P.sa - 1 - col;
      if (pos < npos && i >= 0 && j >= 0 && i < P.bw && j < P.bh && !(j == by && i >= bx)) {
        const size_t nidx = (size_t)j * P.bw + i;
        const uint64_t w = __ldcg(P.done + nidx);
        if (w && !first && stored) continue;  // in the stored statistics
        const uint32_t cand = w ? (uint32_t)w : __ldcg(cur + nidx);
        uint32_t eps = 0;
        int refit = 0;
        const int e = cached_eval(s_cache, cache.on, s_tab, pg, s_snap5, s_snap6, s_wk, cand, own, orig, sumsq,
                                  eps, refit, looked, hits);
        ts.add(pos, row, e, cand, eps, refit);
        if (w) tf.add(pos, row, e, cand, eps, refit);
      }
    }
    if (first && stored) warp_store_partial(tf, wp, lane);
    // after the lane's own positions, which add() expects in scan order
    if (!first && stored && lane == 0) ts.merge(*wp);
    const uint64_t w = publish_intra(P, ts, red, idx, stb, w2, tid, false);
    cache.update(__syncthreads_count(looked > 0), __syncthreads_count(hits > 0));
    if (w != 0) {  // the thread that wrote the result
      const uint32_t x = (uint32_t)w;
      next[idx] = x;
      if (x != __ldcg(cur + idx)) atomicOr(changed_out, 1u);
    }
  }
}

}  // namespace mptc
