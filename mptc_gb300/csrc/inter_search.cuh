// InterBlockSearch (codec/dxt_image.cpp:715-774): the one-block search, the
// run search for sa <= 8 and the overflow search of noisy runs.
#pragma once
#include <cstdint>

#include "completion.cuh"

namespace mptc {

// ------------------------------------------------------------------ inter --
// InterBlockSearch, codec/dxt_image.cpp:715-774: rows j = by-sa .. by+sa-1,
// columns i = bx-sa .. bx+sa-1 (both ascending); motion (i-bx+sa)|0x80,
// (j-by+sa)|0x80. Accepted blocks become final here; the others are left for
// the intra pass (done = 0). One warp per block.
// Refit, validity and error depend only on the block and the candidate index
// word, so positions holding equal words get equal results, and each distinct
// word of the window is evaluated once: on smooth content a 16x16 window holds
// few distinct words (about 15% of the positions on the 1080p test stream).
// Per span of up to 256 positions (the whole window for sa <= 8): the warp
// loads the candidates, inserts the distinct words other than the block's own
// into a shared hash table (open addressing with as many buckets as positions,
// so an insertion always ends; own word = empty marker: the identity
// candidate needs no refit), evaluates the distinct words 32 at a time and
// records each position's result in the lane's selection statistics
// (LaneSel); warp_select then applies the reference's selection rule.
constexpr int kDedupSpan = 256;     // positions per dedup span (8 chunks)
constexpr int kDedupBuckets = 256;  // hash buckets (a span has <= 256 distinct words)

struct DedupTab {
  uint32_t key[kDedupBuckets];  // index word, or the block's own word when empty
  uint16_t slot[kDedupBuckets];
  uint32_t nidx[kDedupSpan];    // a window block holding each distinct word
  uint16_t bkt[kDedupSpan];     // the bucket holding each distinct word
  int e[kDedupSpan];
  uint32_t eps[kDedupSpan];
};

__device__ __forceinline__ uint32_t dedup_hash(uint32_t v) { return (v * 2654435761u) >> 24; }

// The exhaustive inter search of block idx by one warp: every distinct window
// word evaluated once, the reference's selection, the final block and motion
// code written when accepted. Returns the block's completion word (0: left
// open for the intra pass), the same in every lane.
__device__ __forceinline__ uint64_t inter_block_search(const SearchParams &P, const BlockTab &tab, DedupTab &dd,
                                                       const PixelGroups &pg, const uint8_t *s_snap5,
                                                       const uint8_t *s_snap6, int idx, int bx, int by,
                                                       uint64_t stb, int orig, int sumsq, int lane) {
  const uint32_t own = (uint32_t)(stb >> 32);
  const unsigned lt_mask = (1u << lane) - 1u;
  const int w2 = 2 * P.sa, npos = w2 * w2;
  // pos / w2 as one multiply-high: exact for pos < 2^16 and w2 <= 126
  const uint32_t w2_magic = 0xFFFFFFFFu / (uint32_t)w2 + 1u;
  const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
  LaneSel ls_;
  int ls[8];  // slot of each of the lane's positions in the current span
  for (int span = 0; span < npos; span += kDedupSpan) {
    for (int b = lane; b < kDedupBuckets; b += 32) dd.key[b] = own;
    __syncwarp();
    uint32_t lc[8], ln[8];
    unsigned valid = 0;
    int nuniq = 0;
    // all candidate loads of the span first, so their latencies overlap
    {
      const int pos0 = span + lane;
      int row = pos0 / w2, col = pos0 - row * w2;
      const int drow = 32 / w2, dcol = 32 - drow * w2;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const int pos = pos0 + 32 * c;
        const int j = by - P.sa + row, i = bx - P.sa + col;
        uint32_t cand = own, nidx = 0;
        if (pos < npos && i >= 0 && j >= 0 && i < P.bw && j < P.bh) {
          nidx = (uint32_t)(j * P.bw + i);
          cand = __ldg(prev_hi + 2 * (size_t)nidx);
          valid |= 1u << c;
        }
        lc[c] = cand;
        ln[c] = nidx;
        row += drow;
        col += dcol;
        if (col >= w2) {
          col -= w2;
          ++row;
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const uint32_t cand = lc[c], nidx = ln[c];
      const bool need = cand != own;  // invalid positions hold `own` too
      const unsigned peers = __match_any_sync(kFull, cand);
      const int leader = __ffs(peers) - 1;
      uint32_t b = dedup_hash(cand);
      bool is_new = false, found = false;
      if (need && lane == leader) {
        for (int probe = 0; probe < kDedupBuckets; ++probe) {
          const uint32_t old = atomicCAS(&dd.key[b], own, cand);
          if (old == own) {
            is_new = true;
            break;
          }
          if (old == cand) {
            found = true;
            break;
          }
          b = (b + 1) & (kDedupBuckets - 1);
        }
      }
      const unsigned newm = __ballot_sync(kFull, is_new);
      int slot = -1;
      if (is_new) {
        slot = nuniq + __popc(newm & lt_mask);
        dd.slot[b] = (uint16_t)slot;
        dd.nidx[slot] = nidx;
        dd.bkt[slot] = (uint16_t)b;
      } else if (found) {
        slot = dd.slot[b];  // inserted by an earlier chunk of this span
      }
      ls[c] = __shfl_sync(kFull, slot, leader);
      nuniq += __popc(newm);
      __syncwarp();  // this chunk's slot writes land before later chunks read them
    }
    __syncwarp();
    for (int k = lane; k < nuniq; k += 32) {
      const uint32_t nidx = dd.nidx[k], cand = dd.key[dd.bkt[k]];
      const float4 d = __ldg(P.wdesc + nidx);
      const WeightSums ws{d.x, d.y, d.z, d.w};
      uint32_t eps = 0;
      int refit = 0;
      dd.e[k] = eval_candidate(tab, pg, s_snap5, s_snap6, cand, ws, own, orig, sumsq, eps, refit);
      dd.eps[k] = eps;
    }
    __syncwarp();
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      if ((valid >> c) & 1u) {
        const int pos = span + 32 * c + lane;
        ls_.add(pos, (int)__umulhi((uint32_t)pos, w2_magic), lc[c] == own ? 0 : dd.e[ls[c]]);
      }
    }
    __syncwarp();
  }
  int m;
  const int sel = warp_select(ls_, w2, m);
  const bool accept = sel >= 0 && m <= P.thr;  // warp-uniform
  uint64_t word = 0;
  if (accept) {
    // the selected position's index word and refit: the owning lane looks
    // them up (one span; slot -1 marks the block's own word) or evaluates the
    // word again (several spans)
    const int owner = sel & 31;
    uint64_t blk = 0;
    if (lane == owner) {
      if (npos <= kDedupSpan) {
        const int c = sel >> 5;
        int slot = -1;
#pragma unroll
        for (int cc = 0; cc < 8; ++cc)
          if (cc == c) slot = ls[cc];
        blk = slot < 0 ? stb : ((uint64_t)dd.eps[slot] | ((uint64_t)dd.key[dd.bkt[slot]] << 32));
      } else {
        const int i = bx - P.sa + sel % w2, j = by - P.sa + sel / w2;
        const uint32_t cand = __ldg(prev_hi + 2 * (size_t)(j * P.bw + i));
        if (cand == own) {
          blk = stb;
        } else {
          const float4 d = __ldg(P.wdesc + (size_t)(j * P.bw + i));
          const WeightSums ws{d.x, d.y, d.z, d.w};
          uint32_t eps = 0;
          int refit = 0;
          eval_candidate(tab, pg, s_snap5, s_snap6, cand, ws, own, orig, sumsq, eps, refit);
          blk = (uint64_t)eps | ((uint64_t)cand << 32);
        }
      }
      const int row = sel / w2, col = sel - row * w2;
      P.final_blk[idx] = blk;
      P.motion[idx] = (uint16_t)((col | 0x80) | ((row | 0x80) << 8));
      word = done_word(blk);
    }
    word = __shfl_sync(kFull, word, owner);
  }
  return word;
}

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32, 32 / WARPS) inter_dedup_kernel(SearchParams P) {
  __shared__ BlockTab s_tab[WARPS];
  __shared__ DedupTab s_dd[WARPS];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  build_snap_tables(s_snap5, s_snap6);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  BlockTab &tab = s_tab[warp];
  const int nblk = P.bw * P.bh;
  for (int idx = blockIdx.x * WARPS + warp; idx < nblk; idx += gridDim.x * WARPS) {
    const int by = idx / P.bw, bx = idx - by * P.bw;
    const int sumsq = stage_block(tab, P.rgb, P.width, bx, by, lane);
    const PixelGroups pg = load_groups(tab);
    const uint64_t word = inter_block_search(P, tab, s_dd[warp], pg, s_snap5, s_snap6, idx, bx, by, P.stb[idx],
                                             P.orig_err[idx], sumsq, lane);
    if (lane == 0) P.done[idx] = word;
    __syncwarp();
  }
}

// ------------------------------------------------------------ inter runs --
// The same search for sa <= 8, one warp per run of RUN horizontally adjacent
// blocks of a row. Their windows share all rows and overlap in all but
// RUN - 1 columns, so the warp deduplicates the union of the windows (w2 rows
// by w2 + RUN - 1 columns) once, recording for each distinct word the union
// columns where it occurs (a bit mask); block k of the run then evaluates the
// distinct words whose mask meets its columns k .. k + w2 - 1 and selects
// over its own positions, exactly as the one-block search does.
// The hash table's empty marker is the first block's own word, which keeps a
// dedicated slot 0 outside the table; out-of-frame positions carry the marker
// and no column bit. The blocks of a run whose union holds more than
// kRunWords distinct words (noisy content) are appended to a list that
// inter_overflow_kernel searches afterwards with a CTA per block: those runs
// cost several times a smooth one and, kept in one warp, would hold their SM
// long after the other warps finished.
constexpr int kRunWords = 128;  // distinct union words handled by the run table
constexpr int kRunBuckets = 256;

template <int RUN>
struct RunTab {
  static constexpr int kCols = 16 + RUN - 1;  // union columns at sa = 8
  static constexpr int kPos = 16 * kCols;     // union positions at sa = 8
  static constexpr int kChunks = (kPos + 31) / 32;
  // the marker, kRunWords words, and the up to 32 further new words of the
  // chunk that crosses the limit
  static constexpr int kSlots = 1 + kRunWords + 32;
  uint32_t bkey[kRunBuckets];  // word, or the marker when empty
  uint8_t bslot[kRunBuckets];
  uint8_t pslot[kChunks * 32];  // slot of each union position
  uint8_t list[kSlots];         // slots evaluated for the current block
  uint16_t upos[kSlots];        // a union position holding the word
  uint32_t key[kSlots];
  uint32_t cols[kSlots];        // union columns holding the word (bit per column)
  // the union's words while they are inserted, then each slot's err_diff
  // (kSlots entries and the out-of-frame sentinel's kInvalid) and endpoint
  // word (next kSlots) for the current block
  static constexpr int kSentinel = kSlots;  // slot of out-of-frame positions
  static constexpr int kEval = 2 * kSlots + 1 > kChunks * 32 ? 2 * kSlots + 1 : kChunks * 32;
  uint32_t ev[kEval];
  __device__ __forceinline__ uint32_t *ucand() { return ev; }
  __device__ __forceinline__ int *e() { return reinterpret_cast<int *>(ev); }
  __device__ __forceinline__ uint32_t *eps() { return ev + kSlots + 1; }
};

// SA: the search area when fixed at compile time (its constants fold), 0 to
// read it from P. A persistent grid: each warp takes the next unit of work
// from *next_run (zero at launch), which keeps all warps busy to the end
// although runs differ in cost. The units are the runs of the first
// bh - tail_rows rows, then the blocks of the last tail_rows rows one by one
// (runs of one block), so that the work left when the queue empties is short.
template <int WARPS, int RUN, int SA>
__global__ void __launch_bounds__(WARPS * 32, 32 / WARPS)
    inter_run_kernel(SearchParams P, uint32_t *next_run, int tail_rows, uint32_t *ovf_count, uint32_t *ovf_list) {
  using Tab = RunTab<RUN>;
  static_assert(Tab::kCols <= 32, "union columns must fit a 32-bit mask");
  static_assert(sizeof(Tab) <= sizeof(DedupTab), "the one-block kernel's footprint: 32 warps per SM");
  static_assert(Tab::kSentinel <= 255 && Tab::kSlots - 1 <= kRunBuckets, "slots are bytes; buckets hold the words");
  __shared__ BlockTab s_tab[WARPS];
  __shared__ Tab s_run[WARPS];
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  build_snap_tables(s_snap5, s_snap6);
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  BlockTab &tab = s_tab[warp];
  Tab &rt = s_run[warp];
  const unsigned lt_mask = (1u << lane) - 1u;
  const int sa = SA ? SA : P.sa;
  const int w2 = 2 * sa, ucols = w2 + RUN - 1, upos = w2 * ucols;
  // the lane's first union position (row, column) and the step to its next
  const int urow0 = lane / ucols, ucol0 = lane - urow0 * ucols;
  const int drow = 32 / ucols, dcol = 32 - drow * ucols;
  // pos / w2 and u / ucols as multiplies-high: exact below 2^16 for divisors <= 126
  const uint32_t w2_magic = 0xFFFFFFFFu / (uint32_t)w2 + 1u, uc_magic = 0xFFFFFFFFu / (uint32_t)ucols + 1u;
  const uint32_t wmask = (1u << w2) - 1u;
  // the lane's first window position (row, column) and the step to its next
  const int npos = w2 * w2, prow0 = lane / w2, pcol0 = lane - prow0 * w2;
  const int pdrow = 32 / w2, pdcol = 32 - pdrow * w2;
  const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
  const int runs_per_row = (P.bw + RUN - 1) / RUN, main_rows = P.bh - tail_rows;
  const int nmain = runs_per_row * main_rows, nunits = nmain + tail_rows * P.bw;
  for (;;) {
    int unit = 0;
    if (lane == 0) unit = (int)atomicAdd(next_run, 1u);
    unit = __shfl_sync(kFull, unit, 0);
    if (unit >= nunits) break;
    int by, bx0, nb;
    if (unit < nmain) {
      by = unit / runs_per_row;
      bx0 = (unit - by * runs_per_row) * RUN;
      nb = min(RUN, P.bw - bx0);
    } else {
      const int b = main_rows * P.bw + (unit - nmain);
      by = b / P.bw;
      bx0 = b - by * P.bw;
      nb = 1;
    }
    const int j0 = by - sa, i0 = bx0 - sa, ucols_used = w2 + nb - 1;
    const uint32_t marker = (uint32_t)(P.stb[by * P.bw + bx0] >> 32);
    for (int b = lane; b < kRunBuckets; b += 32) rt.bkey[b] = marker;
    if (lane == 0) {
      rt.key[0] = marker;
      rt.cols[0] = 0;
    }
    __syncwarp();
    // the union's words, all loads first so their latencies overlap
    uint32_t *ucand = rt.ucand();
    unsigned valid = 0;
    {
      int urow = urow0, ucol = ucol0;
#pragma unroll
      for (int c = 0; c < Tab::kChunks; ++c) {
        const int j = j0 + urow, i = i0 + ucol;
        uint32_t cand = marker;
        if (32 * c + lane < upos && ucol < ucols_used && i >= 0 && j >= 0 && i < P.bw && j < P.bh) {
          cand = __ldg(prev_hi + 2 * (size_t)(j * P.bw + i));
          valid |= 1u << c;
        }
        ucand[32 * c + lane] = cand;
        urow += drow;
        ucol += dcol;
        if (ucol >= ucols) {
          ucol -= ucols;
          ++urow;
        }
      }
    }
    __syncwarp();
    int nuniq = 1;
    bool overflow = false;
    {
      int ucol = ucol0;
#pragma unroll 1
      for (int c = 0; c < Tab::kChunks; ++c) {
        const uint32_t cand = ucand[32 * c + lane];
        const bool ok = (valid >> c) & 1u;
        const unsigned peers = __match_any_sync(kFull, cand);
        const int leader = __ffs(peers) - 1;
        const uint32_t colbits = __reduce_or_sync(peers, ok ? 1u << ucol : 0u);
        const unsigned okm = __ballot_sync(kFull, ok);
        uint32_t b = 0;
        int slot = 0;
        bool is_new = false;
        if (lane == leader && colbits) {  // groups of out-of-frame positions only are skipped
          if (cand == marker) {
            if (rt.cols[0] == 0) rt.upos[0] = (uint16_t)(32 * c + __ffs(peers & okm) - 1);
            rt.cols[0] |= colbits;
          } else {
            b = dedup_hash(cand);
            for (int probe = 0; probe < kRunBuckets; ++probe) {
              const uint32_t old = atomicCAS(&rt.bkey[b], marker, cand);
              if (old == marker) {
                is_new = true;
                break;
              }
              if (old == cand) {
                slot = rt.bslot[b];  // inserted by an earlier chunk
                rt.cols[slot] |= colbits;
                break;
              }
              b = (b + 1) & (kRunBuckets - 1);
            }
          }
        }
        const unsigned newm = __ballot_sync(kFull, is_new);
        if (is_new) {  // the leader's own position holds the word
          slot = nuniq + __popc(newm & lt_mask);
          rt.bslot[b] = (uint8_t)slot;
          rt.key[slot] = cand;
          rt.cols[slot] = colbits;
          rt.upos[slot] = (uint16_t)(32 * c + lane);
        }
        slot = __shfl_sync(kFull, slot, leader);
        rt.pslot[32 * c + lane] = (uint8_t)(ok ? slot : Tab::kSentinel);
        nuniq += __popc(newm);
        __syncwarp();  // this chunk's slot writes land before later chunks read them
        if (nuniq > 1 + kRunWords) {  // warp-uniform
          overflow = true;
          break;
        }
        ucol += dcol;
        if (ucol >= ucols) ucol -= ucols;
      }
    }
    if (overflow) {
      if (lane == 0) {
        const uint32_t at = atomicAdd(ovf_count, (uint32_t)nb);
        for (int k = 0; k < nb; ++k) ovf_list[at + k] = (uint32_t)(by * P.bw + bx0 + k);
      }
      continue;
    }
    if (lane == 0) rt.e()[Tab::kSentinel] = kInvalid;
    for (int k = 0; k < nb; ++k) {
      const int bx = bx0 + k, idx = by * P.bw + bx;
      const uint64_t stb = P.stb[idx];
      const uint32_t own = (uint32_t)(stb >> 32);
      const int orig = P.orig_err[idx];
      const int sumsq = stage_block(tab, P.rgb, P.width, bx, by, lane);
      const PixelGroups pg = load_groups(tab);
      // the distinct words of this block's window; its own word needs no refit
      const uint32_t win = wmask << k;
      int nl = 0;
      for (int s0 = 0; s0 < nuniq; s0 += 32) {
        const int s = s0 + lane;
        bool take = false;
        if (s < nuniq && (rt.cols[s] & win)) {
          if (rt.key[s] == own)
            rt.e()[s] = 0;
          else
            take = true;
        }
        const unsigned tm = __ballot_sync(kFull, take);
        if (take) rt.list[nl + __popc(tm & lt_mask)] = (uint8_t)s;
        nl += __popc(tm);
      }
      __syncwarp();
      for (int q = lane; q < nl; q += 32) {
        const int s = rt.list[q];
        const int u = rt.upos[s];
        const int ur = (int)__umulhi((uint32_t)u, uc_magic);
        const float4 d = __ldg(P.wdesc + (size_t)((j0 + ur) * P.bw + i0 + u - ur * ucols));
        const WeightSums ws{d.x, d.y, d.z, d.w};
        uint32_t eps = 0;
        int refit = 0;
        rt.e()[s] = eval_candidate(tab, pg, s_snap5, s_snap6, rt.key[s], ws, own, orig, sumsq, eps, refit);
        rt.eps()[s] = eps;
      }
      __syncwarp();
      // the block's positions in scan order, 32 at a time
      LaneSel sel;
      {
        int row = prow0, col = pcol0;
#pragma unroll 1
        for (int pos = lane; pos < npos; pos += 32) {
          sel.add(pos, row, rt.e()[rt.pslot[row * ucols + col + k]]);
          row += pdrow;
          col += pdcol;
          if (col >= w2) {
            col -= w2;
            ++row;
          }
        }
      }
      int m;
      const int sp = warp_select(sel, w2, m);
      if (lane == 0) {
        uint64_t word = 0;
        if (sp >= 0 && m <= P.thr) {
          const int row = (int)__umulhi((uint32_t)sp, w2_magic), col = sp - row * w2;
          const int slot = rt.pslot[row * ucols + col + k];
          const uint32_t cand = rt.key[slot];
          const uint64_t blk = cand == own ? stb : ((uint64_t)rt.eps()[slot] | ((uint64_t)cand << 32));
          P.final_blk[idx] = blk;
          P.motion[idx] = (uint16_t)((col | 0x80) | ((row | 0x80) << 8));
          word = done_word(blk);
        }
        P.done[idx] = word;
      }
      __syncwarp();
    }
  }
}

// Weight sums of the refit for every block's index word (the candidates the
// next inter search reads), one thread per block.
__global__ void __launch_bounds__(256) weight_desc_kernel(const uint64_t *__restrict__ blocks, int n,
                                                          float4 *__restrict__ desc) {
  __shared__ float4 s_wk[4];
  build_weight_table(s_wk);
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const WeightSums w = weight_sums((uint32_t)(__ldg(blocks + i) >> 32), s_wk);
    desc[i] = make_float4(w.asq, w.bsq, w.ab, w.f);
  }
}

// The blocks of the runs whose union overflowed the run table (noisy
// content), list[0 .. *count): one CTA per block and one window position per
// thread (sa <= 8: at most 256 positions), every position evaluated by its
// own thread, then the closed-form selection over the CTA (cta_select). The
// many distinct words of such windows are evaluated side by side instead of
// in a warp's successive rounds.
// One listed block searched by a CTA (THREADS >= 256, sa <= 8): thread t
// evaluates window position t, then the CTA-wide closed-form selection.
// Starts with a barrier (the previous block's readers of s_tab are done).
template <int THREADS>
__device__ __forceinline__ void cta_block_search(const SearchParams &P, int idx, BlockTab &s_tab,
                                                 const uint8_t *s_snap5, const uint8_t *s_snap6,
                                                 CtaReduce<THREADS> &red, int *s_sumsq) {
  const int tid = threadIdx.x, lane = tid & 31;
  const int w2 = 2 * P.sa, npos = w2 * w2;
  const int row = tid / w2, col = tid - row * w2;  // the thread's window position tid
  const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
  const int by = idx / P.bw, bx = idx - by * P.bw;
  const uint64_t stb = __ldg(P.stb + idx);
  const uint32_t own = (uint32_t)(stb >> 32);
  __syncthreads();
  if (tid < 32) {
    const int sq = stage_block(s_tab, P.rgb, P.width, bx, by, lane);
    if (tid == 0) *s_sumsq = sq;
  }
  __syncthreads();
  const int orig = __ldg(P.orig_err + idx), sumsq = *s_sumsq;
  const PixelGroups pg = load_groups(s_tab);
  LaneSel ls;
  uint32_t cand = own, eps = 0;
  const int j = by - P.sa + row, i = bx - P.sa + col;
  if (tid < npos && i >= 0 && j >= 0 && i < P.bw && j < P.bh) {
    const size_t nidx = (size_t)j * P.bw + i;
    cand = __ldg(prev_hi + 2 * nidx);
    int e = 0;  // the block's own word: the stb block, no refit
    if (cand != own) {
      const float4 d = __ldg(P.wdesc + nidx);
      const WeightSums ws{d.x, d.y, d.z, d.w};
      int refit = 0;
      e = eval_candidate(s_tab, pg, s_snap5, s_snap6, cand, ws, own, orig, sumsq, eps, refit);
    }
    ls.add(tid, row, e);
  }
  int m, pick;
  const int sel = cta_select<THREADS>(ls, red, w2, m, pick);
  const bool accept = sel >= 0 && m <= P.thr;  // CTA-uniform
  if (accept ? tid == sel : tid == 0) {
    uint64_t word = 0;
    if (accept) {
      const uint64_t blk = cand == own ? stb : ((uint64_t)eps | ((uint64_t)cand << 32));
      P.final_blk[idx] = blk;
      P.motion[idx] = (uint16_t)((col | 0x80) | ((row | 0x80) << 8));
      word = done_word(blk);
    }
    P.done[idx] = word;
  }
}

template <int THREADS>
__global__ void __launch_bounds__(THREADS) inter_overflow_kernel(SearchParams P, const uint32_t *__restrict__ list,
                                                                 const uint32_t *__restrict__ count) {
  static_assert(THREADS >= 256, "one thread per position of a 16x16 window");
  const int n = (int)__ldcg(count);
  if ((int)blockIdx.x >= n) return;  // the whole CTA, before its barriers
  __shared__ BlockTab s_tab;
  __shared__ uint8_t s_snap5[256], s_snap6[256];
  __shared__ int s_red[2 * (THREADS / 32)];
  __shared__ int s_sumsq;
  build_snap_tables(s_snap5, s_snap6);
  CtaReduce<THREADS> red{s_red, 0};
  for (int k = blockIdx.x; k < n; k += gridDim.x)
    cta_block_search<THREADS>(P, (int)__ldcg(list + k), s_tab, s_snap5, s_snap6, red, &s_sumsq);
}

}  // namespace mptc
