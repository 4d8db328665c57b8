// The reference's selection rule over a search window in closed form, for a
// warp (LaneSel, warp_select) and for a CTA (ThreadSel, CtaReduce,
// cta_select), and the parameters every search kernel takes.
#pragma once
#include <cstdint>

#include "candidate_eval.cuh"

namespace mptc {

// The selection rule in closed form, for a warp that holds all positions of
// a window spread over its lanes (each lane visits its positions in scan
// order). The reference loop (if e < m { m = e; sel = pos; if e <= 0 { m = 0;
// break the row } }) selects:
// - if some valid position has e <= 0: let P0 be the first (scan order) and
//   r0 its row. Later rows replace the selection with their first e < 0 (e < 0
//   beats m = 0, then the row breaks), so the last row after r0 holding an
//   e < 0 gives its first e < 0; without one the selection stays P0. Rows
//   before r0 hold no e <= 0, and row r0 breaks at P0. m = 0.
// - otherwise the first position of the minimum e (strict improvement), m = it.
// Each lane keeps the three positions (first e <= 0; the key
// row << 16 | (0xFFFF - pos) of its e < 0 positions; first minimum, ties
// broken by position, so a lane may visit its positions in any order); four
// warp reductions give the selected position, whose candidate data the caller
// recovers.
struct LaneSel {
  int le0_pos = 0x7fffffff;  // first position with e <= 0
  int neg_key = -1;          // max over e < 0 of (row << 16 | (0xFFFF - pos))
  int min_e = kInvalid, min_pos = 0x7fffffff;
  __device__ __forceinline__ void add(int pos, int row, int e) {
    if (e == kInvalid) return;
    if (e <= 0 && pos < le0_pos) le0_pos = pos;
    if (e < 0) neg_key = max(neg_key, (row << 16) | (0xFFFF - pos));
    if (e < min_e || (e == min_e && pos < min_pos)) {  // the first minimum, in any arrival order
      min_e = e;
      min_pos = pos;
    }
  }
};

// Returns the selected position (-1 when no position is valid) and its m.
__device__ __forceinline__ int warp_select(const LaneSel &l, int w2, int &m) {
  const int p0 = __reduce_min_sync(kFull, l.le0_pos);
  if (p0 != 0x7fffffff) {
    m = 0;
    const int key = __reduce_max_sync(kFull, l.neg_key);
    return (key >= 0 && (key >> 16) > p0 / w2) ? 0xFFFF - (key & 0xFFFF) : p0;
  }
  m = __reduce_min_sync(kFull, l.min_e);
  const int p = __reduce_min_sync(kFull, l.min_e == m ? l.min_pos : 0x7fffffff);
  return p == 0x7fffffff ? -1 : p;
}

// The same closed form for a CTA whose threads each hold positions base + tid
// of successive rounds, keeping for each of the three statistics the
// candidate data of its position (the owner of the selected position writes
// the result).
struct SelPick {
  uint32_t cand = 0, eps = 0;
  int refit = 0;
};
struct ThreadSel : LaneSel {
  SelPick le0, neg, mn;
  __device__ __forceinline__ void add(int pos, int row, int e, uint32_t cand, uint32_t eps, int refit) {
    if (e == kInvalid) return;
    if (e <= 0 && pos < le0_pos) {
      le0_pos = pos;
      le0 = SelPick{cand, eps, refit};
    }
    if (e < 0) {
      const int key = (row << 16) | (0xFFFF - pos);
      if (key > neg_key) {
        neg_key = key;
        neg = SelPick{cand, eps, refit};
      }
    }
    if (e < min_e || (e == min_e && pos < min_pos)) {
      min_e = e;
      min_pos = pos;
      mn = SelPick{cand, eps, refit};
    }
  }
  // Takes in statistics of other positions (the minimum's ties broken by
  // position, as scan order does).
  template <class S>
  __device__ __forceinline__ void merge(const S &o) {
    if (o.le0_pos < le0_pos) {
      le0_pos = o.le0_pos;
      le0 = o.le0;
    }
    if (o.neg_key > neg_key) {
      neg_key = o.neg_key;
      neg = o.neg;
    }
    if (o.min_e < min_e || (o.min_e == min_e && o.min_pos < min_pos)) {
      min_e = o.min_e;
      min_pos = o.min_pos;
      mn = o.mn;
    }
  }
};

// A warp's selection statistics over some of its positions, kept in global
// memory from one fixed-point sweep to the next (intra_sweep_kernel).
struct SweepPartial {
  int le0_pos, neg_key, min_e, min_pos;
  SelPick le0, neg, mn;
};

// Reduces the warp's ThreadSel statistics into *dst (lanes holding a
// statistic write its candidate data; positions are distinct).
__device__ __forceinline__ void warp_store_partial(const ThreadSel &t, SweepPartial *dst, int lane) {
  const int le0 = __reduce_min_sync(kFull, t.le0_pos);
  const int nk = __reduce_max_sync(kFull, t.neg_key);
  const int me = __reduce_min_sync(kFull, t.min_e);
  const int mp = __reduce_min_sync(kFull, t.min_e == me ? t.min_pos : 0x7fffffff);
  if (lane == 0) {
    dst->le0_pos = le0;
    dst->neg_key = nk;
    dst->min_e = me;
    dst->min_pos = mp;
  }
  if (le0 != 0x7fffffff && t.le0_pos == le0) dst->le0 = t.le0;
  if (nk >= 0 && t.neg_key == nk) dst->neg = t.neg;
  if (mp != 0x7fffffff && t.min_e == me && t.min_pos == mp) dst->mn = t.mn;
}

// Completion word of a final block: bit 32 set, the low half the block's
// index word, which is all a waiting block reads of it.
__device__ __forceinline__ uint64_t done_word(uint64_t blk) { return (1ull << 32) | (blk >> 32); }

struct SearchParams {
  const uint8_t *rgb;
  const float4 *wdesc;    // weight sums of the previous frame's final blocks (inter)
  const uint64_t *stb;
  const int32_t *orig_err;
  const uint64_t *prev;   // previous frame's final blocks (inter)
  uint64_t *final_blk;
  uint16_t *motion;       // (x | y << 8) per block
  uint64_t *done;         // per block: 0 while open, done_word(final block) once final
  uint32_t *work;         // dataflow work counter
  uint32_t *status;       // device status bits
  int width, bw, bh, sa, thr;
};

// Block-wide reductions for the intra CTA (THREADS/32 warps). `buf` holds two
// alternating rows of per-warp partials so one barrier per reduction suffices.
template <int THREADS>
struct CtaReduce {
  int *buf;  // [2][THREADS/32]
  int phase;
  __device__ __forceinline__ int min(int v) {
    const int w = __reduce_min_sync(kFull, v);
    int *b = buf + phase * (THREADS / 32);
    phase ^= 1;
    if ((threadIdx.x & 31) == 0) b[threadIdx.x >> 5] = w;
    __syncthreads();
    int r = b[0];
#pragma unroll
    for (int k = 1; k < THREADS / 32; ++k) r = r < b[k] ? r : b[k];
    return r;
  }
  __device__ __forceinline__ int max(int v) { return -min(-v); }
};

// Closed-form selection over the CTA (see LaneSel): two or three block-wide
// reductions. Returns the selected position (-1: none valid), its m, and in
// `pick` the statistic that holds it (0 first e <= 0, 1 last-row e < 0, 2
// first minimum); the position's owner is thread sel % THREADS.
template <int THREADS>
__device__ __forceinline__ int cta_select(const LaneSel &t, CtaReduce<THREADS> &red, int w2, int &m, int &pick) {
  const int p0 = red.min(t.le0_pos);
  if (p0 != 0x7fffffff) {
    m = 0;
    const int key = red.max(t.neg_key);
    if (key >= 0 && (key >> 16) > p0 / w2) {
      pick = 1;
      return 0xFFFF - (key & 0xFFFF);
    }
    pick = 0;
    return p0;
  }
  m = red.min(t.min_e);
  const int p = red.min(t.min_e == m ? t.min_pos : 0x7fffffff);
  pick = 2;
  return p == 0x7fffffff ? -1 : p;
}

}  // namespace mptc
