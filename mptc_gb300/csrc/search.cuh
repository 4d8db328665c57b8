// K-b: the index-block search of DXTImage::Reencode (codec/dxt_image.cpp:652-957).
//
// For a block and a candidate index word (the interp of a block in the search
// window) the reference assigns the candidate's indices, refits both endpoints
// by least squares in float, snaps them with ToFiveBits/ToSixBits, and keeps
// the candidate only if Pack565(ep1) > Pack565(ep2); the candidate's error is
// floor(SSE/48) against the block's own pixels, compared with the block's stb
// error (orig_err). A warp evaluates one block, its lanes walking the window in
// 32-position chunks of the reference's scan order; a warp-uniform state
// machine then applies the reference's selection rule exactly:
//
//   positions are scanned row by row; a candidate replaces the running minimum
//   when err_diff < min; the first err_diff <= 0 pins min to 0 and ends that
//   ROW only (the `break` leaves the inner loop), so a later row can still
//   replace the selection with a strictly negative err_diff.
//
// The inter search reads the previous frame only and runs fully parallel. The
// intra search reads this frame's blocks as already finalised in raster order,
// so it runs as a dataflow over blocks: each block waits (bounded) on per-block
// release flags of every block in its causal window, then decides and
// publishes its own flag.
#pragma once
#include <cstdint>

namespace mptc {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kInvalid = 0x7fffffff;  // invalid candidate / no selection (INT_MAX)

// Device status bits (OR-ed into the context's status word).
constexpr uint32_t kDevTimeout = 1u;

// Staging of the block being searched (one per warp in the inter search, one
// per CTA in the intra search).
//
// The refit accumulates, per pixel i and channel c, ax += px*a and bx += px*b
// with (a, b) = ((3-order)/3, order/3), order = {0,3,1,2}[index]. For the four
// index values the products are exactly (px, 0), (0, px), (2q, q), (q, 2q)
// with q = fl(px * fl(1/3)) (fl(2/3) = 2 fl(1/3), and doubling is exact), so
// the block keeps them as a table ab[i][index] = {A.xyz, B.xyz} and a
// candidate's refit becomes one lookup and six adds per pixel.
//
// Layout ab[pixel][part][index] (float2): part 0 = (A_r, A_g), 1 = (A_b, B_r),
// 2 = (B_g, B_b). The four index variants of one (pixel, part) are adjacent,
// so the lanes of a warp, whatever their indices, read distinct banks.
struct __align__(16) BlockTab {
  float2 ab[16][3][4];
  uint32_t pg[3][4];    // channel c bytes of pixels 4g .. 4g+3 (for dp4a)
};

// The twelve channel-group words of the staged block, held in registers.
struct PixelGroups {
  uint32_t w[3][4];
};

__device__ __forceinline__ PixelGroups load_groups(const BlockTab &t) {
  PixelGroups g;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int k = 0; k < 4; ++k) g.w[c][k] = t.pg[c][k];
  return g;
}

// Per-candidate weight sums of the refit (they depend on the index word only).
struct WeightSums {
  float asq, bsq, ab, f;  // f = 1 / (asq*bsq - ab*ab)
};

// ToFiveBits / ToSixBits (codec/dxt_image.cpp:72-121) as 256-entry tables,
// built per CTA in shared memory: value -> snapped 8-bit value.
__device__ __forceinline__ uint8_t snap_value(uint32_t x, uint32_t keep, uint32_t step, uint32_t sh) {
  uint32_t base = x & keep;
  uint32_t high = (base == 255u) ? base : base + step;
  uint32_t low = (base == 0u) ? base : base - step;
  base = (base | (base >> sh)) & 0xFF;
  high = (high | (high >> sh)) & 0xFF;
  low = (low | (low >> sh)) & 0xFF;
  const uint32_t db = x > base ? x - base : base - x;
  const uint32_t dh = x > high ? x - high : high - x;
  const uint32_t dl = x > low ? x - low : low - x;
  if (db <= dh) return (uint8_t)(db < dl ? base : low);
  return (uint8_t)high;
}

__device__ __forceinline__ void build_snap_tables(uint8_t *snap5, uint8_t *snap6) {
  for (int t = threadIdx.x; t < 256; t += blockDim.x) {
    snap5[t] = snap_value((uint32_t)t, 0xF8u, 4u, 5u);
    snap6[t] = snap_value((uint32_t)t, 0xFCu, 2u, 6u);
  }
}

// Stages block (bx, by) into `t` with the 32 lanes of one warp and returns
// the block's sum of squared pixel values (all lanes).
__device__ __forceinline__ int stage_block(BlockTab &t, const uint8_t *__restrict__ rgb, int width, int bx, int by,
                                           int lane) {
  int sq = 0;
  uint32_t pk = 0;
  if (lane < 16) {
    const int r = lane >> 2, c = lane & 3;
    const uint8_t *p = rgb + ((size_t)(4 * by + r) * width + 4 * bx + c) * 3;
    const uint32_t R = p[0], G = p[1], B = p[2];
    const float third = __fdiv_rn(1.0f, 3.0f);
    const float fr = __uint2float_rn(R), fg = __uint2float_rn(G), fb = __uint2float_rn(B);
    const float qr = __fmul_rn(fr, third), qg = __fmul_rn(fg, third), qb = __fmul_rn(fb, third);
    const float4 P = make_float4(fr, fg, fb, 0.0f), Z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 Q = make_float4(qr, qg, qb, 0.0f);
    const float4 Q2 = make_float4(__fadd_rn(qr, qr), __fadd_rn(qg, qg), __fadd_rn(qb, qb), 0.0f);
    // (A, B) per index: 0: (px, 0), 1: (0, px), 2: (2q, q), 3: (q, 2q)
    const float4 va[4] = {P, Z, Q2, Q}, vb[4] = {Z, P, Q, Q2};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      t.ab[lane][0][k] = make_float2(va[k].x, va[k].y);
      t.ab[lane][1][k] = make_float2(va[k].z, vb[k].x);
      t.ab[lane][2][k] = make_float2(vb[k].y, vb[k].z);
    }
    pk = R | (G << 8) | (B << 16);
    sq = (int)(R * R + G * G + B * B);
  }
  // channel bytes of each group of four pixels
  const int c = lane >> 2, g = lane & 3;
  const uint32_t p0 = __shfl_sync(kFull, pk, 4 * g + 0), p1 = __shfl_sync(kFull, pk, 4 * g + 1);
  const uint32_t p2 = __shfl_sync(kFull, pk, 4 * g + 2), p3 = __shfl_sync(kFull, pk, 4 * g + 3);
  if (lane < 12) {
    const uint32_t sh = 8 * c;
    t.pg[c][g] = ((p0 >> sh) & 0xFF) | (((p1 >> sh) & 0xFF) << 8) | (((p2 >> sh) & 0xFF) << 16) |
                 (((p3 >> sh) & 0xFF) << 24);
  }
  __syncwarp();
  return __reduce_add_sync(kFull, sq);
}

// Weight sums of the refit for index word `cand`, accumulated in the
// reference's order (codec/dxt_image.cpp:307-312) from the per-index constants
// wk[index] = (a*a, b*b, a*b).
__device__ __forceinline__ WeightSums weight_sums(uint32_t cand, const float4 *wk) {
  float asq = 0.f, bsq = 0.f, ab = 0.f;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const float4 w = wk[(cand >> (2 * i)) & 3u];
    asq = __fadd_rn(asq, w.x);
    bsq = __fadd_rn(bsq, w.y);
    ab = __fadd_rn(ab, w.z);
  }
  WeightSums r;
  r.asq = asq;
  r.bsq = bsq;
  r.ab = ab;
  r.f = __frcp_rn(__fsub_rn(__fmul_rn(asq, bsq), __fmul_rn(ab, ab)));
  return r;
}

// The per-index constants (a*a, b*b, a*b) with a, b as the reference computes
// them: a = (3-order)/3.0f, b = order/3.0f.
__device__ __forceinline__ void build_weight_table(float4 *wk) {
  if (threadIdx.x < 4) {
    const float order = threadIdx.x == 0 ? 0.f : threadIdx.x == 1 ? 3.f : threadIdx.x == 2 ? 1.f : 2.f;
    const float a = __fdiv_rn(__fsub_rn(3.0f, order), 3.0f), b = __fdiv_rn(order, 3.0f);
    wk[threadIdx.x] = make_float4(__fmul_rn(a, a), __fmul_rn(b, b), __fmul_rn(a, b), 0.0f);
  }
}

// Byte selector for __byte_perm from one byte of an index word: the four 2-bit
// indices of a group of pixels, spread to nibbles.
__device__ __forceinline__ uint32_t spread_nibbles(uint32_t b) {
  b = (b | (b << 4)) & 0x0F0Fu;
  return (b | (b << 2)) & 0x3333u;
}

// x86 cvttss2si of v followed by max(0, min(255, .)) (codec/dxt_image.cpp:330-331):
// NaN and |v| >= 2^31 convert to INT_MIN and therefore clamp to 0.
__device__ __forceinline__ uint32_t quantize_endpoint(float v) {
  float w = (v < 2147483648.0f) ? v : 0.0f;  // also maps NaN to 0
  w = fminf(fmaxf(w, 0.0f), 255.0f);
  return __float_as_uint(__fadd_rd(w, 8388608.0f)) - 0x4B000000u;  // floor(w)
}

__device__ __forceinline__ uint32_t pack565(uint32_t r, uint32_t g, uint32_t b) {
  return ((r & 0xF8u) << 8) | ((g & 0xFCu) << 3) | (b >> 3);
}

// Evaluates candidate `cand` on the staged block. Returns err_diff, or
// kInvalid when the refit would swap the endpoints (the candidate is skipped).
// `own` is the block's stb interp: AssignIndices with it is the identity
// (blk == blk2), which keeps the stb block with err_diff 0 and no refit.
// ws holds the candidate's weight sums.
__device__ __forceinline__ int eval_candidate(const BlockTab &t, const PixelGroups &pg, const uint8_t *snap5,
                                              const uint8_t *snap6, uint32_t cand, const WeightSums &ws,
                                              uint32_t own, int orig_err, int sumsq, uint32_t &eps, int &refit) {
  if (cand == own) {
    eps = 0;
    refit = 0;
    return 0;
  }
  refit = 1;
  // refit sums, pixel by pixel in the reference's order (codec/dxt_image.cpp:298-318)
  float ax0 = 0.f, ax1 = 0.f, ax2 = 0.f, bx0 = 0.f, bx1 = 0.f, bx2 = 0.f;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint32_t k = (cand >> (2 * i)) & 3u;
    const float2 u = t.ab[i][0][k], v = t.ab[i][1][k], w = t.ab[i][2][k];
    ax0 = __fadd_rn(ax0, u.x);
    bx0 = __fadd_rn(bx0, v.y);
    ax1 = __fadd_rn(ax1, u.y);
    bx1 = __fadd_rn(bx1, w.x);
    ax2 = __fadd_rn(ax2, v.x);
    bx2 = __fadd_rn(bx2, w.y);
  }
  // 2x2 solve (codec/dxt_image.cpp:320-326)
  const float f = ws.f, asq = ws.asq, bsq = ws.bsq, ab = ws.ab;
  const float p1r = __fmul_rn(f, __fsub_rn(__fmul_rn(ax0, bsq), __fmul_rn(bx0, ab)));
  const float p1g = __fmul_rn(f, __fsub_rn(__fmul_rn(ax1, bsq), __fmul_rn(bx1, ab)));
  const float p1b = __fmul_rn(f, __fsub_rn(__fmul_rn(ax2, bsq), __fmul_rn(bx2, ab)));
  const float p2r = __fmul_rn(f, __fsub_rn(__fmul_rn(bx0, asq), __fmul_rn(ax0, ab)));
  const float p2g = __fmul_rn(f, __fsub_rn(__fmul_rn(bx1, asq), __fmul_rn(ax1, ab)));
  const float p2b = __fmul_rn(f, __fsub_rn(__fmul_rn(bx2, asq), __fmul_rn(ax2, ab)));
  // quantise + snap (codec/dxt_image.cpp:329-341)
  const uint32_t e1r = snap5[quantize_endpoint(__fadd_rn(p1r, 0.5f))];
  const uint32_t e1g = snap6[quantize_endpoint(__fadd_rn(p1g, 0.5f))];
  const uint32_t e1b = snap5[quantize_endpoint(__fadd_rn(p1b, 0.5f))];
  const uint32_t e2r = snap5[quantize_endpoint(__fadd_rn(p2r, 0.5f))];
  const uint32_t e2g = snap6[quantize_endpoint(__fadd_rn(p2g, 0.5f))];
  const uint32_t e2b = snap5[quantize_endpoint(__fadd_rn(p2b, 0.5f))];
  const uint32_t q1 = pack565(e1r, e1g, e1b), q2 = pack565(e2r, e2g, e2b);
  if (q1 <= q2) return kInvalid;  // LogicalToPhysical would swap: skipped
  eps = q1 | (q2 << 16);
  // 4-colour palette of the refit (LerpChannels 1/3, 2/3, :346-347), one word
  // per channel holding the channel's four palette bytes
  const uint32_t wr = e1r | (e2r << 8) | (((2 * e1r + e2r) / 3) << 16) | (((e1r + 2 * e2r) / 3) << 24);
  const uint32_t wg = e1g | (e2g << 8) | (((2 * e1g + e2g) / 3) << 16) | (((e1g + 2 * e2g) / 3) << 24);
  const uint32_t wb = e1b | (e2b << 8) | (((2 * e1b + e2b) / 3) << 16) | (((e1b + 2 * e2b) / 3) << 24);
  // SSE = sum|s|^2 - 2 sum s.pal[idx] + sum |pal[idx]|^2 over four-pixel groups:
  // __byte_perm gathers the indexed palette bytes, dp4a multiplies-adds them.
  uint32_t cross = 0, norm = 0;
#pragma unroll
  for (int g = 0; g < 4; ++g) {
    const uint32_t sel = spread_nibbles((cand >> (8 * g)) & 0xFFu);
    const uint32_t vr = __byte_perm(wr, 0u, sel), vg = __byte_perm(wg, 0u, sel), vb = __byte_perm(wb, 0u, sel);
    cross = __dp4a(pg.w[0][g], vr, cross);
    cross = __dp4a(pg.w[1][g], vg, cross);
    cross = __dp4a(pg.w[2][g], vb, cross);
    norm = __dp4a(vr, vr, norm);
    norm = __dp4a(vg, vg, norm);
    norm = __dp4a(vb, vb, norm);
  }
  const int sse = sumsq - 2 * (int)cross + (int)norm;
  return (int)((uint32_t)sse / 48u) - orig_err;
}

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
// row << 16 | (0xFFFF - pos) of its e < 0 positions; first minimum); four warp
// reductions give the selected position, whose candidate data the caller
// recovers.
struct LaneSel {
  int le0_pos = 0x7fffffff;  // first position with e <= 0
  int neg_key = -1;          // max over e < 0 of (row << 16 | (0xFFFF - pos))
  int min_e = kInvalid, min_pos = 0x7fffffff;
  __device__ __forceinline__ void add(int pos, int row, int e) {
    if (e == kInvalid) return;
    if (e <= 0 && pos < le0_pos) le0_pos = pos;
    if (e < 0) neg_key = max(neg_key, (row << 16) | (0xFFFF - pos));
    if (e < min_e) {  // positions arrive in increasing order: keeps the first minimum
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
    if (e < min_e) {
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

// ------------------------------------------------------------------ intra --
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

// The blocks of the runs whose union overflowed the run table (noisy
// content), list[0 .. *count): one CTA per block and one window position per
// thread (sa <= 8: at most 256 positions), every position evaluated by its
// own thread, then the closed-form selection over the CTA (cta_select). The
// many distinct words of such windows are evaluated side by side instead of
// in a warp's successive rounds.
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
  const int tid = threadIdx.x, lane = tid & 31;
  const int w2 = 2 * P.sa, npos = w2 * w2;
  const int row = tid / w2, col = tid - row * w2;  // the thread's window position tid
  const uint32_t *prev_hi = reinterpret_cast<const uint32_t *>(P.prev) + 1;
  for (int k = blockIdx.x; k < n; k += gridDim.x) {
    const int idx = (int)__ldcg(list + k);
    const int by = idx / P.bw, bx = idx - by * P.bw;
    const uint64_t stb = __ldg(P.stb + idx);
    const uint32_t own = (uint32_t)(stb >> 32);
    __syncthreads();  // the previous block's readers of s_tab are done
    if (tid < 32) {
      const int sq = stage_block(s_tab, P.rgb, P.width, bx, by, lane);
      if (tid == 0) s_sumsq = sq;
    }
    __syncthreads();
    const int orig = __ldg(P.orig_err + idx), sumsq = s_sumsq;
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
}

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

struct EvalCache {
  uint32_t key[kEvalBuckets];
  unsigned long long val[kEvalBuckets];
};

__device__ __forceinline__ void eval_cache_reset(EvalCache &c, uint32_t own) {
  for (int b = threadIdx.x; b < kEvalBuckets; b += blockDim.x) {
    c.key[b] = own;
    c.val[b] = kEvalPending;
  }
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

__device__ __forceinline__ int cached_eval(EvalCache &c, bool use, const BlockTab &tab, const PixelGroups &pg,
                                           const uint8_t *snap5, const uint8_t *snap6, const float4 *wk,
                                           uint32_t cand, uint32_t own, int orig, int sumsq, uint32_t &eps,
                                           int &refit, int &looked, int &hits) {
  if (cand == own) {
    eps = 0;
    refit = 0;
    return 0;
  }
  refit = 1;
  uint32_t b = (cand * 2654435761u) >> 23;  // 9 bits: kEvalBuckets
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
    b = (b + 1) & (kEvalBuckets - 1);
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
