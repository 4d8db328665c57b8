// Evaluation of a candidate index word on a block (the refit, snap, validity
// and error of DXTImage::Reencode, codec/dxt_image.cpp:258-349) and the
// staging of the block it needs.
#pragma once
#include <cstdint>

#include "status_bits.cuh"

namespace mptc {

constexpr uint32_t kFull = 0xffffffffu;
constexpr int kInvalid = 0x7fffffff;  // invalid candidate / no selection (INT_MAX)


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

// Stages two blocks with one warp, lanes 0-15 the pixels of block (ax, ay)
// into ta, lanes 16-31 those of (bx2, by2) into tb (a block with has_* false
// is not read); the same tables as stage_block. Returns each lane's half's sum
// of squared pixel values.
__device__ __forceinline__ int stage_block_pair(BlockTab &ta, BlockTab &tb, const uint8_t *__restrict__ rgb,
                                                int width, int ax, int ay, bool has_a, int bx2, int by2, bool has_b,
                                                int lane) {
  const int half = lane >> 4, p = lane & 15;
  BlockTab &t = half ? tb : ta;
  const bool has = half ? has_b : has_a;
  const int bx = half ? bx2 : ax, by = half ? by2 : ay;
  int sq = 0;
  uint32_t pk = 0;
  if (has) {
    const int r = p >> 2, c = p & 3;
    const uint8_t *px = rgb + ((size_t)(4 * by + r) * width + 4 * bx + c) * 3;
    const uint32_t R = px[0], G = px[1], B = px[2];
    const float third = __fdiv_rn(1.0f, 3.0f);
    const float fr = __uint2float_rn(R), fg = __uint2float_rn(G), fb = __uint2float_rn(B);
    const float qr = __fmul_rn(fr, third), qg = __fmul_rn(fg, third), qb = __fmul_rn(fb, third);
    const float4 P = make_float4(fr, fg, fb, 0.0f), Z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float4 Q = make_float4(qr, qg, qb, 0.0f);
    const float4 Q2 = make_float4(__fadd_rn(qr, qr), __fadd_rn(qg, qg), __fadd_rn(qb, qb), 0.0f);
    const float4 va[4] = {P, Z, Q2, Q}, vb[4] = {Z, P, Q, Q2};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      t.ab[p][0][k] = make_float2(va[k].x, va[k].y);
      t.ab[p][1][k] = make_float2(va[k].z, vb[k].x);
      t.ab[p][2][k] = make_float2(vb[k].y, vb[k].z);
    }
    pk = R | (G << 8) | (B << 16);
    sq = (int)(R * R + G * G + B * B);
  }
  // channel bytes of each group of four pixels of this half's block
  const int c = p >> 2, g = p & 3, base = lane & 16;
  const uint32_t p0 = __shfl_sync(kFull, pk, base + 4 * g + 0), p1 = __shfl_sync(kFull, pk, base + 4 * g + 1);
  const uint32_t p2 = __shfl_sync(kFull, pk, base + 4 * g + 2), p3 = __shfl_sync(kFull, pk, base + 4 * g + 3);
  if (has && p < 12) {
    const uint32_t sh = 8 * c;
    t.pg[c][g] = ((p0 >> sh) & 0xFF) | (((p1 >> sh) & 0xFF) << 8) | (((p2 >> sh) & 0xFF) << 16) |
                 (((p3 >> sh) & 0xFF) << 24);
  }
#pragma unroll
  for (int o = 8; o > 0; o >>= 1) sq += __shfl_xor_sync(kFull, sq, o);
  __syncwarp();
  return sq;
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

}  // namespace mptc
