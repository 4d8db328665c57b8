// Learned candidate proposal, the embedding half on the fifth-generation
// tensor cores (tcgen05): the two MLPs as fused persistent kernels (weights
// staged once per CTA by a bulk TMA copy, every layer an MMA into TMEM, bias +
// ReLU epilogues that turn the accumulator into the next layer's bf16 operand
// in shared memory).
//
// Model: f(block) 54 -> 128 -> 128 -> 64 over the block's 48 pixel bytes
// (normalised per channel to the block's own range) and its stb endpoints
// (5/6/5-bit values normalised to [0, 1]); g(word) 32 -> 128 -> 64 over the
// bits of an index word; score = f . g. Operands BF16, accumulation FP32.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

#include "learned_common.cuh"
#include "status_bits.cuh"
#include "tc_sm100.cuh"

namespace mptc {

// ---- packed weight image -------------------------------------------------------
// Every layer's weight as the MMA's B operand: output rows (N) x input columns
// (K, padded to a multiple of 64), K-major, 128-byte swizzled, in chunks of
// 64 input columns (chunk kc holds N rows x 128 bytes). f1 | f2 | f3 | g1 | g2.
constexpr uint32_t kImgF1 = 0;                                       // kH1 x 64
constexpr uint32_t kImgF2 = kImgF1 + (uint32_t)kH1 * kFeatPad * 2;   // kH2 x kH1: kH1 / 64 chunks
constexpr uint32_t kImgF3 = kImgF2 + (uint32_t)kH2 * kH1 * 2;        // 64 x kH2: kH2 / 64 chunks
constexpr uint32_t kImgG1 = kImgF3 + (uint32_t)kEmb * kH2 * 2;       // kCandH x 64 (32 inputs, zero padded)
constexpr uint32_t kImgG2 = kImgG1 + (uint32_t)kCandH * 64 * 2;      // 64 x kCandH: kCandH / 64 chunks
constexpr uint32_t kImgBytes = kImgG2 + (uint32_t)kEmb * kCandH * 2;
static_assert(kH1 % 64 == 0 && kH2 % 64 == 0 && kH1 + kH2 <= 512, "f's accumulators fit in TMEM");

// Image element (n, k) of a layer with `in` inputs and `out` outputs from the
// fp32 master weight W[in][out] (y = x W + b).
static __global__ void pack_layer_kernel(const float *__restrict__ W, int in, int out, int kpad, uint8_t *__restrict__ img) {
  const int total = out * kpad;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int n = e / kpad, k = e - n * kpad;
    const int kc = k >> 6, kk = k & 63;
    const uint32_t off = (uint32_t)kc * (uint32_t)out * 128u + tc::sw128_offset(n, kk >> 3) + (kk & 7) * 2;
    *reinterpret_cast<__nv_bfloat16 *>(img + off) = __float2bfloat16(k < in ? W[(size_t)k * out + n] : 0.f);
  }
}

// ---- fused MLP kernels -----------------------------------------------------------
struct EmbedArgs {
  const uint8_t *rgb;       // blocks: the frame
  int width, bw, n;         // n rows (blocks or words)
  const uint64_t *stb;      // blocks: stb endpoints; words: NULL
  const uint32_t *blocks;   // blocks: block index of row i (NULL: block i)
  const uint32_t *words;    // words: index word of row i at words[i * word_stride]
  int word_stride;
  const uint8_t *wimg;      // packed weight image (kImgBytes)
  const float *b1, *b2, *b3;  // biases (fp32)
  __nv_bfloat16 *out;       // n x 64 (row out_rows[i] for row i when out_rows is set)
  uint32_t *status;         // device status word (kDevTimeout on an expired wait)
  const uint32_t *n_dev;    // rows: min(n, *n_dev) when set (a count written on the device)
  const uint32_t *out_rows; // output row of row i, or NULL (row i)
};

// A launch covers the rows of up to kMaxBatch jobs (the streams of a batch,
// or one): tiles of 128 rows are numbered across the jobs (job j owns tiles
// [tile_end[j-1], tile_end[j]), counted by each CTA at its start from the
// jobs' row counts) and CTAs take them from one counter, so streams of uneven
// resolution share the persistent grid.
struct EmbedBatch {
  int n;                     // jobs
  EmbedArgs a[kMaxBatch];
  uint32_t *next;            // tile counter (zero before the launch)
};

// The f network (three layers, TMEM kH1 + kH2 columns: acc1 [0, kH1), acc2
// [kH1, kH1 + kH2), acc3 [0, 64)) and the g network (two layers, TMEM 256
// columns: acc1 [0,128), acc2 [128,192)).
struct NetF {
  static constexpr int kLayers = 3, N1 = kH1, N2 = kH2, N3 = kEmb, kTmem = kH1 + kH2;
  static constexpr uint32_t kW = kImgF1, kWBytes = kImgG1 - kImgF1;
  static constexpr uint32_t kW1 = kImgF1 - kW, kW2 = kImgF2 - kW, kW3 = kImgF3 - kW;
};
struct NetG {
  static constexpr int kLayers = 2, N1 = 128, N2 = 64, N3 = 0, kTmem = 256;
  static constexpr uint32_t kW = kImgG1, kWBytes = kImgBytes - kImgG1;
  static constexpr uint32_t kW1 = kImgG1 - kW, kW2 = kImgG2 - kW, kW3 = 0;
};

constexpr int kEmbedThreads = 256;
using tc::kTileBytes;

template <class Net>
constexpr size_t embed_smem_bytes() {
  return 1024 + Net::kWBytes + 2 * kTileBytes + 64;
}

// Reads 32 accumulator columns of this thread's row, adds the bias, applies
// ReLU and stores them as bf16 into 16-byte chunks 4*h .. 4*h+3 of the row in a
// swizzled operand tile.
__device__ __forceinline__ void epilogue_to_tile(uint32_t taddr, const float *__restrict__ bias, uint8_t *tile,
                                                 int row, int h) {
  float v[32], bb[32];
  const float4 *b4 = reinterpret_cast<const float4 *>(bias);  // 32 biases, 16-byte aligned
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const float4 t = __ldg(b4 + j);
    bb[4 * j] = t.x;
    bb[4 * j + 1] = t.y;
    bb[4 * j + 2] = t.z;
    bb[4 * j + 3] = t.w;
  }
  tc::tmem_ld32(taddr, v);
  uint32_t pk[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const float x0 = fmaxf(v[2 * j] + bb[2 * j], 0.f), x1 = fmaxf(v[2 * j + 1] + bb[2 * j + 1], 0.f);
    const __nv_bfloat162 b = __floats2bfloat162_rn(x0, x1);
    pk[j] = *reinterpret_cast<const uint32_t *>(&b);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j)
    *reinterpret_cast<uint4 *>(tile + tc::sw128_offset(row, 4 * h + j)) =
        make_uint4(pk[4 * j], pk[4 * j + 1], pk[4 * j + 2], pk[4 * j + 3]);
}

// One layer: D (+)= A(tile, 64 input columns) * W(chunk)^T over 4 K steps.
__device__ __forceinline__ void issue_chunk(uint32_t d_tmem, const uint8_t *a_tile, const uint8_t *w_chunk,
                                            uint32_t idesc, bool accumulate) {
  const uint32_t a = tc::smem_addr(a_tile), b = tc::smem_addr(w_chunk);
#pragma unroll
  for (int k = 0; k < 4; ++k)
    tc::mma_bf16(d_tmem, tc::desc_sw128(a + 32 * k), tc::desc_sw128(b + 32 * k), idesc,
                 (accumulate || k > 0) ? 1u : 0u);
}

// Persistent fused MLP over tiles of 128 rows. 256 threads: two per row build
// the input features; for the epilogues warp w reads TMEM lanes 32*(w%4) ..
// (its rows) and the 32-column half w/4 of every 64-column chunk. Thread 0
// issues the MMAs. Chunk kc of a hidden layer goes to operand buffer kc%2, so
// the epilogue of chunk kc+1 overlaps the MMAs of chunk kc.
template <class Net, bool kBlocks>
__global__ void __launch_bounds__(kEmbedThreads, 1) embed_kernel(const __grid_constant__ EmbedBatch batch) {
  extern __shared__ uint8_t dsm[];
  uint8_t *sm = tc::align_1024(dsm);
  uint8_t *sW = sm;
  uint8_t *const sA0 = sm + Net::kWBytes, *const sA1 = sm + Net::kWBytes + kTileBytes;
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + Net::kWBytes + 2 * kTileBytes);  // weights, mma, buf0, buf1
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 4);
  volatile uint32_t *abort_flag = tslot + 1;
  volatile int *s_tile = reinterpret_cast<volatile int *>(tslot + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = warp & 3, h = warp >> 2;
  // the jobs' row counts and tile ends; the first tile is claimed before the
  // setup, so that CTAs left without a tile (device-side counts below the
  // launch's bound) return at once
  __shared__ int s_rows[kMaxBatch], s_tend[kMaxBatch];
  if (tid == 0) {
    int acc = 0;
    for (int j = 0; j < batch.n; ++j) {
      const EmbedArgs &aj = batch.a[j];
      const int rows = aj.n_dev ? min(aj.n, (int)*aj.n_dev) : aj.n;
      acc += (rows + 127) / 128;
      s_rows[j] = rows;
      s_tend[j] = acc;
    }
    *s_tile = (int)atomicAdd(batch.next, 1u);
  }
  __syncthreads();
  const int total = s_tend[batch.n - 1];
  if (*s_tile >= total) return;
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) tc::mbar_init(bar + i, 1);
    *abort_flag = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(tslot, Net::kTmem);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tslot;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(bar, Net::kWBytes);
    for (uint32_t o = 0; o < Net::kWBytes; o += 32768)
      tc::bulk_g2s(sW + o, batch.a[0].wimg + Net::kW + o, min(32768u, Net::kWBytes - o), bar);
  }
  if (!tc::mbar_wait(bar, 0, abort_flag)) *abort_flag = 1;
  uint32_t ph_mma = 0, ph_buf = 0;  // ph_buf bit b: parity of operand buffer b's barrier
  auto wait_buf = [&](int b) {
    if (!tc::mbar_wait(bar + 2 + b, (ph_buf >> b) & 1u, abort_flag)) *abort_flag = 1;
    ph_buf ^= 1u << b;
  };
  const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
  const int row = 32 * q + lane;
  // The next tile is drawn while the current one is in its hidden layers and
  // its input words are loaded then, so the feature build never waits on
  // global memory.
  struct Pending {
    uint32_t w[12];
    uint64_t stb;
    uint32_t word;
    bool valid;
  } pf;
  auto locate = [&](int gt, int &jb, int &tile) {
    jb = 0;
    while (gt >= s_tend[jb]) ++jb;
    tile = gt - (jb ? s_tend[jb - 1] : 0);
  };
  auto prefetch = [&](int gt) {
    pf.valid = false;
    if (gt >= total) return;
    int jb, tile;
    locate(gt, jb, tile);
    const EmbedArgs &a = batch.a[jb];
    const int gi = tile * 128 + (tid >> 1);
    if (gi >= s_rows[jb]) return;
    pf.valid = true;
    if constexpr (kBlocks) {
      const int bi = a.blocks ? (int)__ldg(a.blocks + gi) : gi;
      const int by = bi / a.bw, bx = bi - by * a.bw;
      load_block_words(a.rgb, a.width, bx, by, pf.w);
      pf.stb = __ldg(a.stb + bi);
    } else {
      pf.word = __ldg(a.words + (size_t)gi * a.word_stride);
    }
  };
  int gt = *s_tile;
  prefetch(gt);
  for (;;) {
    if (gt >= total || *abort_flag) break;
    int jb, tile;
    locate(gt, jb, tile);
    const EmbedArgs &a = batch.a[jb];
    // input features -> sA0
    {
      const int r = tid >> 1, half = tid & 1;
      uint32_t f[16];
      if (pf.valid) {
        if constexpr (kBlocks)
          block_feature_words(pf.w, pf.stb, half, f);
        else
          word_feature_half(pf.word, half, f);
      } else {
#pragma unroll
        for (int j = 0; j < 16; ++j) f[j] = 0u;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j)
        *reinterpret_cast<uint4 *>(sA0 + tc::sw128_offset(r, 4 * half + j)) =
            make_uint4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      issue_chunk(tmem, sA0, sW + Net::kW1, tc::idesc_bf16(128, Net::N1), false);
      tc::mma_commit(bar + 1);
      *s_tile = (int)atomicAdd(batch.next, 1u);  // the next tile, read after the next barrier
    }
    int gt_next = total;
    if (!tc::mbar_wait(bar + 1, ph_mma, abort_flag)) *abort_flag = 1;
    ph_mma ^= 1;
    tc::tc_fence_after();
    // layer 2 from acc1 [0, N1) into acc2 [N1, N1 + N2)
    constexpr int KC2 = Net::N1 / 64;
#pragma unroll 1
    for (int kc = 0; kc < KC2; ++kc) {
      const int b = kc & 1;
      if (kc >= 2) wait_buf(b);
      uint8_t *const buf = b ? sA1 : sA0;
      epilogue_to_tile(lane_base + 64 * kc + 32 * h, a.b1 + 64 * kc + 32 * h, buf, row, h);
      tc::fence_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc::tc_fence_after();
        issue_chunk(tmem + Net::N1, buf, sW + Net::kW2 + (uint32_t)kc * Net::N2 * 128u, tc::idesc_bf16(128, Net::N2),
                    kc > 0);
        tc::mma_commit(bar + 2 + b);
      }
      if (kc == 0) {
        gt_next = *s_tile;
        prefetch(gt_next);
      }
    }
    wait_buf(0);
    if (KC2 > 1) wait_buf(1);
    tc::tc_fence_after();
    uint32_t out_col = Net::N1;  // accumulator holding the embedding
    const float *out_bias = a.b2;
    if constexpr (Net::kLayers == 3) {
      // layer 3 from acc2 into acc3 [0, N3)
      constexpr int KC3 = Net::N2 / 64;
#pragma unroll 1
      for (int kc = 0; kc < KC3; ++kc) {
        const int b = kc & 1;
        if (kc >= 2) wait_buf(b);
        uint8_t *const buf = b ? sA1 : sA0;
        epilogue_to_tile(lane_base + Net::N1 + 64 * kc + 32 * h, a.b2 + 64 * kc + 32 * h, buf, row, h);
        tc::fence_async_smem();
        tc::tc_fence_before();
        __syncthreads();
        if (tid == 0) {
          tc::tc_fence_after();
          issue_chunk(tmem, buf, sW + Net::kW3 + (uint32_t)kc * Net::N3 * 128u, tc::idesc_bf16(128, Net::N3),
                      kc > 0);
          tc::mma_commit(bar + 2 + b);
        }
      }
      wait_buf(0);
      if (KC3 > 1) wait_buf(1);
      tc::tc_fence_after();
      out_col = 0;
      out_bias = a.b3;
    }
    // embedding: 64 columns, half h of them per warp, + bias, bf16 to the output row
    {
      float v[32], bb[32];
      const float4 *b4 = reinterpret_cast<const float4 *>(out_bias + 32 * h);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float4 t = __ldg(b4 + j);
        bb[4 * j] = t.x;
        bb[4 * j + 1] = t.y;
        bb[4 * j + 2] = t.z;
        bb[4 * j + 3] = t.w;
      }
      tc::tmem_ld32(lane_base + out_col + 32 * h, v);
      const int gi = tile * 128 + row;
      if (gi < s_rows[jb]) {
        uint32_t pk[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const __nv_bfloat162 b2 = __floats2bfloat162_rn(v[2 * j] + bb[2 * j], v[2 * j + 1] + bb[2 * j + 1]);
          pk[j] = *reinterpret_cast<const uint32_t *>(&b2);
        }
        const size_t orow = a.out_rows ? (size_t)__ldg(a.out_rows + gi) : (size_t)gi;
        uint4 *dst = reinterpret_cast<uint4 *>(a.out + orow * kEmb + 32 * h);
#pragma unroll
        for (int j = 0; j < 4; ++j) dst[j] = make_uint4(pk[4 * j], pk[4 * j + 1], pk[4 * j + 2], pk[4 * j + 3]);
      }
    }
    tc::tc_fence_before();
    __syncthreads();
    gt = gt_next;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_free(tmem, Net::kTmem);
  if (tid == 0 && *abort_flag)
    for (int j = 0; j < batch.n; ++j) atomicOr(batch.a[j].status, kDevTimeout);
}


}  // namespace mptc
