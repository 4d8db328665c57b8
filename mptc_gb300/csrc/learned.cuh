// Training and embedding kernels of the learned candidate proposal (see
// learned_common.cuh for the model): tensor-core GEMM with transposes and
// fused bias/ReLU, feature builders, sampled softmax cross-entropy, AdamW.
#pragma once
#include "learned_common.cuh"
#include "tc_sm100.cuh"

namespace mptc {

// C[M x N] = op(A)[M x K] * op(B)[K x N], then the epilogue GemmEpi, on the
// fifth-generation tensor cores: BF16 operands, FP32 accumulators in TMEM.
// TA: A is stored K x M (row-major, lda), else M x K; TB: B is stored N x K,
// else K x N. Split K (gridDim.z > 1): slice z writes its partial product to
// C + z * M * ldc and nothing else; the caller sums the slices in order.
//
// Tiles of 128 x 128 (one TMEM lane per row), K in steps of 64 through two
// shared-memory stages in the 128-byte-swizzled K-major layout (rows of 64 K
// values). Each thread holds its share of the next step's operand tiles in
// registers while the tensor cores work on the current one: an operand whose
// K run is contiguous in memory (A not transposed, B transposed) moves as
// 16-byte vectors, the other is read 8 rows (or columns) at a time along its
// contiguous dimension and goes into the tile's rows through a register
// transpose. Thread 0 issues 4 tcgen05.mma (K = 16 each) per step and commits
// them to the stage's mbarrier; a stage is refilled once the MMAs that read it
// have completed. The epilogue moves the accumulator through shared memory 32
// columns at a time so that every warp store covers one 128-byte row segment.
constexpr int kTcBM = 128, kTcBN = 128, kTcBK = 64;
constexpr int kTcStage = (kTcBM + kTcBN) * 128;           // bytes of one stage (A and B tiles)
constexpr int kTcSmem = 2 * kTcStage + 1024;              // two stages + alignment slack
static_assert(kTcBM * 33 * 4 + 4 * 32 * 4 <= 2 * kTcStage, "epilogue staging fits in the stages");

// Epilogue of gemm_tc_kernel, applied in this order to each output x:
// + bias[n]; ReLU; x = 0 where mask[m * ldc + n] <= 0 (ReLU backward); then
// C (fp32) and/or Cb (bf16) receive x, and colpart[blockIdx.y * ldc + n] the
// sum of x over the tile's rows (rows in a fixed order: the same bits every
// run). Null pointers skip their step.
struct GemmEpi {
  float *C;
  __nv_bfloat16 *Cb;
  int ldc;
  const float *bias;
  int relu;
  const __nv_bfloat16 *mask;
  float *colpart;
};

// Eight consecutive bf16 at p, of which the first `valid` exist (zeros after):
// one 16-byte load when all eight exist and p is 16-byte aligned.
__device__ __forceinline__ uint4 load8_bf16(const __nv_bfloat16 *p, int valid) {
  if (valid >= 8 && (reinterpret_cast<uintptr_t>(p) & 15) == 0) return *reinterpret_cast<const uint4 *>(p);
  uint16_t h[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) h[j] = j < valid ? reinterpret_cast<const uint16_t *>(p)[j] : (uint16_t)0;
  return make_uint4(h[0] | ((uint32_t)h[1] << 16), h[2] | ((uint32_t)h[3] << 16), h[4] | ((uint32_t)h[5] << 16),
                    h[6] | ((uint32_t)h[7] << 16));
}

// One 128 x 64 operand tile (rows row0 .. row0 + 127 of nrows, K values
// k0 .. k0 + 63 below kend; zeros outside) in this thread's 8 registers.
// KMAJOR: src[row][k], stride ld: register i is K values 8 (t % 8) .. of row
// t / 8 + 16 i. Otherwise src[k][row]: register i is rows 8 (t / 8) .. of K
// value 8 (t % 8) + i.
template <bool KMAJOR>
__device__ __forceinline__ void load_tile(uint4 (&r)[8], const __nv_bfloat16 *__restrict__ src, int ld, int row0,
                                          int nrows, int k0, int kend, int tid) {
  const int kb = tid & 7;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    r[i] = make_uint4(0u, 0u, 0u, 0u);
    if (KMAJOR) {
      const int row = row0 + (tid >> 3) + 16 * i, k = k0 + 8 * kb;
      if (row < nrows && k < kend) r[i] = load8_bf16(src + (size_t)row * ld + k, kend - k);
    } else {
      const int row = row0 + 8 * (tid >> 3), k = k0 + 8 * kb + i;
      if (row < nrows && k < kend) r[i] = load8_bf16(src + (size_t)k * ld + row, nrows - row);
    }
  }
}

// Stores the registers of load_tile<KMAJOR> into the swizzled tile. The
// transposed case builds row r + j's 8 K values from element j of the 8
// registers: each output word is one byte permutation of two input words.
template <bool KMAJOR>
__device__ __forceinline__ void store_tile(uint8_t *tile, const uint4 (&r)[8], int tid) {
  const uint32_t kb = tid & 7;
  if (KMAJOR) {
#pragma unroll
    for (int i = 0; i < 8; ++i)
      *reinterpret_cast<uint4 *>(tile + tc::sw128_offset((uint32_t)((tid >> 3) + 16 * i), kb)) = r[i];
  } else {
    const uint32_t w[8][4] = {{r[0].x, r[0].y, r[0].z, r[0].w}, {r[1].x, r[1].y, r[1].z, r[1].w},
                              {r[2].x, r[2].y, r[2].z, r[2].w}, {r[3].x, r[3].y, r[3].z, r[3].w},
                              {r[4].x, r[4].y, r[4].z, r[4].w}, {r[5].x, r[5].y, r[5].z, r[5].w},
                              {r[6].x, r[6].y, r[6].z, r[6].w}, {r[7].x, r[7].y, r[7].z, r[7].w}};
    const uint32_t row = 8u * (uint32_t)(tid >> 3);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t sel = (j & 1) ? 0x7632u : 0x5410u;
      const uint4 o = make_uint4(__byte_perm(w[0][j >> 1], w[1][j >> 1], sel),
                                 __byte_perm(w[2][j >> 1], w[3][j >> 1], sel),
                                 __byte_perm(w[4][j >> 1], w[5][j >> 1], sel),
                                 __byte_perm(w[6][j >> 1], w[7][j >> 1], sel));
      *reinterpret_cast<uint4 *>(tile + tc::sw128_offset(row + (uint32_t)j, kb)) = o;
    }
  }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_tc_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                                                      const __nv_bfloat16 *__restrict__ B, int ldb, GemmEpi ep,
                                                      int M, int N, int K, uint32_t *__restrict__ status) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = tc::align_1024(smem_raw);
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  __shared__ volatile uint32_t abort_flag, drain_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTcBM, n0 = blockIdx.x * kTcBN;
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    abort_flag = 0;
    drain_flag = 0;
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::tmem_alloc(&tslot, kTcBN);
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  const uint32_t idesc = tc::idesc_bf16(kTcBM, kTcBN);
  // split K (blockIdx.z): this slice's K range, in whole steps
  const int ksplit = gridDim.z > 1 ? (K + gridDim.z - 1) / gridDim.z : K;
  const int kstep = (ksplit + kTcBK - 1) / kTcBK * kTcBK;
  const int kbeg = blockIdx.z * kstep, kend = min(K, kbeg + kstep);
  const int steps = kend > kbeg ? (kend - kbeg + kTcBK - 1) / kTcBK : 0;
  uint4 ra[8], rb[8];
  if (steps > 0) {
    load_tile<!TA>(ra, A, lda, m0, M, kbeg, kend, tid);
    load_tile<TB>(rb, B, ldb, n0, N, kbeg, kend, tid);
  }
  // A wait that gives up sets abort_flag: the remaining waits return at once,
  // the steps still run (uniform control flow) and the results are reported
  // invalid through *status.
  for (int s = 0; s < steps; ++s) {
    const int st = s & 1;
    uint8_t *sA = smem + st * kTcStage, *sB = sA + kTcBM * 128;
    // the MMAs of step s - 2 read this stage
    if (s >= 2 && !tc::mbar_wait(&bar[st], (uint32_t)((s - 2) >> 1) & 1u, &abort_flag)) abort_flag = 1;
    store_tile<!TA>(sA, ra, tid);
    store_tile<TB>(sB, rb, tid);
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t a = tc::smem_addr(sA), b = tc::smem_addr(sB);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(tmem, tc::desc_sw128(a + 32 * k), tc::desc_sw128(b + 32 * k), idesc, (s > 0 || k > 0) ? 1u : 0u);
      tc::mma_commit(&bar[st]);
    }
    if (s + 1 < steps) {
      const int k0 = kbeg + (s + 1) * kTcBK;
      load_tile<!TA>(ra, A, lda, m0, M, k0, kend, tid);
      load_tile<TB>(rb, B, ldb, n0, N, k0, kend, tid);
    }
  }
  // every MMA has completed once the last step's commit has arrived
  const uint32_t last_parity = (uint32_t)((steps - 1) >> 1) & 1u;
  if (steps > 0 && !tc::mbar_wait(&bar[(steps - 1) & 1], last_parity, &abort_flag)) abort_flag = 1;
  tc::tc_fence_after();
  const bool failed = __syncthreads_or(abort_flag != 0) != 0;
  if (failed) {
    // let MMAs still in flight finish (bounded) before the TMEM is freed
    if (steps > 0) tc::mbar_wait(&bar[(steps - 1) & 1], last_parity, &drain_flag, 100000000ull);
    if (tid == 0 && status) atomicOr(status, 1u);
  } else {
    // epilogue, 32 columns at a time: thread (warp, lane) moves its TMEM row
    // 32 w + lane into the staging rows, then writes column lane of rows
    // w, w + 4, ... (each warp store one 128-byte row segment)
    float *stg = reinterpret_cast<float *>(smem);  // 128 rows x 33 floats (the pad spreads the banks)
    float *csum = stg + kTcBM * 33;                // 4 warps x 32 columns
    const int row = 32 * warp + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
    const bool split = gridDim.z > 1;
#pragma unroll 1
    for (int c0 = 0; c0 < kTcBN && n0 + c0 < N; c0 += 32) {
      float v[32];
      tc::tmem_ld32(lane_base + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) stg[row * 33 + j] = steps > 0 ? v[j] : 0.f;
      __syncthreads();
      const int n = n0 + c0 + lane;
      float cs = 0.f;
      if (n < N && split) {
        float *Cz = ep.C + (size_t)blockIdx.z * M * ep.ldc;
#pragma unroll 8
        for (int i = 0; i < 32; ++i) {
          const int r = warp + 4 * i, m = m0 + r;
          if (m < M) Cz[(size_t)m * ep.ldc + n] = stg[r * 33 + lane];
        }
      } else if (n < N) {
        // the mask's 32 values are read before any store (a store through
        // another pointer could otherwise order each read after it)
        uint16_t mk[32];
        if (ep.mask) {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const int m = m0 + warp + 4 * i;
            mk[i] = m < M ? __bfloat16_as_ushort(ep.mask[(size_t)m * ep.ldc + n]) : (uint16_t)0;
          }
        }
        const float bn = ep.bias ? ep.bias[n] : 0.f;
#pragma unroll
        for (int i = 0; i < 32; ++i) {
          const int r = warp + 4 * i, m = m0 + r;
          if (m < M) {
            const size_t o = (size_t)m * ep.ldc + n;
            float x = stg[r * 33 + lane] + bn;
            if (ep.relu) x = x > 0.f ? x : 0.f;
            if (ep.mask && !(__bfloat162float(__ushort_as_bfloat16(mk[i])) > 0.f)) x = 0.f;
            if (ep.C) ep.C[o] = x;
            if (ep.Cb) ep.Cb[o] = __float2bfloat16(x);
            cs += x;
          }
        }
      }
      csum[warp * 32 + lane] = cs;
      __syncthreads();
      if (ep.colpart && !split && warp == 0 && n < N)
        ep.colpart[(size_t)blockIdx.y * ep.ldc + n] =
            ((csum[lane] + csum[32 + lane]) + csum[64 + lane]) + csum[96 + lane];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_free(tmem, kTcBN);
}

// Block features (block_feature_half) of blocks[r] (NULL: block r), n rows of
// kFeatPad bf16.
__global__ void block_features_kernel(const uint8_t *__restrict__ rgb, int width, int bw, const uint64_t *__restrict__ stb,
                                      const uint32_t *__restrict__ blocks, int n, __nv_bfloat16 *__restrict__ X) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 2 * n; e += gridDim.x * blockDim.x) {
    const int r = e >> 1, half = e & 1;
    const int idx = blocks ? (int)blocks[r] : r;
    const int by = idx / bw, bx = idx - by * bw;
    uint32_t f[16];
    block_feature_half(rgb, width, bx, by, stb[idx], half, f);
    uint4 *dst = reinterpret_cast<uint4 *>(X + (size_t)r * kFeatPad + 32 * half);
#pragma unroll
    for (int j = 0; j < 4; ++j) dst[j] = make_uint4(f[4 * j], f[4 * j + 1], f[4 * j + 2], f[4 * j + 3]);
  }
}

// Candidate features: the 32 bits of an index word as 0/1.
__global__ void cand_features_kernel(const uint32_t *__restrict__ words, int word_stride, int n,
                                     __nv_bfloat16 *__restrict__ X) {
  const int total = n * kCandIn;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int r = e / kCandIn, c = e % kCandIn;
    X[e] = __float2bfloat16((float)((words[(size_t)r * word_stride] >> c) & 1u));
  }
}

__global__ void bf16_to_f32_kernel(const __nv_bfloat16 *__restrict__ x, float *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = __bfloat162float(x[i]);
}

__global__ void to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = __float2bfloat16(x[i]);
}

// out[i] = sum over slices k < slices of part[k * n + i], in a fixed order
// (the same bits every run): warp w of a CTA of 256 threads sums slices
// w, w + 8, ... for the CTA's 32 outputs (lane = output) in four interleaved
// chains; the chains, then the warps, are added in order.
__global__ void __launch_bounds__(256) slice_sum_kernel(const float *__restrict__ part, int slices, int n,
                                                        float *__restrict__ out) {
  __shared__ float red[8][32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int i = blockIdx.x * 32 + lane;
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  if (i < n) {
    int k = warp;
    for (; k + 24 < slices; k += 32) {
      a0 += part[(size_t)k * n + i];
      a1 += part[(size_t)(k + 8) * n + i];
      a2 += part[(size_t)(k + 16) * n + i];
      a3 += part[(size_t)(k + 24) * n + i];
    }
    for (; k < slices; k += 8) a0 += part[(size_t)k * n + i];
  }
  red[warp][lane] = (a0 + a1) + (a2 + a3);
  __syncthreads();
  if (warp == 0 && i < n) {
    float t = 0.f;
#pragma unroll
    for (int w = 0; w < 8; ++w) t += red[w][lane];
    out[i] = t;
  }
}

constexpr int kMaxCE = 64;  // candidates per block in one training example

// Sampled softmax cross-entropy: block b scores its C candidates (row b*C .. of
// G) against F[b]; candidate 0 is the accepted one. Adds the mean loss
// (atomic) and writes the bf16 gradients dF [B x 64] and dG [B*C x 64], and
// for the bias gradients the fp32 column sums of each CTA's rows of dF and
// dG: partF / partG [gridDim.x x 64] (fixed order: candidates, then warps).
// One warp per block, 8 blocks per CTA of 256 threads, lane = dims lane and
// 32 + lane.
__global__ void __launch_bounds__(256) softmax_ce_kernel(const float *__restrict__ F, const float *__restrict__ G,
                                                         int B, int C, __nv_bfloat16 *__restrict__ dF,
                                                         __nv_bfloat16 *__restrict__ dG, float *__restrict__ partF,
                                                         float *__restrict__ partG, float *__restrict__ loss) {
  __shared__ float colF[8][kEmb], colG[8][kEmb];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.x * 8 + w;
  float df0 = 0.f, df1 = 0.f, cg0 = 0.f, cg1 = 0.f;
  if (b < B) {
    const float f0 = F[(size_t)b * kEmb + lane], f1 = F[(size_t)b * kEmb + 32 + lane];
    float s[kMaxCE];
    float mx = -1e30f;
    for (int j = 0; j < C; ++j) {  // score = F[b] . G[b, j], warp sum of per-lane partials
      const float *g = G + ((size_t)b * C + j) * kEmb;
      float v = f0 * g[lane] + f1 * g[32 + lane];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
      s[j] = v;
      mx = fmaxf(mx, v);
    }
    float z = 0.f;
    for (int j = 0; j < C; ++j) z += __expf(s[j] - mx);
    const float inv = 1.f / z;
    if (lane == 0) atomicAdd(loss, (mx + __logf(z) - s[0]) / B);
    for (int j = 0; j < C; ++j) {
      const float p = __expf(s[j] - mx) * inv;
      const float ds = (p - (j == 0 ? 1.f : 0.f)) / B;
      const float *g = G + ((size_t)b * C + j) * kEmb;
      df0 += ds * g[lane];
      df1 += ds * g[32 + lane];
      const float d0 = ds * f0, d1 = ds * f1;
      __nv_bfloat16 *dg = dG + ((size_t)b * C + j) * kEmb;
      dg[lane] = __float2bfloat16(d0);
      dg[32 + lane] = __float2bfloat16(d1);
      cg0 += d0;
      cg1 += d1;
    }
    dF[(size_t)b * kEmb + lane] = __float2bfloat16(df0);
    dF[(size_t)b * kEmb + 32 + lane] = __float2bfloat16(df1);
  }
  colF[w][lane] = df0;
  colF[w][32 + lane] = df1;
  colG[w][lane] = cg0;
  colG[w][32 + lane] = cg1;
  __syncthreads();
  const int t = threadIdx.x;
  if (t < 2 * kEmb) {
    const int c = t & (kEmb - 1);
    float(*col)[kEmb] = t < kEmb ? colF : colG;
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += col[k][c];
    (t < kEmb ? partF : partG)[(size_t)blockIdx.x * kEmb + c] = acc;
  }
}

// AdamW on fp32 master weights, refreshing their bf16 copies.
__global__ void adamw_kernel(float *__restrict__ w, __nv_bfloat16 *__restrict__ wb, const float *__restrict__ grad,
                             float *__restrict__ m, float *__restrict__ v, int n, float lr, float b1, float b2,
                             float eps, float wd, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / c1) / (sqrtf(vi / c2) + eps) + wd * w[i];
    const float wi = w[i] - lr * upd;
    w[i] = wi;
    if (wb) wb[i] = __float2bfloat16(wi);
  }
}

}  // namespace mptc
