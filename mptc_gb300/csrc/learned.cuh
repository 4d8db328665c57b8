// Training and embedding kernels of the learned candidate proposal (see
// learned_common.cuh for the model): tensor-core GEMM with transposes and
// fused bias/ReLU, feature builders, sampled softmax cross-entropy, AdamW.
#pragma once
#include "learned_common.cuh"
#include "tc_sm100.cuh"

namespace mptc {

// C[M x N] = op(A)[M x K] * op(B)[K x N] (+ C) (+ bias) (ReLU) on the
// fifth-generation tensor cores, BF16 in, FP32 accumulate in TMEM. TA: A is
// stored K x M (row-major, lda), else M x K; TB: B is stored N x K, else
// K x N. Outputs: C (fp32) and/or Cb (bf16), row-major ldc. Split K
// (gridDim.z > 1): slice z writes its partial product to C + z * M * ldc, no
// bias, ReLU or bf16 copy; the caller sums the slices in order. Tiles of
// 128 x 128 (one TMEM lane per row), K in steps of 64: each operand tile is
// staged in shared memory in the 128-byte-swizzled K-major layout (rows of
// 64 K values); an operand whose K run is contiguous in memory (A not
// transposed, B transposed) moves as 16-byte vectors, the other is read 8
// rows (or columns) at a time along its contiguous dimension and goes into
// the tile's rows through a register transpose (stage_transposed). Thread 0
// issues 4 tcgen05.mma (K = 16 each) per step; the epilogue reads the
// accumulator with tcgen05.ld, warp w rows 32w .. .
constexpr int kTcBM = 128, kTcBN = 128, kTcBK = 64;

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

// Stages an operand whose rows (tile rows r = 0..127, index row0 + r < nrows)
// are contiguous along the other dimension: src[k][row0 + r] for k in
// [k0, kend), stride ld. Thread t takes the 8 x 8 block of K values
// k0 + 8 (t % 8) .. and rows 8 (t / 8) ..: eight 16-byte loads (one per K
// value), a register transpose (each output word one byte permutation of two
// input words) and eight 16-byte stores (one per tile row).
__device__ __forceinline__ void stage_transposed(uint8_t *tile, const __nv_bfloat16 *__restrict__ src, int ld,
                                                 int row0, int nrows, int k0, int kend, int tid) {
  const int kb = tid & 7, rb = tid >> 3;  // 8 K blocks x 16 row blocks
  const int r = 8 * rb, row = row0 + r;
  uint32_t w[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int k = k0 + 8 * kb + i;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (k < kend && row < nrows) v = load8_bf16(src + (size_t)k * ld + row, nrows - row);
    w[i][0] = v.x;
    w[i][1] = v.y;
    w[i][2] = v.z;
    w[i][3] = v.w;
  }
  // out[j][q] = (w[2q] element j, w[2q+1] element j): row r + j, K values 8 kb + 2q, + 1
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const uint32_t sel = (j & 1) ? 0x7632u : 0x5410u;
    const uint4 o = make_uint4(__byte_perm(w[0][j >> 1], w[1][j >> 1], sel), __byte_perm(w[2][j >> 1], w[3][j >> 1], sel),
                               __byte_perm(w[4][j >> 1], w[5][j >> 1], sel), __byte_perm(w[6][j >> 1], w[7][j >> 1], sel));
    *reinterpret_cast<uint4 *>(tile + tc::sw128_offset((uint32_t)(r + j), (uint32_t)kb)) = o;
  }
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_tc_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                                                      const __nv_bfloat16 *__restrict__ B, int ldb,
                                                      float *__restrict__ C, __nv_bfloat16 *__restrict__ Cb, int ldc,
                                                      const float *__restrict__ bias, int M, int N, int K, int relu,
                                                      int accumulate) {
  __shared__ __align__(1024) uint8_t sA[kTcBM * 128];
  __shared__ __align__(1024) uint8_t sB[kTcBN * 128];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ volatile uint32_t abort_flag;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.y * kTcBM, n0 = blockIdx.x * kTcBN;
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    abort_flag = 0;
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
  const uint4 zero4 = make_uint4(0u, 0u, 0u, 0u);
  uint32_t phase = 0;
  int steps = 0;
  for (int k0 = kbeg; k0 < kend; k0 += kTcBK, ++steps) {
    // A tile: row r = m0 + r, K values k0 .. k0 + 63
    if (!TA) {
      for (int e = tid; e < kTcBM * 8; e += 128) {
        const int r = e >> 3, c = e & 7, m = m0 + r, k = k0 + 8 * c;
        uint4 v = zero4;
        if (m < M && k < kend) v = load8_bf16(A + (size_t)m * lda + k, kend - k);
        *reinterpret_cast<uint4 *>(sA + tc::sw128_offset((uint32_t)r, (uint32_t)c)) = v;
      }
    } else {  // A stored K x M
      stage_transposed(sA, A, lda, m0, M, k0, kend, tid);
    }
    // B tile: row r = n0 + r, K values k0 .. k0 + 63
    if (TB) {  // B stored N x K
      for (int e = tid; e < kTcBN * 8; e += 128) {
        const int r = e >> 3, c = e & 7, n = n0 + r, k = k0 + 8 * c;
        uint4 v = zero4;
        if (n < N && k < kend) v = load8_bf16(B + (size_t)n * ldb + k, kend - k);
        *reinterpret_cast<uint4 *>(sB + tc::sw128_offset((uint32_t)r, (uint32_t)c)) = v;
      }
    } else {  // B stored K x N
      stage_transposed(sB, B, ldb, n0, N, k0, kend, tid);
    }
    tc::fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t a = tc::smem_addr(sA), b = tc::smem_addr(sB);
#pragma unroll
      for (int k = 0; k < 4; ++k)
        tc::mma_bf16(tmem, tc::desc_sw128(a + 32 * k), tc::desc_sw128(b + 32 * k), idesc, (steps > 0 || k > 0) ? 1u : 0u);
      tc::mma_commit(&bar);
    }
    // the MMAs have read the tiles before they are overwritten
    if (!tc::mbar_wait(&bar, phase, &abort_flag)) abort_flag = 1;
    phase ^= 1;
    tc::tc_fence_after();
  }
  // epilogue: this thread's row, 32 columns at a time
  const int m = m0 + 32 * warp + lane;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);
#pragma unroll 1
  for (int c0 = 0; c0 < kTcBN; c0 += 32) {
    float v[32];
    tc::tmem_ld32(lane_base + (uint32_t)c0, v);
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      const int n = n0 + c0 + j;
      if (n >= N) continue;
      float x = steps > 0 ? v[j] : 0.f;
      if (gridDim.z > 1) {  // a K slice: its partial sum into slice z of C (no bias, ReLU or bf16 copy)
        C[(size_t)blockIdx.z * M * ldc + (size_t)m * ldc + n] = x;
        continue;
      }
      if (accumulate && C) x += C[(size_t)m * ldc + n];
      if (bias) x += bias[n];
      if (relu) x = x > 0.f ? x : 0.f;
      if (C) C[(size_t)m * ldc + n] = x;
      if (Cb) Cb[(size_t)m * ldc + n] = __float2bfloat16(x);
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

// ReLU backward in place: d *= (h > 0).
__global__ void relu_backward_kernel(float *__restrict__ d, const float *__restrict__ h, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (!(h[i] > 0.f)) d[i] = 0.f;
}

// Transposed bf16 copy: y[c][r] = bf16(x[r][c]) for an R x C fp32 matrix.
__global__ void transpose_bf16_kernel(const float *__restrict__ x, int R, int C, __nv_bfloat16 *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R * C; i += gridDim.x * blockDim.x) {
    const int r = i / C, c = i - r * C;
    y[(size_t)c * R + r] = __float2bfloat16(x[i]);
  }
}

__global__ void bf16_to_f32_kernel(const __nv_bfloat16 *__restrict__ x, float *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = __bfloat162float(x[i]);
}

__global__ void to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = __float2bfloat16(x[i]);
}

// Partial column sums of d [rows x cols]: slice blockIdx.y sums rows y,
// y + gridDim.y, ... into part[y * cols + c].
__global__ void colsum_kernel(const float *__restrict__ d, int rows, int cols, float *__restrict__ part) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = blockIdx.y; r < rows; r += gridDim.y) s += d[(size_t)r * cols + c];
  part[(size_t)blockIdx.y * cols + c] = s;
}

// out[i] = sum over slices k = 0 .. slices-1 of part[k * n + i], in slice
// order (the same bits on every run).
__global__ void slice_sum_kernel(const float *__restrict__ part, int slices, int n, float *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < slices; ++k) s += part[(size_t)k * n + i];
    out[i] = s;
  }
}

constexpr int kMaxCE = 64;  // candidates per block in one training example

// Sampled softmax cross-entropy: block b scores its C candidates (row b*C .. of
// G) against F[b]; candidate 0 is the accepted one. Writes the mean loss
// (atomic) and dF [B x 64], dG [B*C x 64]. One warp per block, lane = dim pair.
__global__ void softmax_ce_kernel(const float *__restrict__ F, const float *__restrict__ G, int B, int C,
                                  float *__restrict__ dF, float *__restrict__ dG, float *__restrict__ loss) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= B) return;
  const float f0 = F[(size_t)warp * kEmb + lane], f1 = F[(size_t)warp * kEmb + 32 + lane];
  float s[kMaxCE];
  float mx = -1e30f;
  for (int j = 0; j < C; ++j) {  // score = F[b] . G[b, j], warp sum of per-lane partials
    const float *g = G + ((size_t)warp * C + j) * kEmb;
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
  float df0 = 0.f, df1 = 0.f;
  for (int j = 0; j < C; ++j) {
    const float p = __expf(s[j] - mx) * inv;
    const float ds = (p - (j == 0 ? 1.f : 0.f)) / B;
    const float *g = G + ((size_t)warp * C + j) * kEmb;
    df0 += ds * g[lane];
    df1 += ds * g[32 + lane];
    float *dg = dG + ((size_t)warp * C + j) * kEmb;
    dg[lane] = ds * f0;
    dg[32 + lane] = ds * f1;
  }
  dF[(size_t)warp * kEmb + lane] = df0;
  dF[(size_t)warp * kEmb + 32 + lane] = df1;
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
