// Training and embedding kernels of the learned candidate proposal (see
// learned_common.cuh for the model): tensor-core GEMM with transposes and
// fused bias/ReLU, feature builders, sampled softmax cross-entropy, AdamW.
#pragma once
#include "learned_common.cuh"

namespace mptc {

// C[M x N] = op(A)[M x K] * op(B)[K x N] (+ C) (+ bias) (ReLU), BF16 in, FP32
// accumulate. TA: A is stored K x M (row-major, lda); else M x K. TB: B is
// stored N x K; else K x N. Outputs: C (fp32) and/or Cb (bf16), row-major ldc.
// Tiles of 64 x 64 x 32; 4 warps, each 32 x 32 (2 x 4 mma tiles).
constexpr int kGBM = 64, kGBN = 64, kGBK = 32;

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) gemm_bf16_kernel(const __nv_bfloat16 *__restrict__ A, int lda,
                                                        const __nv_bfloat16 *__restrict__ B, int ldb,
                                                        float *__restrict__ C, __nv_bfloat16 *__restrict__ Cb,
                                                        int ldc, const float *__restrict__ bias, int M, int N, int K,
                                                        int relu, int accumulate) {
  __shared__ __align__(16) __nv_bfloat16 As[kGBM][kGBK + 8];
  __shared__ __align__(16) __nv_bfloat16 Bs[kGBN][kGBK + 8];  // stored [n][k]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int g = lane >> 2, t = lane & 3;
  const int m0 = blockIdx.y * kGBM, n0 = blockIdx.x * kGBN;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;
  const __nv_bfloat16 zero = __float2bfloat16(0.f);
  // split K (blockIdx.z): slice z writes its partial product to C + z * M * ldc
  const int ksplit = gridDim.z > 1 ? (K + gridDim.z - 1) / gridDim.z : K;
  const int kbeg = blockIdx.z * ((ksplit + kGBK - 1) / kGBK * kGBK);
  const int kend = min(K, kbeg + (ksplit + kGBK - 1) / kGBK * kGBK);
  for (int k0 = kbeg; k0 < kend; k0 += kGBK) {
    // tiles with k contiguous in memory move as 16-byte vectors when aligned
    const bool avec = !TA && (lda % 8 == 0) && (k0 + kGBK <= kend) && ((reinterpret_cast<uintptr_t>(A) & 15) == 0);
    const bool bvec = TB && (ldb % 8 == 0) && (k0 + kGBK <= kend) && ((reinterpret_cast<uintptr_t>(B) & 15) == 0);
    if (avec) {
      for (int e = tid; e < kGBM * kGBK / 8; e += 128) {
        const int r = e / (kGBK / 8), c = 8 * (e % (kGBK / 8)), m = m0 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (m < M) v = *reinterpret_cast<const uint4 *>(A + (size_t)m * lda + k0 + c);
        *reinterpret_cast<uint4 *>(&As[r][c]) = v;
      }
    } else {
      for (int e = tid; e < kGBM * kGBK; e += 128) {
        const int r = e / kGBK, c = e % kGBK, m = m0 + r, k = k0 + c;
        __nv_bfloat16 v = zero;
        if (m < M && k < kend) v = TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
        As[r][c] = v;
      }
    }
    if (bvec) {
      for (int e = tid; e < kGBN * kGBK / 8; e += 128) {
        const int r = e / (kGBK / 8), c = 8 * (e % (kGBK / 8)), n = n0 + r;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (n < N) v = *reinterpret_cast<const uint4 *>(B + (size_t)n * ldb + k0 + c);
        *reinterpret_cast<uint4 *>(&Bs[r][c]) = v;
      }
    } else {
      for (int e = tid; e < kGBN * kGBK; e += 128) {
        const int r = e / kGBK, c = e % kGBK, n = n0 + r, k = k0 + c;
        __nv_bfloat16 v = zero;
        if (n < N && k < kend) v = TB ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
        Bs[r][c] = v;
      }
    }
    __syncthreads();
#pragma unroll
    for (int ks = 0; ks < kGBK; ks += 16) {
      uint32_t af[2][4], bf[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r = wm + 16 * i + g, c = ks + 2 * t;
        af[i][0] = pack_bf16x2(As[r][c], As[r][c + 1]);
        af[i][1] = pack_bf16x2(As[r + 8][c], As[r + 8][c + 1]);
        af[i][2] = pack_bf16x2(As[r][c + 8], As[r][c + 9]);
        af[i][3] = pack_bf16x2(As[r + 8][c + 8], As[r + 8][c + 9]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int n = wn + 8 * j + g, c = ks + 2 * t;
        bf[j][0] = pack_bf16x2(Bs[n][c], Bs[n][c + 1]);
        bf[j][1] = pack_bf16x2(Bs[n][c + 8], Bs[n][c + 9]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16_16816(acc[i][j], af[i], bf[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int m = m0 + wm + 16 * i + g + (q >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * t + (q & 1);
        if (m >= M || n >= N) continue;
        float v = acc[i][j][q];
        if (gridDim.z > 1) {  // a K slice: its partial sum into slice z of C (no bias, ReLU or bf16 copy)
          C[(size_t)blockIdx.z * M * ldc + (size_t)m * ldc + n] = v;
          continue;
        }
        if (accumulate && C) v += C[(size_t)m * ldc + n];
        if (bias) v += bias[n];
        if (relu) v = v > 0.f ? v : 0.f;
        if (C) C[(size_t)m * ldc + n] = v;
        if (Cb) Cb[(size_t)m * ldc + n] = __float2bfloat16(v);
      }
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
