// Learned proposal model: parameters, training step (forward, sampled softmax
// cross-entropy, backward, AdamW; kernels of learned.cuh), the packed bf16
// weight image the tensor-core inference kernels stage by TMA, and the
// launchers of those embedding kernels (learned_tc.cuh). C ABI in
// include/mptc_gb300.h.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mptc_gb300.h"
#include <mutex>

#include "learned.cuh"
#include "learned_embed.cuh"
#include "model_internal.h"

namespace {

using bf16 = __nv_bfloat16;

// Parameter blocks, in the order of the flat parameter vector.
struct Layer {
  int in, out;  // weight [in x out] (row-major: y = x W + b)
};
constexpr Layer kLayers[5] = {{mptc::kFeatPad, mptc::kH1}, {mptc::kH1, mptc::kH2}, {mptc::kH2, mptc::kEmb},
                              {mptc::kCandIn, mptc::kCandH}, {mptc::kCandH, mptc::kEmb}};

struct Offsets {
  size_t w[5], b[5], total;
  Offsets() {
    size_t o = 0;
    for (int l = 0; l < 5; ++l) {
      w[l] = o;
      o += (size_t)kLayers[l].in * kLayers[l].out;
      b[l] = o;
      o += (size_t)kLayers[l].out;
    }
    total = o;
  }
};
const Offsets kOff;

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

template <typename T>
cudaError_t dmalloc(T **p, size_t n) {
  return cudaMalloc(reinterpret_cast<void **>(p), (n ? n : 1) * sizeof(T));
}

}  // namespace

struct mptc_model {
  float *w = nullptr;   // fp32 master parameters
  bf16 *wb = nullptr;   // bf16 copy (same layout)
  float *g = nullptr;   // gradients
  float *m = nullptr, *v = nullptr;  // AdamW moments
  int64_t step = 0;
  // training workspace (grown on demand)
  int cap_b = 0, cap_bc = 0;
  bf16 *x = nullptr, *h1b = nullptr, *h2b = nullptr, *xc = nullptr, *g1b = nullptr;
  float *h1 = nullptr, *h2 = nullptr, *f = nullptr, *g1 = nullptr, *gg = nullptr;
  float *df = nullptr, *dgg = nullptr, *dh1 = nullptr, *dh2 = nullptr, *dg1 = nullptr;
  bf16 *dfb = nullptr, *dggb = nullptr, *dh1b = nullptr, *dh2b = nullptr, *dg1b = nullptr;
  float *loss = nullptr;
  // packed bf16 weight image of the inference kernels (refreshed after every
  // parameter change) and a bf16 staging buffer for mptc_model_embed
  uint8_t *img = nullptr;
  __nv_bfloat16 *emb_tmp = nullptr;
  int emb_cap = 0;
  uint32_t *status = nullptr;
  float *part = nullptr;  // partial sums of the split gradient reductions
};

namespace {

void free_ws(mptc_model *m) {
  void *ps[] = {m->x, m->h1b, m->h2b, m->xc, m->g1b, m->h1, m->h2, m->f, m->g1, m->gg,
                m->df, m->dgg, m->dh1, m->dh2, m->dg1, m->dfb, m->dggb, m->dh1b, m->dh2b, m->dg1b};
  for (void *p : ps) cudaFree(p);
  m->x = m->h1b = m->h2b = m->xc = m->g1b = nullptr;
  m->h1 = m->h2 = m->f = m->g1 = m->gg = m->df = m->dgg = m->dh1 = m->dh2 = m->dg1 = nullptr;
  m->dfb = m->dggb = m->dh1b = m->dh2b = m->dg1b = nullptr;
  m->cap_b = m->cap_bc = 0;
}

mptc_status ensure_ws(mptc_model *m, int B, int BC) {
  if (B <= m->cap_b && BC <= m->cap_bc) return MPTC_OK;
  free_ws(m);
  using namespace mptc;
  bool bad = dmalloc(&m->x, (size_t)B * kFeatPad) || dmalloc(&m->h1b, (size_t)B * kH1) ||
             dmalloc(&m->h2b, (size_t)B * kH2) || dmalloc(&m->xc, (size_t)BC * kCandIn) ||
             dmalloc(&m->g1b, (size_t)BC * kCandH) || dmalloc(&m->h1, (size_t)B * kH1) ||
             dmalloc(&m->h2, (size_t)B * kH2) || dmalloc(&m->f, (size_t)B * kEmb) ||
             dmalloc(&m->g1, (size_t)BC * kCandH) || dmalloc(&m->gg, (size_t)BC * kEmb) ||
             dmalloc(&m->df, (size_t)B * kEmb) || dmalloc(&m->dgg, (size_t)BC * kEmb) ||
             dmalloc(&m->dh1, (size_t)B * kH1) || dmalloc(&m->dh2, (size_t)B * kH2) ||
             dmalloc(&m->dg1, (size_t)BC * kCandH) || dmalloc(&m->dfb, (size_t)B * kEmb) ||
             dmalloc(&m->dggb, (size_t)BC * kEmb) || dmalloc(&m->dh1b, (size_t)B * kH1) ||
             dmalloc(&m->dh2b, (size_t)B * kH2) || dmalloc(&m->dg1b, (size_t)BC * kCandH);
  if (bad) {
    free_ws(m);
    return MPTC_ENOMEM;
  }
  m->cap_b = B;
  m->cap_bc = BC;
  return MPTC_OK;
}

int blocks_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

// y[M x N] = x[M x K] W + b (opt. ReLU), outputs fp32 and bf16.
void gemm_fwd(const bf16 *x, const bf16 *W, const float *b, float *y, bf16 *yb, int M, int K, int N, bool relu,
              cudaStream_t s) {
  dim3 grid((N + mptc::kTcBN - 1) / mptc::kTcBN, (M + mptc::kTcBM - 1) / mptc::kTcBM);
  mptc::gemm_tc_kernel<false, false><<<grid, 128, 0, s>>>(x, K, W, N, y, yb, N, b, M, N, K, relu ? 1 : 0, 0);
}

// Partial sums of the split reductions below (slices x outputs floats).
constexpr size_t kPartFloats = 1 << 20;

// dW[K x N] = x^T[K x M] dy[M x N]: few outputs and a long reduction over the
// M examples, so the reduction is split into slices of about 2048 rows whose
// partial products are summed in slice order afterwards (deterministic).
void gemm_dw(const bf16 *x, const bf16 *dy, float *dW, int M, int K, int N, float *part, cudaStream_t s) {
  const int splits = (int)std::min<size_t>(std::min(64, std::max(1, M / 2048)), kPartFloats / ((size_t)K * N));
  dim3 grid((N + mptc::kTcBN - 1) / mptc::kTcBN, (K + mptc::kTcBM - 1) / mptc::kTcBM, std::max(1, splits));
  mptc::gemm_tc_kernel<true, false><<<grid, 128, 0, s>>>(x, K, dy, N, splits > 1 ? part : dW, nullptr, N, nullptr, K, N,
                                                        M, 0, 0);
  if (splits > 1) mptc::slice_sum_kernel<<<blocks_for((size_t)K * N), 256, 0, s>>>(part, splits, K * N, dW);
}

// Bias gradient db[cols] = column sums of d[rows x cols].
void colsum(const float *d, int rows, int cols, float *db, float *part, cudaStream_t s) {
  const int slices = (int)std::min<size_t>(std::min(512, std::max(1, rows / 64)), kPartFloats / cols);
  dim3 grid((cols + 127) / 128, slices);
  mptc::colsum_kernel<<<grid, 128, 0, s>>>(d, rows, cols, part);
  mptc::slice_sum_kernel<<<blocks_for((size_t)cols), 256, 0, s>>>(part, slices, cols, db);
}

// dx[M x K] = dy[M x N] W^T  (W stored K x N, i.e. "N x K" transposed access)
void gemm_dx(const bf16 *dy, const bf16 *W, float *dx, int M, int K, int N, cudaStream_t s) {
  dim3 grid((K + mptc::kTcBN - 1) / mptc::kTcBN, (M + mptc::kTcBM - 1) / mptc::kTcBM);
  mptc::gemm_tc_kernel<false, true><<<grid, 128, 0, s>>>(dy, N, W, N, dx, nullptr, K, nullptr, M, K, N, 0, 0);
}

// Forward through both MLPs for a training batch; then, if `grads`, the loss
// gradient into m->g.
mptc_status forward_backward(mptc_model *m, const uint8_t *rgb, int width, int bw, const uint64_t *stb,
                             const uint32_t *blocks, const uint32_t *cands, int B, int C, bool grads, cudaStream_t s) {
  using namespace mptc;
  const int BC = B * C;
  mptc_status st = ensure_ws(m, B, BC);
  if (st != MPTC_OK) return st;
  const bf16 *W[5];
  const float *b[5];
  for (int l = 0; l < 5; ++l) {
    W[l] = m->wb + kOff.w[l];
    b[l] = m->w + kOff.b[l];
  }
  block_features_kernel<<<blocks_for((size_t)B * kFeatPad), 256, 0, s>>>(rgb, width, bw, stb, blocks, B, m->x);
  gemm_fwd(m->x, W[0], b[0], m->h1, m->h1b, B, kFeatPad, kH1, true, s);
  gemm_fwd(m->h1b, W[1], b[1], m->h2, m->h2b, B, kH1, kH2, true, s);
  gemm_fwd(m->h2b, W[2], b[2], m->f, nullptr, B, kH2, kEmb, false, s);
  cand_features_kernel<<<blocks_for((size_t)BC * kCandIn), 256, 0, s>>>(cands, 1, BC, m->xc);
  gemm_fwd(m->xc, W[3], b[3], m->g1, m->g1b, BC, kCandIn, kCandH, true, s);
  gemm_fwd(m->g1b, W[4], b[4], m->gg, nullptr, BC, kCandH, kEmb, false, s);
  cudaMemsetAsync(m->loss, 0, sizeof(float), s);
  softmax_ce_kernel<<<(B * 32 + 255) / 256, 256, 0, s>>>(m->f, m->gg, B, C, m->df, m->dgg, m->loss);
  if (!grads) return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
  float *G[5], *Gb[5];
  for (int l = 0; l < 5; ++l) {
    G[l] = m->g + kOff.w[l];
    Gb[l] = m->g + kOff.b[l];
  }
  // block MLP
  to_bf16_kernel<<<blocks_for((size_t)B * kEmb), 256, 0, s>>>(m->df, m->dfb, B * kEmb);
  gemm_dw(m->h2b, m->dfb, G[2], B, kH2, kEmb, m->part, s);
  colsum(m->df, B, kEmb, Gb[2], m->part, s);
  gemm_dx(m->dfb, W[2], m->dh2, B, kH2, kEmb, s);
  relu_backward_kernel<<<blocks_for((size_t)B * kH2), 256, 0, s>>>(m->dh2, m->h2, B * kH2);
  to_bf16_kernel<<<blocks_for((size_t)B * kH2), 256, 0, s>>>(m->dh2, m->dh2b, B * kH2);
  gemm_dw(m->h1b, m->dh2b, G[1], B, kH1, kH2, m->part, s);
  colsum(m->dh2, B, kH2, Gb[1], m->part, s);
  gemm_dx(m->dh2b, W[1], m->dh1, B, kH1, kH2, s);
  relu_backward_kernel<<<blocks_for((size_t)B * kH1), 256, 0, s>>>(m->dh1, m->h1, B * kH1);
  to_bf16_kernel<<<blocks_for((size_t)B * kH1), 256, 0, s>>>(m->dh1, m->dh1b, B * kH1);
  gemm_dw(m->x, m->dh1b, G[0], B, kFeatPad, kH1, m->part, s);
  colsum(m->dh1, B, kH1, Gb[0], m->part, s);
  // candidate MLP
  to_bf16_kernel<<<blocks_for((size_t)BC * kEmb), 256, 0, s>>>(m->dgg, m->dggb, BC * kEmb);
  gemm_dw(m->g1b, m->dggb, G[4], BC, kCandH, kEmb, m->part, s);
  colsum(m->dgg, BC, kEmb, Gb[4], m->part, s);
  gemm_dx(m->dggb, W[4], m->dg1, BC, kCandH, kEmb, s);
  relu_backward_kernel<<<blocks_for((size_t)BC * kCandH), 256, 0, s>>>(m->dg1, m->g1, BC * kCandH);
  to_bf16_kernel<<<blocks_for((size_t)BC * kCandH), 256, 0, s>>>(m->dg1, m->dg1b, BC * kCandH);
  gemm_dw(m->xc, m->dg1b, G[3], BC, kCandIn, kCandH, m->part, s);
  colsum(m->dg1, BC, kCandH, Gb[3], m->part, s);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

// Refreshes the packed bf16 weight image from the fp32 master weights.
void repack(mptc_model *m, cudaStream_t s) {
  const uint32_t img_off[5] = {mptc::kImgF1, mptc::kImgF2, mptc::kImgF3, mptc::kImgG1, mptc::kImgG2};
  for (int l = 0; l < 5; ++l) {
    const int kpad = (kLayers[l].in + 63) / 64 * 64;
    mptc::pack_layer_kernel<<<blocks_for((size_t)kpad * kLayers[l].out), 256, 0, s>>>(
        m->w + kOff.w[l], kLayers[l].in, kLayers[l].out, kpad, m->img + img_off[l]);
  }
}

// Dynamic shared memory of the embedding kernels, set once per device. The f
// kernel needs all but 2 KB of an SM's shared memory (one CTA per SM, its
// 512 TMEM columns); the g kernel asks for 80 KB so that at most two CTAs
// (256 TMEM columns each) share an SM.
constexpr int kMaxDev = 64;
std::mutex g_attr_mu;
bool g_attr_done[kMaxDev] = {};
constexpr size_t kSmemF = mptc::embed_smem_bytes<mptc::NetF>();
constexpr size_t kSmemG = mptc::embed_smem_bytes<mptc::NetG>() > 81920 ? mptc::embed_smem_bytes<mptc::NetG>() : 81920;

cudaError_t ensure_embed_attrs() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDev) return e != cudaSuccess ? e : cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_attr_mu);
  if (g_attr_done[dev]) return cudaSuccess;
  e = cudaFuncSetAttribute(mptc::embed_kernel<mptc::NetF, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)kSmemF);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(mptc::embed_kernel<mptc::NetG, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kSmemG);
  if (e == cudaSuccess) g_attr_done[dev] = true;
  return e;
}

int sm_count_now() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

}  // namespace

namespace mptc_internal {

mptc_status model_embed(const mptc_model *m, bool blocks, const EmbedJob *jobs, int n_jobs, uint32_t *next,
                        cudaStream_t s) {
  if (!m || !jobs || n_jobs <= 0 || n_jobs > mptc::kMaxBatch || !next) return MPTC_EINVAL;
  if (ensure_embed_attrs() != cudaSuccess) return MPTC_ECUDA;
  mptc::EmbedBatch b{};
  b.n = n_jobs;
  b.next = next;
  int tiles = 0;
  const int l0 = blocks ? 0 : 3;
  for (int j = 0; j < n_jobs; ++j) {
    const EmbedJob &J = jobs[j];
    mptc::EmbedArgs &a = b.a[j];
    a.rgb = J.rgb;
    a.width = J.width;
    a.bw = J.width / 4;
    a.n = J.n;
    a.stb = J.stb;
    a.blocks = J.blocks;
    a.words = J.words;
    a.word_stride = J.word_stride;
    a.wimg = m->img;
    a.b1 = m->w + kOff.b[l0];
    a.b2 = m->w + kOff.b[l0 + 1];
    a.b3 = blocks ? m->w + kOff.b[2] : nullptr;
    a.out = J.out;
    a.status = J.status ? J.status : m->status;
    tiles += (J.n + 127) / 128;
    b.tile_end[j] = tiles;
  }
  if (tiles == 0) return MPTC_OK;
  const int sms = sm_count_now();
  if (blocks)
    mptc::embed_kernel<mptc::NetF, true><<<std::min(tiles, sms), mptc::kEmbedThreads, kSmemF, s>>>(b);
  else
    mptc::embed_kernel<mptc::NetG, false><<<std::min(tiles, 2 * sms), mptc::kEmbedThreads, kSmemG, s>>>(b);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

}  // namespace mptc_internal

extern "C" {

int64_t mptc_model_num_params(void) { return (int64_t)kOff.total; }

mptc_status mptc_model_create(uint64_t seed, mptc_model **out) {
  if (!out) return MPTC_EINVAL;
  *out = nullptr;
  mptc_model *m = new (std::nothrow) mptc_model();
  if (!m) return MPTC_ENOMEM;
  const size_t n = kOff.total;
  if (dmalloc(&m->w, n) || dmalloc(&m->wb, n) || dmalloc(&m->g, n) || dmalloc(&m->m, n) || dmalloc(&m->v, n) ||
      dmalloc(&m->loss, 1) || dmalloc(&m->img, mptc::kImgBytes) || dmalloc(&m->status, 4) || dmalloc(&m->part, kPartFloats) ||
      cudaMemset(m->img, 0, mptc::kImgBytes) != cudaSuccess || cudaMemset(m->status, 0, 16) != cudaSuccess) {
    mptc_model_destroy(m);
    return MPTC_ENOMEM;
  }
  // He-uniform weights from a seeded generator, zero biases; the padded
  // feature rows of the first layer start (and stay) at zero.
  std::vector<float> h(n, 0.f);
  uint64_t s = seed;
  for (int l = 0; l < 5; ++l) {
    const int fan_in = l == 0 ? mptc::kFeatIn : kLayers[l].in;
    const float lim = std::sqrt(6.0f / (float)fan_in);
    for (int i = 0; i < kLayers[l].in; ++i)
      for (int o = 0; o < kLayers[l].out; ++o) {
        const double u = (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
        const bool pad = l == 0 && i >= mptc::kFeatIn;
        h[kOff.w[l] + (size_t)i * kLayers[l].out + o] = pad ? 0.f : (float)((2.0 * u - 1.0) * lim);
      }
  }
  mptc_status st = mptc_model_set_params(m, h.data());
  if (st != MPTC_OK) {
    mptc_model_destroy(m);
    return st;
  }
  cudaMemset(m->m, 0, n * sizeof(float));
  cudaMemset(m->v, 0, n * sizeof(float));
  *out = m;
  return MPTC_OK;
}

mptc_status mptc_model_destroy(mptc_model *m) {
  if (!m) return MPTC_EINVAL;
  free_ws(m);
  cudaFree(m->w);
  cudaFree(m->wb);
  cudaFree(m->g);
  cudaFree(m->m);
  cudaFree(m->v);
  cudaFree(m->loss);
  cudaFree(m->img);
  cudaFree(m->emb_tmp);
  cudaFree(m->status);
  cudaFree(m->part);
  delete m;
  return MPTC_OK;
}

mptc_status mptc_model_set_params(mptc_model *m, const float *host) {
  if (!m || !host) return MPTC_EINVAL;
  const size_t n = kOff.total;
  if (cudaMemcpy(m->w, host, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return MPTC_ECUDA;
  mptc::to_bf16_kernel<<<blocks_for(n), 256>>>(m->w, m->wb, (int)n);
  repack(m, nullptr);
  return cudaDeviceSynchronize() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

mptc_status mptc_model_get_params(mptc_model *m, float *host) {
  if (!m || !host) return MPTC_EINVAL;
  return cudaMemcpy(host, m->w, kOff.total * sizeof(float), cudaMemcpyDeviceToHost) == cudaSuccess ? MPTC_OK
                                                                                                  : MPTC_ECUDA;
}

mptc_status mptc_model_grads(mptc_model *m, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                             const uint32_t *blocks_dev, const uint32_t *cands_dev, int32_t B, int32_t C,
                             float *grads_host, float *loss_host, void *stream) {
  if (!m || !rgb_dev || !stb_dev || !blocks_dev || !cands_dev || B <= 0 || C < 2 || C > mptc::kMaxCE ||
      width <= 0 || (width & 3))
    return MPTC_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mptc_status st = forward_backward(m, rgb_dev, width, width / 4, stb_dev, blocks_dev, cands_dev, B, C,
                                    grads_host != nullptr, s);
  if (st != MPTC_OK) return st;
  if (cudaStreamSynchronize(s) != cudaSuccess) return MPTC_ECUDA;
  if (grads_host && cudaMemcpy(grads_host, m->g, kOff.total * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return MPTC_ECUDA;
  if (loss_host && cudaMemcpy(loss_host, m->loss, sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
    return MPTC_ECUDA;
  return MPTC_OK;
}

mptc_status mptc_model_train_step(mptc_model *m, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                                  const uint32_t *blocks_dev, const uint32_t *cands_dev, int32_t B, int32_t C,
                                  float lr, float weight_decay, float *loss_host, void *stream) {
  if (!m || !rgb_dev || !stb_dev || !blocks_dev || !cands_dev || B <= 0 || C < 2 || C > mptc::kMaxCE ||
      width <= 0 || (width & 3) || !(lr > 0.f))
    return MPTC_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  mptc_status st = forward_backward(m, rgb_dev, width, width / 4, stb_dev, blocks_dev, cands_dev, B, C, true, s);
  if (st != MPTC_OK) return st;
  m->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - (float)std::pow(b1, (double)m->step), c2 = 1.f - (float)std::pow(b2, (double)m->step);
  const size_t n = kOff.total;
  mptc::adamw_kernel<<<blocks_for(n), 256, 0, s>>>(m->w, m->wb, m->g, m->m, m->v, (int)n, lr, b1, b2, 1e-8f,
                                                   weight_decay, c1, c2);
  repack(m, s);
  if (cudaGetLastError() != cudaSuccess) return MPTC_ECUDA;
  if (loss_host) {
    if (cudaMemcpyAsync(loss_host, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return MPTC_ECUDA;
  }
  return MPTC_OK;
}

mptc_status mptc_model_save(mptc_model *m, const char *path) {
  if (!m || !path) return MPTC_EINVAL;
  const size_t n = kOff.total;
  std::vector<float> buf(3 * n);
  if (cudaMemcpy(buf.data(), m->w, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(buf.data() + n, m->m, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(buf.data() + 2 * n, m->v, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return MPTC_ECUDA;
  FILE *f = std::fopen(path, "wb");
  if (!f) return MPTC_EINVAL;
  const char magic[8] = {'M', 'P', 'T', 'C', 'M', 'L', 'P', '1'};
  const int64_t hdr[2] = {(int64_t)n, m->step};
  bool ok = std::fwrite(magic, 1, 8, f) == 8 && std::fwrite(hdr, 8, 2, f) == 2 &&
            std::fwrite(buf.data(), 4, buf.size(), f) == buf.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? MPTC_OK : MPTC_EINVAL;
}

mptc_status mptc_model_load(mptc_model *m, const char *path) {
  if (!m || !path) return MPTC_EINVAL;
  FILE *f = std::fopen(path, "rb");
  if (!f) return MPTC_EINVAL;
  char magic[8];
  int64_t hdr[2];
  const size_t n = kOff.total;
  std::vector<float> buf(3 * n);
  bool ok = std::fread(magic, 1, 8, f) == 8 && std::memcmp(magic, "MPTCMLP1", 8) == 0 &&
            std::fread(hdr, 8, 2, f) == 2 && hdr[0] == (int64_t)n && std::fread(buf.data(), 4, buf.size(), f) == buf.size();
  std::fclose(f);
  if (!ok) return MPTC_EINVAL;
  mptc_status st = mptc_model_set_params(m, buf.data());
  if (st != MPTC_OK) return st;
  if (cudaMemcpy(m->m, buf.data() + n, n * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(m->v, buf.data() + 2 * n, n * 4, cudaMemcpyHostToDevice) != cudaSuccess)
    return MPTC_ECUDA;
  m->step = hdr[1];
  return MPTC_OK;
}

// Embeddings through the inference kernels (tcgen05, bf16 out) converted to
// fp32: F = f(block features) for `n_blocks` blocks (blocks_dev NULL = the
// first n_blocks blocks in raster order), G = g(words).
mptc_status mptc_model_embed(mptc_model *m, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                             const uint32_t *blocks_dev, int32_t n_blocks, float *emb_blocks_dev,
                             const uint32_t *words_dev, int32_t word_stride, int32_t n_words, float *emb_words_dev,
                             void *stream) {
  if (!m || (n_blocks > 0 && (!rgb_dev || !stb_dev || !emb_blocks_dev || width <= 0 || (width & 3))) ||
      (n_words > 0 && (!words_dev || !emb_words_dev || word_stride < 1)))
    return MPTC_EINVAL;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int need = std::max(n_blocks, n_words);
  if (need <= 0) return MPTC_OK;
  if (need > m->emb_cap) {
    cudaFree(m->emb_tmp);
    m->emb_tmp = nullptr;
    m->emb_cap = 0;
    if (dmalloc(&m->emb_tmp, (size_t)need * mptc::kEmb)) return MPTC_ENOMEM;
    m->emb_cap = need;
  }
  if (cudaMemsetAsync(m->status, 0, 16, s) != cudaSuccess) return MPTC_ECUDA;
  mptc_status st = MPTC_OK;
  if (n_blocks > 0) {
    mptc_internal::EmbedJob j;
    j.rgb = rgb_dev;
    j.width = width;
    j.stb = stb_dev;
    j.blocks = blocks_dev;
    j.n = n_blocks;
    j.out = m->emb_tmp;
    st = mptc_internal::model_embed(m, true, &j, 1, m->status + 1, s);
    if (st != MPTC_OK) return st;
    mptc::bf16_to_f32_kernel<<<blocks_for((size_t)n_blocks * mptc::kEmb), 256, 0, s>>>(m->emb_tmp, emb_blocks_dev,
                                                                                      n_blocks * mptc::kEmb);
  }
  if (n_words > 0) {
    mptc_internal::EmbedJob j;
    j.words = words_dev;
    j.word_stride = word_stride;
    j.n = n_words;
    j.out = m->emb_tmp;
    st = mptc_internal::model_embed(m, false, &j, 1, m->status + 2, s);
    if (st != MPTC_OK) return st;
    mptc::bf16_to_f32_kernel<<<blocks_for((size_t)n_words * mptc::kEmb), 256, 0, s>>>(m->emb_tmp, emb_words_dev,
                                                                                     n_words * mptc::kEmb);
  }
  uint32_t flag = 0;
  if (cudaMemcpyAsync(&flag, m->status, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MPTC_ECUDA;
  return flag ? MPTC_ETIMEOUT : (cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA);
}

}  // extern "C"
