// Learned proposal model: parameters, training step (forward, sampled softmax
// cross-entropy, backward, AdamW) and inference embeddings, all on the GPU in
// the kernels of learned.cuh. C ABI in include/mptc_gb300.h.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/mptc_gb300.h"
#include "learned.cuh"
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
  dim3 grid((N + mptc::kGBN - 1) / mptc::kGBN, (M + mptc::kGBM - 1) / mptc::kGBM);
  mptc::gemm_bf16_kernel<false, false><<<grid, 128, 0, s>>>(x, K, W, N, y, yb, N, b, M, N, K, relu ? 1 : 0, 0);
}

// dW[K x N] = x^T[K x M] dy[M x N]
void gemm_dw(const bf16 *x, const bf16 *dy, float *dW, int M, int K, int N, cudaStream_t s) {
  dim3 grid((N + mptc::kGBN - 1) / mptc::kGBN, (K + mptc::kGBM - 1) / mptc::kGBM);
  mptc::gemm_bf16_kernel<true, false><<<grid, 128, 0, s>>>(x, K, dy, N, dW, nullptr, N, nullptr, K, N, M, 0, 0);
}

// dx[M x K] = dy[M x N] W^T  (W stored K x N, i.e. "N x K" transposed access)
void gemm_dx(const bf16 *dy, const bf16 *W, float *dx, int M, int K, int N, cudaStream_t s) {
  dim3 grid((K + mptc::kGBN - 1) / mptc::kGBN, (M + mptc::kGBM - 1) / mptc::kGBM);
  mptc::gemm_bf16_kernel<false, true><<<grid, 128, 0, s>>>(dy, N, W, N, dx, nullptr, K, nullptr, M, K, N, 0, 0);
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
  gemm_dw(m->h2b, m->dfb, G[2], B, kH2, kEmb, s);
  colsum_kernel<<<1, kEmb, 0, s>>>(m->df, B, kEmb, Gb[2]);
  gemm_dx(m->dfb, W[2], m->dh2, B, kH2, kEmb, s);
  relu_backward_kernel<<<blocks_for((size_t)B * kH2), 256, 0, s>>>(m->dh2, m->h2, B * kH2);
  to_bf16_kernel<<<blocks_for((size_t)B * kH2), 256, 0, s>>>(m->dh2, m->dh2b, B * kH2);
  gemm_dw(m->h1b, m->dh2b, G[1], B, kH1, kH2, s);
  colsum_kernel<<<1, kH2, 0, s>>>(m->dh2, B, kH2, Gb[1]);
  gemm_dx(m->dh2b, W[1], m->dh1, B, kH1, kH2, s);
  relu_backward_kernel<<<blocks_for((size_t)B * kH1), 256, 0, s>>>(m->dh1, m->h1, B * kH1);
  to_bf16_kernel<<<blocks_for((size_t)B * kH1), 256, 0, s>>>(m->dh1, m->dh1b, B * kH1);
  gemm_dw(m->x, m->dh1b, G[0], B, kFeatPad, kH1, s);
  colsum_kernel<<<1, kH1, 0, s>>>(m->dh1, B, kH1, Gb[0]);
  // candidate MLP
  to_bf16_kernel<<<blocks_for((size_t)BC * kEmb), 256, 0, s>>>(m->dgg, m->dggb, BC * kEmb);
  gemm_dw(m->g1b, m->dggb, G[4], BC, kCandH, kEmb, s);
  colsum_kernel<<<1, kEmb, 0, s>>>(m->dgg, BC, kEmb, Gb[4]);
  gemm_dx(m->dggb, W[4], m->dg1, BC, kCandH, kEmb, s);
  relu_backward_kernel<<<blocks_for((size_t)BC * kCandH), 256, 0, s>>>(m->dg1, m->g1, BC * kCandH);
  to_bf16_kernel<<<blocks_for((size_t)BC * kCandH), 256, 0, s>>>(m->dg1, m->dg1b, BC * kCandH);
  gemm_dw(m->xc, m->dg1b, G[3], BC, kCandIn, kCandH, s);
  colsum_kernel<<<1, kCandH, 0, s>>>(m->dg1, BC, kCandH, Gb[3]);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

}  // namespace

extern "C" {

int64_t mptc_model_num_params(void) { return (int64_t)kOff.total; }

mptc_status mptc_model_create(uint64_t seed, mptc_model **out) {
  if (!out) return MPTC_EINVAL;
  *out = nullptr;
  mptc_model *m = new (std::nothrow) mptc_model();
  if (!m) return MPTC_ENOMEM;
  const size_t n = kOff.total;
  if (dmalloc(&m->w, n) || dmalloc(&m->wb, n) || dmalloc(&m->g, n) || dmalloc(&m->m, n) || dmalloc(&m->v, n) ||
      dmalloc(&m->loss, 1)) {
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
  delete m;
  return MPTC_OK;
}

mptc_status mptc_model_set_params(mptc_model *m, const float *host) {
  if (!m || !host) return MPTC_EINVAL;
  const size_t n = kOff.total;
  if (cudaMemcpy(m->w, host, n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) return MPTC_ECUDA;
  mptc::to_bf16_kernel<<<blocks_for(n), 256>>>(m->w, m->wb, (int)n);
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

// Embeddings for inference and tests: F = f(block features) for `n` blocks
// (blocks_dev NULL = all blocks of the frame in raster order), G = g(words).
mptc_status mptc_model_embed(mptc_model *m, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                             const uint32_t *blocks_dev, int32_t n_blocks, float *emb_blocks_dev,
                             const uint32_t *words_dev, int32_t word_stride, int32_t n_words, float *emb_words_dev,
                             void *stream) {
  if (!m || (n_blocks > 0 && (!rgb_dev || !stb_dev || !emb_blocks_dev)) || (n_words > 0 && (!words_dev || !emb_words_dev)))
    return MPTC_EINVAL;
  using namespace mptc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int B = n_blocks > 0 ? n_blocks : 0, BC = n_words > 0 ? n_words : 0;
  mptc_status st = ensure_ws(m, B > 0 ? B : 1, BC > 0 ? BC : 1);
  if (st != MPTC_OK) return st;
  const bf16 *W[5];
  const float *b[5];
  for (int l = 0; l < 5; ++l) {
    W[l] = m->wb + kOff.w[l];
    b[l] = m->w + kOff.b[l];
  }
  if (B > 0) {
    block_features_kernel<<<blocks_for((size_t)B * kFeatPad), 256, 0, s>>>(rgb_dev, width, width / 4, stb_dev,
                                                                           blocks_dev, B, m->x);
    gemm_fwd(m->x, W[0], b[0], m->h1, m->h1b, B, kFeatPad, kH1, true, s);
    gemm_fwd(m->h1b, W[1], b[1], m->h2, m->h2b, B, kH1, kH2, true, s);
    gemm_fwd(m->h2b, W[2], b[2], emb_blocks_dev, nullptr, B, kH2, kEmb, false, s);
  }
  if (BC > 0) {
    cand_features_kernel<<<blocks_for((size_t)BC * kCandIn), 256, 0, s>>>(words_dev, word_stride, BC, m->xc);
    gemm_fwd(m->xc, W[3], b[3], m->g1, m->g1b, BC, kCandIn, kCandH, true, s);
    gemm_fwd(m->g1b, W[4], b[4], emb_words_dev, nullptr, BC, kCandH, kEmb, false, s);
  }
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

}  // extern "C"

namespace mptc_internal {

mptc_status embed_workspace_alloc(EmbedWorkspace &ws, int rows) {
  using namespace mptc;
  embed_workspace_free(ws);
  const size_t r = (size_t)rows;
  if (dmalloc(&ws.x, r * kFeatPad) || dmalloc(&ws.h1b, r * kH1) || dmalloc(&ws.h2b, r * kH2) ||
      dmalloc(&ws.h1, r * kH1) || dmalloc(&ws.h2, r * kH2) || dmalloc(&ws.wt, kOff.total)) {
    embed_workspace_free(ws);
    return MPTC_ENOMEM;
  }
  ws.cap = rows;
  return MPTC_OK;
}

void embed_workspace_free(EmbedWorkspace &ws) {
  cudaFree(ws.x);
  cudaFree(ws.h1b);
  cudaFree(ws.h2b);
  cudaFree(ws.h1);
  cudaFree(ws.h2);
  cudaFree(ws.wt);
  ws = EmbedWorkspace{};
}

mptc_status model_embed_frame(const mptc_model *m, EmbedWorkspace &ws, const uint8_t *rgb, int width,
                              const uint64_t *stb, int n, float *F, const uint32_t *words, int word_stride,
                              float *G, cudaStream_t s) {
  using namespace mptc;
  if (!m || n > ws.cap) return MPTC_EINVAL;
  // transposed bf16 weights ([out x in]) so both GEMM operands load as
  // contiguous 16-byte vectors along k
  const bf16 *Wt[5];
  const float *b[5];
  for (int l = 0; l < 5; ++l) {
    const size_t cnt = (size_t)kLayers[l].in * kLayers[l].out;
    transpose_bf16_kernel<<<blocks_for(cnt), 256, 0, s>>>(m->w + kOff.w[l], kLayers[l].in, kLayers[l].out,
                                                          ws.wt + kOff.w[l]);
    Wt[l] = ws.wt + kOff.w[l];
    b[l] = m->w + kOff.b[l];
  }
  auto fwd = [&](const bf16 *x, int l, float *y, bf16 *yb, bool relu) {
    const int K = kLayers[l].in, N = kLayers[l].out;
    dim3 grid((N + kGBN - 1) / kGBN, (n + kGBM - 1) / kGBM);
    gemm_bf16_kernel<false, true><<<grid, 128, 0, s>>>(x, K, Wt[l], K, y, yb, N, b[l], n, N, K, relu ? 1 : 0, 0);
  };
  block_features_kernel<<<blocks_for((size_t)n * kFeatPad), 256, 0, s>>>(rgb, width, width / 4, stb, nullptr, n, ws.x);
  fwd(ws.x, 0, ws.h1, ws.h1b, true);
  fwd(ws.h1b, 1, ws.h2, ws.h2b, true);
  fwd(ws.h2b, 2, F, nullptr, false);
  // candidate MLP: reuse x (n x 32 fits in n x 64) and h1 (n x 128 fits in n x 256)
  cand_features_kernel<<<blocks_for((size_t)n * kCandIn), 256, 0, s>>>(words, word_stride, n, ws.x);
  fwd(ws.x, 3, ws.h1, ws.h1b, true);
  fwd(ws.h1b, 4, G, nullptr, false);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

}  // namespace mptc_internal
