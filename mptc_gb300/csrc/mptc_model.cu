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
  float *f = nullptr, *gg = nullptr;
  bf16 *dfb = nullptr, *dggb = nullptr, *dh1b = nullptr, *dh2b = nullptr, *dg1b = nullptr;
  float *part = nullptr;  // partial sums of the split gradient reductions (part_floats)
  size_t part_floats = 0;
  float *loss = nullptr;
  // packed bf16 weight image of the inference kernels (refreshed after every
  // parameter change) and a bf16 staging buffer for mptc_model_embed
  uint8_t *img = nullptr;
  __nv_bfloat16 *emb_tmp = nullptr;
  int emb_cap = 0;
  // status words: 0 - 3 of mptc_model_embed; 4 the training kernels' timeout
  // flag (sticky until a step reads it back)
  uint32_t *status = nullptr;
};

namespace {

void free_ws(mptc_model *m) {
  void *ps[] = {m->x, m->h1b, m->h2b, m->xc, m->g1b, m->f, m->gg, m->dfb, m->dggb, m->dh1b, m->dh2b, m->dg1b, m->part};
  for (void *p : ps) cudaFree(p);
  m->x = m->h1b = m->h2b = m->xc = m->g1b = nullptr;
  m->f = m->gg = nullptr;
  m->dfb = m->dggb = m->dh1b = m->dh2b = m->dg1b = nullptr;
  m->part = nullptr;
  m->cap_b = m->cap_bc = 0;
  m->part_floats = 0;
}

// Partial sums of the split dW reductions below (slices x outputs floats).
constexpr size_t kSplitFloats = 1 << 22;
// Column partial sums of the bias gradients: softmax_ce (2 x 64 per 8
// blocks) and the dx epilogues (one row of K_layer per 128 examples).
size_t part_floats_for(int B, int BC) {
  using namespace mptc;
  const size_t ce = 2 * (size_t)((B + 7) / 8) * kEmb;
  const size_t dxb = (size_t)((B + kTcBM - 1) / kTcBM) * kH2;
  const size_t dxc = (size_t)((BC + kTcBM - 1) / kTcBM) * kCandH;
  return std::max(std::max(kSplitFloats, ce), std::max(dxb, dxc));
}

mptc_status ensure_ws(mptc_model *m, int B, int BC) {
  if (B <= m->cap_b && BC <= m->cap_bc) return MPTC_OK;
  free_ws(m);
  using namespace mptc;
  const size_t pf = part_floats_for(B, BC);
  bool bad = dmalloc(&m->x, (size_t)B * kFeatPad) || dmalloc(&m->h1b, (size_t)B * kH1) ||
             dmalloc(&m->h2b, (size_t)B * kH2) || dmalloc(&m->xc, (size_t)BC * kCandIn) ||
             dmalloc(&m->g1b, (size_t)BC * kCandH) || dmalloc(&m->f, (size_t)B * kEmb) ||
             dmalloc(&m->gg, (size_t)BC * kEmb) || dmalloc(&m->dfb, (size_t)B * kEmb) ||
             dmalloc(&m->dggb, (size_t)BC * kEmb) || dmalloc(&m->dh1b, (size_t)B * kH1) ||
             dmalloc(&m->dh2b, (size_t)B * kH2) || dmalloc(&m->dg1b, (size_t)BC * kCandH) || dmalloc(&m->part, pf);
  if (bad) {
    free_ws(m);
    return MPTC_ENOMEM;
  }
  m->cap_b = B;
  m->cap_bc = BC;
  m->part_floats = pf;
  return MPTC_OK;
}

int blocks_for(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 4096); }

// The split training products run as up to 3 CTAs per SM of a 152-SM part
// (the most two pipeline stages of shared memory allow), fixed so that the
// split and with it the summation order do not depend on the device.
constexpr int kTrainCtas = 456;

cudaError_t ensure_gemm_attrs() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    err = cudaFuncSetAttribute(mptc::gemm_tc_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               mptc::kTcSmem);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(mptc::gemm_tc_kernel<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 mptc::kTcSmem);
    if (err == cudaSuccess)
      err = cudaFuncSetAttribute(mptc::gemm_tc_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 mptc::kTcSmem);
  });
  return err;
}

// y[M x N] = x[M x K] W + b (opt. ReLU) into y (fp32) and/or yb (bf16).
void gemm_fwd(const bf16 *x, const bf16 *W, const float *b, float *y, bf16 *yb, int M, int K, int N, bool relu,
              uint32_t *status, cudaStream_t s) {
  dim3 grid((N + mptc::kTcBN - 1) / mptc::kTcBN, (M + mptc::kTcBM - 1) / mptc::kTcBM);
  const mptc::GemmEpi e{y, yb, N, b, relu ? 1 : 0, nullptr, nullptr};
  mptc::gemm_tc_kernel<false, false><<<grid, 128, mptc::kTcSmem, s>>>(x, K, W, N, e, M, N, K, status);
}

// out[n] = sum of the `slices` rows of part [slices x n], in order.
void slice_sum(const float *part, int slices, int n, float *out, cudaStream_t s) {
  mptc::slice_sum_kernel<<<(n + 31) / 32, 256, 0, s>>>(part, slices, n, out);
}

// dW[K x N] = x^T[K x M] dy[M x N]: few outputs and a long reduction over the
// M examples, so the reduction is split into slices of at least 256 rows
// (up to kTrainCtas CTAs in all) whose partial products are summed in slice
// order afterwards (deterministic).
void gemm_dw(const bf16 *x, const bf16 *dy, float *dW, int M, int K, int N, float *part, uint32_t *status,
             cudaStream_t s) {
  const int tiles = ((N + mptc::kTcBN - 1) / mptc::kTcBN) * ((K + mptc::kTcBM - 1) / mptc::kTcBM);
  int splits = std::min(M / 256, std::max(1, kTrainCtas / tiles));
  splits = (int)std::max<size_t>(1, std::min<size_t>((size_t)splits, kSplitFloats / ((size_t)K * N)));
  dim3 grid((N + mptc::kTcBN - 1) / mptc::kTcBN, (K + mptc::kTcBM - 1) / mptc::kTcBM, splits);
  const mptc::GemmEpi e{splits > 1 ? part : dW, nullptr, N, nullptr, 0, nullptr, nullptr};
  mptc::gemm_tc_kernel<true, false><<<grid, 128, mptc::kTcSmem, s>>>(x, K, dy, N, e, K, N, M, status);
  if (splits > 1) slice_sum(part, splits, K * N, dW, s);
}

// dx[M x K] = (dy[M x N] W^T) masked by the ReLU of the layer's input (h > 0)
// into dxb (bf16), and db[K] = the column sums of that dx (the bias gradient
// of the layer below).
void gemm_dx(const bf16 *dy, const bf16 *W, const bf16 *h, bf16 *dxb, float *db, int M, int K, int N, float *part,
             uint32_t *status, cudaStream_t s) {
  dim3 grid((K + mptc::kTcBN - 1) / mptc::kTcBN, (M + mptc::kTcBM - 1) / mptc::kTcBM);
  const mptc::GemmEpi e{nullptr, dxb, K, nullptr, 0, h, part};
  mptc::gemm_tc_kernel<false, true><<<grid, 128, mptc::kTcSmem, s>>>(dy, N, W, N, e, M, K, N, status);
  slice_sum(part, (int)grid.y, K, db, s);
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
  if (ensure_gemm_attrs() != cudaSuccess) return MPTC_ECUDA;
  uint32_t *status = m->status + 4;
  block_features_kernel<<<blocks_for((size_t)B * kFeatPad), 256, 0, s>>>(rgb, width, bw, stb, blocks, B, m->x);
  gemm_fwd(m->x, W[0], b[0], nullptr, m->h1b, B, kFeatPad, kH1, true, status, s);
  gemm_fwd(m->h1b, W[1], b[1], nullptr, m->h2b, B, kH1, kH2, true, status, s);
  gemm_fwd(m->h2b, W[2], b[2], m->f, nullptr, B, kH2, kEmb, false, status, s);
  cand_features_kernel<<<blocks_for((size_t)BC * kCandIn), 256, 0, s>>>(cands, 1, BC, m->xc);
  gemm_fwd(m->xc, W[3], b[3], nullptr, m->g1b, BC, kCandIn, kCandH, true, status, s);
  gemm_fwd(m->g1b, W[4], b[4], m->gg, nullptr, BC, kCandH, kEmb, false, status, s);
  cudaMemsetAsync(m->loss, 0, sizeof(float), s);
  const int nce = (B + 7) / 8;
  float *partF = m->part, *partG = m->part + (size_t)nce * kEmb;
  softmax_ce_kernel<<<nce, 256, 0, s>>>(m->f, m->gg, B, C, m->dfb, m->dggb, partF, partG, m->loss);
  if (!grads) return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
  float *G[5], *Gb[5];
  for (int l = 0; l < 5; ++l) {
    G[l] = m->g + kOff.w[l];
    Gb[l] = m->g + kOff.b[l];
  }
  // output biases from the loss kernel's column sums
  slice_sum(partF, nce, kEmb, Gb[2], s);
  slice_sum(partG, nce, kEmb, Gb[4], s);
  // block MLP
  gemm_dw(m->h2b, m->dfb, G[2], B, kH2, kEmb, m->part, status, s);
  gemm_dx(m->dfb, W[2], m->h2b, m->dh2b, Gb[1], B, kH2, kEmb, m->part, status, s);
  gemm_dw(m->h1b, m->dh2b, G[1], B, kH1, kH2, m->part, status, s);
  gemm_dx(m->dh2b, W[1], m->h1b, m->dh1b, Gb[0], B, kH1, kH2, m->part, status, s);
  gemm_dw(m->x, m->dh1b, G[0], B, kFeatPad, kH1, m->part, status, s);
  // candidate MLP
  gemm_dw(m->g1b, m->dggb, G[4], BC, kCandH, kEmb, m->part, status, s);
  gemm_dx(m->dggb, W[4], m->g1b, m->dg1b, Gb[3], BC, kCandH, kEmb, m->part, status, s);
  gemm_dw(m->xc, m->dg1b, G[3], BC, kCandIn, kCandH, m->part, status, s);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

// Reads back (and clears) the training kernels' timeout flag after the work
// queued on s, together with the loss when loss_host is given.
mptc_status finish_training(mptc_model *m, float *loss_host, cudaStream_t s) {
  uint32_t flag = 0;
  if ((loss_host && cudaMemcpyAsync(loss_host, m->loss, sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess) ||
      cudaMemcpyAsync(&flag, m->status + 4, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return MPTC_ECUDA;
  if (flag) {
    cudaMemsetAsync(m->status + 4, 0, 4, s);
    return MPTC_ETIMEOUT;
  }
  return MPTC_OK;
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
// kernel's weights and operand buffers (98 KB with 128-wide hidden layers)
// let at most two CTAs share an SM, which is what their TMEM columns
// (kH1 + kH2 = 256 each) allow; the g kernel asks for 80 KB so that at most
// two CTAs (256 TMEM columns each) share an SM.
constexpr int kMaxDev = 64;
std::mutex g_attr_mu;
bool g_attr_done[kMaxDev] = {};
constexpr size_t kSmemF = mptc::embed_smem_bytes<mptc::NetF>();
constexpr int kCtasF = 512 / mptc::NetF::kTmem;  // f CTAs per SM
static_assert(kCtasF == 1 || kSmemF * 3 > 228 * 1024, "shared memory keeps f's CTAs within the TMEM columns");
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
    a.n_dev = J.n_dev;
    a.out_rows = J.out_rows;
    tiles += (J.n + 127) / 128;  // an upper bound when n_dev is set
  }
  if (tiles == 0) return MPTC_OK;
  const int sms = sm_count_now();
  if (blocks)
    mptc::embed_kernel<mptc::NetF, true><<<std::min(tiles, kCtasF * sms), mptc::kEmbedThreads, kSmemF, s>>>(b);
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
      dmalloc(&m->loss, 1) || dmalloc(&m->img, mptc::kImgBytes) || dmalloc(&m->status, 8) ||
      cudaMemset(m->img, 0, mptc::kImgBytes) != cudaSuccess || cudaMemset(m->status, 0, 32) != cudaSuccess) {
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
  st = finish_training(m, loss_host, s);
  if (st != MPTC_OK) return st;
  if (grads_host && cudaMemcpy(grads_host, m->g, kOff.total * sizeof(float), cudaMemcpyDeviceToHost) != cudaSuccess)
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
  // without loss_host the step stays asynchronous; a timeout flag it raised
  // is reported by the next step that reads back
  return loss_host ? finish_training(m, loss_host, s) : MPTC_OK;
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
