// C ABI of the endpoint transform and of the GPU decoder (include/mptc_gb300.h).
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "../../include/mptc_gb300.h"
#include "endpoint_codec.cuh"

namespace {

bool tiled_size(int32_t width, int32_t height) {
  return width > 0 && height > 0 && width % 256 == 0 && height % 256 == 0 &&
         (int64_t)(width / 4) * (height / 4) <= (int64_t)1 << 30;
}

}  // namespace

struct mptc_decoder {
  int width = 0, height = 0, bw = 0, bh = 0, nblk = 0, sa = 0, ntiles = 0, rounds = 0;
  int32_t *ptr[2] = {nullptr, nullptr};
  uint32_t *val[2] = {nullptr, nullptr};
  uint32_t *tile_counts = nullptr;
  uint16_t *ep = nullptr;    // [2][nblk] decoded endpoint words
  uint32_t *flags = nullptr; // device error flags
  std::string err;
};

namespace {

mptc_status dfail(mptc_decoder *d, mptc_status st, const std::string &msg) {
  if (d) d->err = msg;
  return st;
}

void release(mptc_decoder *d) {
  cudaFree(d->ptr[0]);
  cudaFree(d->ptr[1]);
  cudaFree(d->val[0]);
  cudaFree(d->val[1]);
  cudaFree(d->tile_counts);
  cudaFree(d->ep);
  cudaFree(d->flags);
}

}  // namespace

extern "C" {

mptc_status mptc_endpoint_coefficients(int32_t width, int32_t height, const uint64_t *blocks_dev,
                                       uint8_t *coeff_dev, void *stream) {
  if (!tiled_size(width, height) || !blocks_dev || !coeff_dev) return MPTC_EINVAL;
  const int bw = width / 4, bh = height / 4;
  const dim3 grid(bw / mptc::kTile, bh / mptc::kTile, 6);
  mptc::endpoint_forward_kernel<<<grid, mptc::kCodecThreads, 0, (cudaStream_t)stream>>>(blocks_dev, bw, bh,
                                                                                        coeff_dev);
  return cudaGetLastError() == cudaSuccess ? MPTC_OK : MPTC_ECUDA;
}

mptc_status mptc_decoder_create(int32_t width, int32_t height, int32_t search_area, mptc_decoder **out) {
  if (!out || !tiled_size(width, height) || search_area < 1 || search_area > 63) return MPTC_EINVAL;
  mptc_decoder *d = new (std::nothrow) mptc_decoder();
  if (!d) return MPTC_ENOMEM;
  d->width = width;
  d->height = height;
  d->bw = width / 4;
  d->bh = height / 4;
  d->nblk = d->bw * d->bh;
  d->sa = search_area;
  d->ntiles = (d->nblk + mptc::kDecTile - 1) / mptc::kDecTile;
  int r = 1;
  while ((1ll << (r - 1)) < d->nblk) ++r;  // chains are shorter than nblk <= 2^(r-1)
  d->rounds = r;
  const size_t n = (size_t)d->nblk;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaMalloc(&d->ptr[k], n * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d->val[k], n * sizeof(uint32_t));
  }
  if (e == cudaSuccess) e = cudaMalloc(&d->tile_counts, (size_t)d->ntiles * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&d->ep, 2 * n * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&d->flags, sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMemset(d->flags, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    release(d);
    delete d;
    return e == cudaErrorMemoryAllocation ? MPTC_ENOMEM : MPTC_ECUDA;
  }
  *out = d;
  return MPTC_OK;
}

mptc_status mptc_decoder_destroy(mptc_decoder *d) {
  if (!d) return MPTC_EINVAL;
  release(d);
  delete d;
  return MPTC_OK;
}

mptc_status mptc_decode_frame(mptc_decoder *d, const uint8_t *coeff_dev, const uint8_t *motion_dev,
                              const uint32_t *unique_dev, uint32_t n_unique, const uint64_t *prev_dev,
                              uint64_t *out_dev, void *stream) {
  if (!d) return MPTC_EINVAL;
  if (!coeff_dev || !motion_dev || !out_dev || (n_unique && !unique_dev))
    return dfail(d, MPTC_EINVAL, "decode_frame: NULL buffer");
  if (n_unique > (uint32_t)d->nblk) return dfail(d, MPTC_EINVAL, "decode_frame: more unique entries than blocks");
  cudaStream_t s = (cudaStream_t)stream;
  const dim3 tiles(d->bw / mptc::kTile, d->bh / mptc::kTile, 2);
  mptc::endpoint_inverse_kernel<<<tiles, mptc::kCodecThreads, 0, s>>>(coeff_dev, d->bw, d->bh, d->ep);
  mptc::decode_classify_kernel<<<d->ntiles, 256, 0, s>>>(motion_dev, prev_dev, d->bw, d->nblk, d->sa, d->ptr[0],
                                                         d->val[0], d->tile_counts, d->flags);
  mptc::decode_unique_kernel<<<d->ntiles, 256, 0, s>>>(motion_dev, d->nblk, d->tile_counts, unique_dev, n_unique,
                                                       d->val[0], d->flags);
  const int g = (d->nblk + 255) / 256;
  int cur = 0;
  for (int r = 0; r < d->rounds; ++r, cur ^= 1)
    mptc::decode_jump_kernel<<<g, 256, 0, s>>>(d->ptr[cur], d->val[cur], d->nblk, d->ptr[cur ^ 1], d->val[cur ^ 1]);
  mptc::decode_assemble_kernel<<<g, 256, 0, s>>>(d->ep, d->val[cur], d->nblk, out_dev);
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? MPTC_OK : dfail(d, MPTC_ECUDA, cudaGetErrorString(e));
}

mptc_status mptc_decoder_check(mptc_decoder *d, void *stream, uint32_t *flags) {
  if (!d) return MPTC_EINVAL;
  uint32_t h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, d->flags, sizeof(h), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d->flags, 0, sizeof(uint32_t), (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return dfail(d, MPTC_ECUDA, cudaGetErrorString(e));
  if (flags) *flags = h;
  if (h) {
    std::string m = "decoded frames held";
    if (h & mptc::kDecBadRef) m += " motion codes that copy from outside the frame or from undecoded blocks";
    if (h & mptc::kDecBadUnique) m += (h & mptc::kDecBadRef) ? " and" : "", m += " a unique count that differs from the palette";
    return dfail(d, MPTC_EINVAL, m);
  }
  return MPTC_OK;
}

const char *mptc_decoder_last_error(const mptc_decoder *d) { return d ? d->err.c_str() : "null decoder"; }

}  // extern "C"
