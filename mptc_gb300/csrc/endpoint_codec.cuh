// Endpoint images and stream decode on the GPU.
//
// Encoder side: the two endpoint images of a frame (ep1, ep2 of every final
// block, RGB565) go to YCoCg-667 (codec/image_processing.cpp:10-27), then each
// 64x64 tile of each plane gets the 6-level integer 5/3 lifting wavelet
// (codec/image_processing.h:292-330, codec/wavelet.cpp:30-127): per level
// dim = 64, 32, ..., 2 a column pass then a row pass over the top-left
// dim x dim corner. Coefficients are wrapped to int8 and offset by 128
// (codec/image_utils.h:218-237, pixel_traits.h:261-273).
//
// Decoder side: the inverse (codec/decoder.cpp:68-107, wavelet.cpp:69-155;
// dim = 2, ..., 64, rows then columns), YCoCg-667 -> RGB565 in int8
// arithmetic (decoder.cpp:24-41, 109-201), and the index words from the motion
// codes (decoder.cpp:203-254): unique blocks take the next palette entry in
// raster order, inter blocks copy from the previous frame, intra blocks copy
// from an earlier block of the same frame. The intra copies form chains; they
// are resolved by pointer jumping (log2(blocks) rounds) instead of the
// reference's raster loop.
//
// Forward: one CTA per (64x64 tile, plane), two int16 tiles in shared memory
// (source and destination of each lifting pass). Inverse: one CTA per
// (tile, endpoint) with its three planes (2 x 24 KiB), which the RGB565
// conversion needs together.
#pragma once

#include <cstdint>

namespace mptc {

constexpr int kTile = 64;                 // endpoint tile edge (blocks)
constexpr int kTileElems = kTile * kTile;
constexpr int kCodecThreads = 256;

// Mirror index into [0, len) for the indices the lifting uses (-1 and len).
__device__ __forceinline__ int lift_mirror(int i, int len) { return i < 0 ? -i : (i >= len ? 2 * len - 2 - i : i); }

// One forward lifting pass over `lines` lines of length `len` (power of two)
// of `planes` planes: element k of line l of plane p is at
// p*kTileElems + l*lstride + k*estride. src -> dst, details in the upper half
// (codec/wavelet.cpp:30-66).
__device__ __forceinline__ void forward_pass(const int16_t *src, int16_t *dst, int planes, int len, int lstride,
                                             int estride) {
  const int half = len >> 1;  // len is even: mid point == half
  const int work = planes * len * half;
  for (int w = threadIdx.x; w < work; w += blockDim.x) {
    const int p = w / (len * half), r = w - p * len * half;
    const int l = r / half, k = r - l * half;
    const int16_t *s = src + p * kTileElems + l * lstride;
    const int i = 2 * k + 1;
    dst[p * kTileElems + l * lstride + (half + k) * estride] =
        (int16_t)(s[i * estride] - (s[(i - 1) * estride] + s[lift_mirror(i + 1, len) * estride]) / 2);
  }
  __syncthreads();
  for (int w = threadIdx.x; w < work; w += blockDim.x) {
    const int p = w / (len * half), r = w - p * len * half;
    const int l = r / half, k = r - l * half;
    const int16_t *s = src + p * kTileElems + l * lstride;
    int16_t *d = dst + p * kTileElems + l * lstride;
    const int i = 2 * k;
    const int prev = half + lift_mirror(i - 1, len) / 2, next = half + (i + 1) / 2;
    d[k * estride] = (int16_t)(s[i * estride] + (d[prev * estride] + d[next * estride] + 2) / 4);
  }
  __syncthreads();
}

// Inverse of forward_pass (codec/wavelet.cpp:69-99).
__device__ __forceinline__ void inverse_pass(const int16_t *src, int16_t *dst, int len, int lstride, int estride) {
  const int half = len >> 1;
  const int work = 3 * len * half;
  for (int w = threadIdx.x; w < work; w += blockDim.x) {
    const int p = w / (len * half), r = w - p * len * half;
    const int l = r / half, k = r - l * half;
    const int16_t *s = src + p * kTileElems + l * lstride;
    const int i = 2 * k;
    const int prev = half + lift_mirror(i - 1, len) / 2, next = half + (i + 1) / 2;
    dst[p * kTileElems + l * lstride + i * estride] =
        (int16_t)(s[k * estride] - (s[prev * estride] + s[next * estride] + 2) / 4);
  }
  __syncthreads();
  for (int w = threadIdx.x; w < work; w += blockDim.x) {
    const int p = w / (len * half), r = w - p * len * half;
    const int l = r / half, k = r - l * half;
    const int16_t *s = src + p * kTileElems + l * lstride;
    int16_t *d = dst + p * kTileElems + l * lstride;
    const int i = 2 * k + 1;
    d[i * estride] = (int16_t)(s[(half + k) * estride] + (d[(i - 1) * estride] + d[lift_mirror(i + 1, len) * estride]) / 2);
  }
  __syncthreads();
}

// grid (bw/64, bh/64, 6 planes: Y, Co, Cg of endpoint 1, then of endpoint 2),
// one plane of one tile per CTA. coeff: 6 planes of bw*bh bytes,
// [Y1 | Co1 | Cg1 | Y2 | Co2 | Cg2], each plane raster order over the image.
__global__ void __launch_bounds__(kCodecThreads) endpoint_forward_kernel(const uint64_t *__restrict__ blocks, int bw,
                                                                         int bh, uint8_t *__restrict__ coeff) {
  __shared__ int16_t a[kTileElems], b[kTileElems];
  const int tx = blockIdx.x * kTile, ty = blockIdx.y * kTile, plane = blockIdx.z;
  const int ep = plane / 3, channel = plane - 3 * ep;
  const size_t n = (size_t)bw * bh;
  for (int e = threadIdx.x; e < kTileElems; e += blockDim.x) {
    const int y = e >> 6, x = e & 63;
    const uint32_t lo = (uint32_t)blocks[(size_t)(ty + y) * bw + tx + x];
    const int c = (int)(ep ? (lo >> 16) : (lo & 0xFFFFu));
    const int r5 = c >> 11, g6 = (c >> 5) & 63, b5 = c & 31;
    const int co = r5 - b5, t = r5 + b5 + (b5 >> 4), cg = g6 - t;
    a[e] = (int16_t)(channel == 0 ? t + cg / 2 : (channel == 1 ? co : cg));
  }
  __syncthreads();
  for (int dim = kTile; dim > 1; dim >>= 1) {
    forward_pass(a, b, 1, dim, 1, kTile);   // columns: line = column, element stride = row
    forward_pass(b, a, 1, dim, kTile, 1);   // rows
  }
  uint8_t *out = coeff + (size_t)plane * n;
  for (int e = threadIdx.x; e < kTileElems; e += blockDim.x) {
    const int y = e >> 6, x = e & 63;
    out[(size_t)(ty + y) * bw + tx + x] = (uint8_t)((int)(int8_t)a[e] + 128);
  }
}

// grid (bw/64, bh/64, 2 endpoints): coefficients -> RGB565 endpoint words.
__global__ void __launch_bounds__(kCodecThreads) endpoint_inverse_kernel(const uint8_t *__restrict__ coeff, int bw,
                                                                         int bh, uint16_t *__restrict__ ep_out) {
  __shared__ int16_t a[3 * kTileElems], b[3 * kTileElems];
  const int tx = blockIdx.x * kTile, ty = blockIdx.y * kTile, ep = blockIdx.z;
  const size_t n = (size_t)bw * bh;
  for (int e = threadIdx.x; e < 3 * kTileElems; e += blockDim.x) {
    const int p = e >> 12, q = e & (kTileElems - 1), y = q >> 6, x = q & 63;
    a[e] = (int16_t)((int)coeff[(size_t)(3 * ep + p) * n + (size_t)(ty + y) * bw + tx + x] - 128);
  }
  __syncthreads();
  for (int dim = 2; dim <= kTile; dim <<= 1) {
    inverse_pass(a, b, dim, kTile, 1);      // rows
    inverse_pass(b, a, dim, 1, kTile);      // columns
  }
  for (int e = threadIdx.x; e < kTileElems; e += blockDim.x) {
    const int y = e >> 6, x = e & 63;
    // int8 arithmetic as the reference stores it (decoder.cpp:24-41, 145-160)
    const int8_t Y = (int8_t)a[e], Co = (int8_t)a[kTileElems + e], Cg = (int8_t)a[2 * kTileElems + e];
    const int8_t t = (int8_t)(Y - Cg / 2);
    const int8_t g = (int8_t)(Cg + t);
    const int8_t bb = (int8_t)((t - Co) / 2);
    const int8_t r = (int8_t)(bb + Co);
    uint16_t w = (uint16_t)(int16_t)r;
    w = (uint16_t)(w << 6);
    w |= (uint16_t)(int16_t)g;
    w = (uint16_t)(w << 5);
    w |= (uint16_t)(int16_t)bb;
    ep_out[(size_t)ep * n + (size_t)(ty + y) * bw + tx + x] = w;
  }
}

// --- index words from motion codes ---

constexpr int kDecTile = 1024;  // blocks per CTA of the unique-rank scan
constexpr uint32_t kDecBadRef = 1u, kDecBadUnique = 2u;

// Classifies blocks: ptr = source block of an intra copy (-1 when resolved),
// val = index word when resolved (inter copy). Counts unique blocks per tile.
__global__ void __launch_bounds__(256) decode_classify_kernel(const uint8_t *__restrict__ motion,
                                                              const uint64_t *__restrict__ prev, int bw, int nblk,
                                                              int sa, int32_t *__restrict__ ptr,
                                                              uint32_t *__restrict__ val,
                                                              uint32_t *__restrict__ tile_counts,
                                                              uint32_t *__restrict__ err) {
  const int t0 = blockIdx.x * kDecTile;
  int c = 0;
  for (int i = t0 + threadIdx.x; i < min(nblk, t0 + kDecTile); i += blockDim.x) {
    const int x = motion[2 * i], y = motion[2 * i + 1];
    const int bx = i % bw, by = i / bw;
    if (x == 255 && y == 255) {
      ++c;
      ptr[i] = -1;
      val[i] = 0;
    } else if ((x & 0x80) && (y & 0x80)) {
      // linear index as the reference computes it (decoder.cpp:224-236)
      const long ref = (long)(by + (y & 0x7F) - sa) * bw + bx + (x & 0x7F) - sa;
      uint32_t v = 0;
      if (prev && ref >= 0 && ref < nblk) v = (uint32_t)(prev[ref] >> 32);
      else atomicOr(err, kDecBadRef);
      ptr[i] = -1;
      val[i] = v;
    } else {
      const long ref = (long)(by + y - 2 * sa + 1) * bw + bx + x - sa;
      if (ref >= 0 && ref < i) {
        ptr[i] = (int32_t)ref;
      } else {
        atomicOr(err, kDecBadRef);
        ptr[i] = -1;
      }
      val[i] = 0;
    }
  }
  c = __reduce_add_sync(0xFFFFFFFFu, c);
  __shared__ int s[8];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < 8; ++w) t += s[w];
    tile_counts[blockIdx.x] = (uint32_t)t;
  }
}

// Unique blocks take palette[rank], rank = unique blocks before them in raster order.
__global__ void __launch_bounds__(256) decode_unique_kernel(const uint8_t *__restrict__ motion, int nblk,
                                                            const uint32_t *__restrict__ tile_counts,
                                                            const uint32_t *__restrict__ palette, uint32_t n_unique,
                                                            uint32_t *__restrict__ val, uint32_t *__restrict__ err) {
  __shared__ uint32_t s_base, s_warp[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) {
    uint32_t b = 0, total = 0;
    for (int t = 0; t < (int)gridDim.x; ++t) {
      if (t < (int)blockIdx.x) b += tile_counts[t];
      total += tile_counts[t];
    }
    s_base = b;
    if (blockIdx.x == 0 && total != n_unique) atomicOr(err, kDecBadUnique);
  }
  __syncthreads();
  const int t0 = blockIdx.x * kDecTile, t1 = min(nblk, t0 + kDecTile);
  for (int c0 = t0; c0 < t1; c0 += 256) {
    const int i = c0 + threadIdx.x;
    const bool u = i < t1 && motion[2 * i] == 255 && motion[2 * i + 1] == 255;
    const unsigned bal = __ballot_sync(0xFFFFFFFFu, u);
    if (lane == 0) s_warp[warp] = __popc(bal);
    __syncthreads();
    uint32_t off = s_base;
    for (int w = 0; w < warp; ++w) off += s_warp[w];
    off += __popc(bal & ((1u << lane) - 1u));
    if (u) val[i] = off < n_unique ? palette[off] : 0u;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (int w = 0; w < 8; ++w) t += s_warp[w];
      s_base += t;
    }
    __syncthreads();
  }
}

// One pointer-jumping round: (ptr_in, val_in) -> (ptr_out, val_out).
__global__ void __launch_bounds__(256) decode_jump_kernel(const int32_t *__restrict__ ptr_in,
                                                          const uint32_t *__restrict__ val_in, int nblk,
                                                          int32_t *__restrict__ ptr_out,
                                                          uint32_t *__restrict__ val_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nblk) return;
  const int32_t p = ptr_in[i];
  if (p < 0) {
    ptr_out[i] = -1;
    val_out[i] = val_in[i];
    return;
  }
  const int32_t q = ptr_in[p];
  if (q < 0) {
    ptr_out[i] = -1;
    val_out[i] = val_in[p];
  } else {
    ptr_out[i] = q;
    val_out[i] = 0;
  }
}

__global__ void __launch_bounds__(256) decode_assemble_kernel(const uint16_t *__restrict__ ep, const uint32_t *__restrict__ val,
                                                              int nblk, uint64_t *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nblk) return;
  out[i] = (uint64_t)ep[i] | ((uint64_t)ep[nblk + i] << 16) | ((uint64_t)val[i] << 32);
}

}  // namespace mptc
