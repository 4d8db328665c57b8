// Host-side MPTC stream writer (include/mptc_host.h): the container and the
// endpoint transform of the reference encoder, restated so that a stream
// built from this library's per-frame arrays is byte-identical to the
// reference encoder's stream. The arithmetic coder is in arith_coder.h.
#include "../../include/mptc_host.h"
#include "arith_coder.h"
#include "parallel.h"

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

namespace {

using mptc_host::code_bytes;
using mptc_host::host_threads;
using mptc_host::parallel_for;

constexpr size_t kParallelBlocks = 16384;  // frames this large code their parts concurrently

// --- endpoint transform (codec/image_processing.cpp:10-27, codec/wavelet.cpp:11-131) ---

// Mirror index into [0, range): ... C B A B C D E D C ...
int mirror(int idx, int range) {
  if (idx < 0) return -idx;
  if (idx >= range) return 2 * range - 2 - idx;
  return idx;
}

// One level of the integer 5/3 lifting along a line: details (odd samples
// minus the mean of their neighbours) in the upper half, approximations (even
// samples plus a quarter of the neighbouring details, rounded) in the lower
// half. Divisions truncate toward zero as C's do.
void lift_line(const int16_t *src, int16_t *dst, int len) {
  if (len <= 0) return;
  if (len == 1) {
    dst[0] = src[0];
    return;
  }
  std::fill(dst, dst + len, (int16_t)0);
  const int mid = len - len / 2;
  for (int i = 1; i < len; i += 2)
    dst[mid + i / 2] = (int16_t)(src[i] - (src[mirror(i - 1, len)] + src[mirror(i + 1, len)]) / 2);
  for (int i = 0; i < len; i += 2) {
    const int prev = mid + mirror(i - 1, len) / 2, next = mid + mirror(i + 1, len) / 2;
    dst[i / 2] = (int16_t)(src[i] + (dst[prev] + dst[next] + 2) / 4);
  }
}

// All levels on one 64x64 tile (row stride 64): columns, then rows, on the
// top-left dim x dim corner for dim = 64, 32, ..., 2.
void tile_wavelet(int16_t *t) {
  std::vector<int16_t> a(64), b(64);
  for (int dim = 64; dim > 1; dim /= 2) {
    for (int c = 0; c < dim; ++c) {
      for (int r = 0; r < dim; ++r) a[r] = t[r * 64 + c];
      lift_line(a.data(), b.data(), dim);
      for (int r = 0; r < dim; ++r) t[r * 64 + c] = b[r];
    }
    for (int r = 0; r < dim; ++r) {
      std::copy(t + r * 64, t + r * 64 + dim, a.begin());
      lift_line(a.data(), b.data(), dim);
      std::copy(b.begin(), b.begin() + dim, t + r * 64);
    }
  }
}

// Coefficient bytes of one plane: per-tile wavelet, 8-bit signed wrap, +128,
// raster order over the whole plane.
std::vector<uint8_t> plane_coefficients(const std::vector<int16_t> &plane, int w, int h) {
  std::vector<int16_t> p(plane);
  std::vector<int16_t> tile(64 * 64);
  for (int ty = 0; ty < h; ty += 64)
    for (int tx = 0; tx < w; tx += 64) {
      for (int y = 0; y < 64; ++y)
        for (int x = 0; x < 64; ++x) tile[y * 64 + x] = p[(size_t)(ty + y) * w + tx + x];
      tile_wavelet(tile.data());
      for (int y = 0; y < 64; ++y)
        for (int x = 0; x < 64; ++x) p[(size_t)(ty + y) * w + tx + x] = tile[y * 64 + x];
    }
  std::vector<uint8_t> out(p.size());
  for (size_t i = 0; i < p.size(); ++i) out[i] = (uint8_t)((int)(int8_t)(uint8_t)p[i] + 128);
  return out;
}

void put_u32(std::vector<uint8_t> &v, uint32_t x) {
  for (int k = 0; k < 4; ++k) v.push_back((uint8_t)(x >> (8 * k)));
}

}  // namespace

struct mptc_stream_writer {
  int width = 0, height = 0, bw = 0, bh = 0, sa = 0, unique_interval = 0, total_frames = 0;
  std::vector<uint8_t> stream;             // header + complete groups
  std::vector<uint8_t> group_records;      // frame records of the open group
  std::vector<uint8_t> group_palette;      // palette bytes of the open group
  uint32_t group_frames = 0;
  uint32_t max_unique = 0, max_palette = 0, max_motion = 0, max_ep_y = 0, max_ep_c = 0;
  uint32_t last_motion = 0, last_ep[4] = {0, 0, 0, 0};
  bool failed = false;  // an allocation failed part way through a frame: the stream is unusable
};

namespace {

// The six coefficient planes [Y1 | Co1 | Cg1 | Y2 | Co2 | Cg2] of a frame's
// endpoint images (CompressEndpoint, codec/codec.cpp:804-838).
std::vector<uint8_t> endpoint_coefficients(const uint64_t *blocks, int bw, int bh) {
  const size_t n = (size_t)bw * bh;
  std::vector<uint8_t> out(6 * n);
  for (int e = 0; e < 2; ++e) {
    std::vector<int16_t> Y(n), Co(n), Cg(n);
    for (size_t i = 0; i < n; ++i) {
      const uint32_t x = (uint32_t)((blocks[i] >> (16 * e)) & 0xFFFF);
      const int r = (int)(x >> 11), g = (int)((x >> 5) & 63), b = (int)(x & 31);
      // RGB565 -> YCoCg-667 (reversible): Co = r - b, t = r + b + b/16,
      // Cg = g - t, Y = t + Cg/2 (C division)
      const int co = r - b, t = r + b + (b >> 4), cg = g - t, y = t + cg / 2;
      Y[i] = (int16_t)y;
      Co[i] = (int16_t)co;
      Cg[i] = (int16_t)cg;
    }
    const std::vector<int16_t> *planes[3] = {&Y, &Co, &Cg};
    for (int p = 0; p < 3; ++p) {
      const std::vector<uint8_t> c = plane_coefficients(*planes[p], bw, bh);
      std::copy(c.begin(), c.end(), out.begin() + (3 * e + p) * n);
    }
  }
  return out;
}

// The five independently coded parts of a frame record: motion codes, Y1,
// Co1|Cg1, Y2, Co2|Cg2 (codec/codec.cpp:1140-1155, :860-899). Each part has
// its own coder and model, so parts and frames code independently.
using FrameCode = std::array<std::vector<uint8_t>, 5>;

std::vector<uint8_t> code_part(const uint8_t *coeff, const uint8_t *motion, size_t n, int k) {
  const uint8_t *src[5] = {motion, coeff, coeff + n, coeff + 3 * n, coeff + 4 * n};
  const size_t len[5] = {2 * n, n, 2 * n, n, 2 * n};
  return code_bytes(src[k], len[k]);
}

// Appends a coded frame's record to the open group and closes the group after
// unique_interval frames (codec/codec.cpp:1115-1158, :1471-1505).
void append_record(mptc_stream_writer *w, const FrameCode &z, const uint32_t *unique, uint32_t n_unique) {
  std::vector<uint8_t> &rec = w->group_records;
  put_u32(rec, n_unique);
  for (int k = 0; k < 5; ++k) {
    put_u32(rec, (uint32_t)z[k].size());
    rec.insert(rec.end(), z[k].begin(), z[k].end());
  }
  w->last_motion = (uint32_t)z[0].size();
  w->max_motion = std::max(w->max_motion, w->last_motion);
  for (int k = 0; k < 4; ++k) w->last_ep[k] = (uint32_t)z[k + 1].size();
  w->max_ep_y = std::max({w->max_ep_y, w->last_ep[0], w->last_ep[2]});
  w->max_ep_c = std::max({w->max_ep_c, w->last_ep[1], w->last_ep[3]});
  // unique palette of the group: u32 entries as bytes
  const uint8_t *pb = reinterpret_cast<const uint8_t *>(unique);
  if (n_unique) w->group_palette.insert(w->group_palette.end(), pb, pb + 4 * (size_t)n_unique);
  if (++w->group_frames == (uint32_t)w->unique_interval) {
    const std::vector<uint8_t> zp = code_bytes(w->group_palette.data(), w->group_palette.size());
    put_u32(w->stream, (uint32_t)zp.size());
    w->max_palette = std::max(w->max_palette, (uint32_t)zp.size());
    w->stream.insert(w->stream.end(), zp.begin(), zp.end());
    const uint32_t count = (uint32_t)w->group_palette.size();  // bytes, as the reference counts them
    put_u32(w->stream, count);
    w->max_unique = std::max(w->max_unique, count);
    w->stream.insert(w->stream.end(), w->group_records.begin(), w->group_records.end());
    w->group_records.clear();
    w->group_palette.clear();
    w->group_frames = 0;
  }
}

// One frame: its five parts concurrently when the frame is large.
void append_frame(mptc_stream_writer *w, const uint8_t *coeff, const uint8_t *motion, const uint32_t *unique,
                  uint32_t n_unique) {
  const size_t n = (size_t)w->bw * w->bh;
  FrameCode z;
  if (!parallel_for(5, n >= kParallelBlocks ? 5 : 1, [&](size_t k) {
        z[k] = code_part(coeff, motion, n, (int)k);
        return true;
      }))
    throw std::bad_alloc();
  append_record(w, z, unique, n_unique);
}

// A run of frames (frame f's arrays at blocks + f n, coeff + 6 f n, motion +
// 2 f n, unique + f n): chunks of frames whose endpoint transforms (when
// `blocks` is given) and parts are coded by all the host's cores, then
// appended in frame order, so the bytes are those of frame-by-frame calls.
void append_frames(mptc_stream_writer *w, size_t n_frames, const uint64_t *blocks, const uint8_t *coeff,
                   const uint8_t *motion, const uint32_t *unique, const uint32_t *n_unique) {
  const size_t n = (size_t)w->bw * w->bh, threads = host_threads(), chunk = 2 * threads;
  std::vector<std::vector<uint8_t>> cf;
  std::vector<FrameCode> z;
  for (size_t f0 = 0; f0 < n_frames; f0 += chunk) {
    const size_t m = std::min(chunk, n_frames - f0);
    if (blocks) {
      cf.assign(m, {});
      if (!parallel_for(m, threads, [&](size_t i) {
            cf[i] = endpoint_coefficients(blocks + (f0 + i) * n, w->bw, w->bh);
            return true;
          }))
        throw std::bad_alloc();
    }
    z.assign(m, FrameCode{});
    if (!parallel_for(5 * m, threads, [&](size_t j) {
          const size_t i = j / 5;
          const uint8_t *c = blocks ? cf[i].data() : coeff + (f0 + i) * 6 * n;
          z[i][j % 5] = code_part(c, motion + (f0 + i) * 2 * n, n, (int)(j % 5));
          return true;
        }))
      throw std::bad_alloc();
    for (size_t i = 0; i < m; ++i)
      append_record(w, z[i], n_unique[f0 + i] ? unique + (f0 + i) * n : nullptr, n_unique[f0 + i]);
  }
}

}  // namespace

extern "C" {

mptc_status mptc_stream_writer_create(int32_t width, int32_t height, int32_t search_area, int32_t unique_interval,
                                      int32_t total_frames, mptc_stream_writer **out) {
  if (!out || width <= 0 || height <= 0 || (width % 256) || (height % 256) || unique_interval <= 0 ||
      unique_interval > 255 || total_frames < 0 || search_area < 1 || search_area > 63 ||
      (int64_t)width * height > (int64_t)1 << 30)
    return MPTC_EINVAL;
  mptc_stream_writer *w = new (std::nothrow) mptc_stream_writer();
  if (!w) return MPTC_ENOMEM;
  w->width = width;
  w->height = height;
  w->bw = width / 4;
  w->bh = height / 4;
  w->sa = search_area;
  w->unique_interval = unique_interval;
  w->total_frames = total_frames;
  // header, codec/codec.cpp:1354-1367; the five maxima are patched at the end
  try {
    put_u32(w->stream, (uint32_t)height);
    put_u32(w->stream, (uint32_t)width);
    w->stream.push_back((uint8_t)unique_interval);
    w->stream.push_back((uint8_t)search_area);
    put_u32(w->stream, (uint32_t)(total_frames / unique_interval));
    for (int k = 0; k < 5; ++k) put_u32(w->stream, 0);
  } catch (...) {
    delete w;
    return MPTC_ENOMEM;
  }
  *out = w;
  return MPTC_OK;
}

mptc_status mptc_stream_writer_destroy(mptc_stream_writer *w) {
  if (!w) return MPTC_EINVAL;
  delete w;
  return MPTC_OK;
}

mptc_status mptc_stream_writer_add_frame(mptc_stream_writer *w, const uint64_t *blocks, const uint8_t *motion,
                                         const uint32_t *unique, uint32_t n_unique) {
  if (!w || !blocks || !motion || (n_unique && !unique)) return MPTC_EINVAL;
  if (n_unique > (size_t)w->bw * w->bh) return MPTC_EINVAL;
  if (w->failed) return MPTC_ESTATE;
  try {
    const std::vector<uint8_t> coeff = endpoint_coefficients(blocks, w->bw, w->bh);
    append_frame(w, coeff.data(), motion, unique, n_unique);
  } catch (...) {
    w->failed = true;
    return MPTC_ENOMEM;
  }
  return MPTC_OK;
}

mptc_status mptc_stream_writer_add_frame_coefficients(mptc_stream_writer *w, const uint8_t *coeff,
                                                      const uint8_t *motion, const uint32_t *unique,
                                                      uint32_t n_unique) {
  if (!w || !coeff || !motion || (n_unique && !unique)) return MPTC_EINVAL;
  if (n_unique > (size_t)w->bw * w->bh) return MPTC_EINVAL;
  if (w->failed) return MPTC_ESTATE;
  try {
    append_frame(w, coeff, motion, unique, n_unique);
  } catch (...) {
    w->failed = true;
    return MPTC_ENOMEM;
  }
  return MPTC_OK;
}

// Shared checks and error handling of the two run calls.
static mptc_status add_frames(mptc_stream_writer *w, int32_t n_frames, const uint64_t *blocks, const uint8_t *coeff,
                              const uint8_t *motion, const uint32_t *unique, const uint32_t *n_unique) {
  if (!w || n_frames < 0 || (n_frames > 0 && ((!blocks && !coeff) || !motion || !n_unique))) return MPTC_EINVAL;
  const size_t n = (size_t)w->bw * w->bh;
  for (int32_t f = 0; f < n_frames; ++f)
    if (n_unique[f] > n || (n_unique[f] && !unique)) return MPTC_EINVAL;
  if (w->failed) return MPTC_ESTATE;
  try {
    append_frames(w, (size_t)n_frames, blocks, coeff, motion, unique, n_unique);
  } catch (...) {
    w->failed = true;
    return MPTC_ENOMEM;
  }
  return MPTC_OK;
}

mptc_status mptc_stream_writer_add_frames(mptc_stream_writer *w, int32_t n_frames, const uint64_t *blocks,
                                          const uint8_t *motion, const uint32_t *unique, const uint32_t *n_unique) {
  return add_frames(w, n_frames, blocks, nullptr, motion, unique, n_unique);
}

mptc_status mptc_stream_writer_add_frames_coefficients(mptc_stream_writer *w, int32_t n_frames,
                                                       const uint8_t *coeff, const uint8_t *motion,
                                                       const uint32_t *unique, const uint32_t *n_unique) {
  if (!coeff && n_frames > 0) return MPTC_EINVAL;
  return add_frames(w, n_frames, nullptr, coeff, motion, unique, n_unique);
}

mptc_status mptc_stream_writer_finish(mptc_stream_writer *w, uint8_t *out, uint64_t *size) {
  if (!w || !size) return MPTC_EINVAL;
  if (w->failed) return MPTC_ESTATE;
  // the five maxima at byte 14 (codec/codec.cpp:1514-1520)
  const uint32_t mx[5] = {w->max_unique, w->max_palette, w->max_motion, w->max_ep_y, w->max_ep_c};
  for (int k = 0; k < 5; ++k)
    for (int b = 0; b < 4; ++b) w->stream[14 + 4 * k + b] = (uint8_t)(mx[k] >> (8 * b));
  *size = w->stream.size();
  if (out) std::memcpy(out, w->stream.data(), w->stream.size());
  return MPTC_OK;
}

mptc_status mptc_stream_writer_frame_sizes(const mptc_stream_writer *w, uint32_t *motion_bytes,
                                           uint32_t *endpoint_bytes) {
  if (!w) return MPTC_EINVAL;
  if (motion_bytes) *motion_bytes = w->last_motion;
  if (endpoint_bytes)
    for (int k = 0; k < 4; ++k) endpoint_bytes[k] = w->last_ep[k];
  return MPTC_OK;
}

}  // extern "C"
