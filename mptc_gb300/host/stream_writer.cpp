// Host-side MPTC stream writer (include/mptc_host.h): the container, the
// adaptive arithmetic coder and the endpoint transform of the reference
// encoder, restated so that a stream built from this library's per-frame
// arrays is byte-identical to the reference encoder's stream.
//
// Arithmetic coder: the 32-bit multiplication-based coder with adaptive
// multi-symbol models of A. Said's "FastAC" (as vendored in the reference,
// entropy/arithmetic_codec.cpp:80-120, :360-388, :498-507, :547-573,
// :781-826): interval [base, base + length), models that rescale a cumulative
// distribution of 2^15 periodically from symbol counts, carry propagation into
// the bytes already written.
#include "../../include/mptc_host.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

namespace {

constexpr uint32_t kMinLength = 0x01000000u;  // renormalise below this length
constexpr uint32_t kMaxLength = 0xFFFFFFFFu;
constexpr uint32_t kLengthShift = 15;         // distribution resolution (bits)
constexpr uint32_t kMaxCount = 1u << kLengthShift;

// Adaptive multi-symbol model: counts start at one; the cumulative
// distribution is recomputed after `update_cycle` symbols, the cycle growing
// by 5/4 up to 8 * (symbols + 6); counts are halved past kMaxCount.
class AdaptiveModel {
 public:
  explicit AdaptiveModel(uint32_t symbols) : n_(symbols), dist_(symbols), count_(symbols, 1u) {
    total_ = 0;
    cycle_ = n_;
    rebuild();
    until_ = cycle_ = (n_ + 6) >> 1;
  }
  uint32_t symbols() const { return n_; }
  uint32_t lo(uint32_t s) const { return dist_[s]; }
  uint32_t hi(uint32_t s) const { return dist_[s + 1]; }
  void seen(uint32_t s) {
    ++count_[s];
    if (--until_ == 0) rebuild();
  }

 private:
  void rebuild() {
    if ((total_ += cycle_) > kMaxCount) {
      total_ = 0;
      for (uint32_t k = 0; k < n_; ++k) total_ += (count_[k] = (count_[k] + 1) >> 1);
    }
    const uint32_t scale = 0x80000000u / total_;
    uint32_t sum = 0;
    for (uint32_t k = 0; k < n_; ++k) {
      dist_[k] = (scale * sum) >> (31 - kLengthShift);
      sum += count_[k];
    }
    cycle_ = (5 * cycle_) >> 2;
    const uint32_t max_cycle = (n_ + 6) << 3;
    if (cycle_ > max_cycle) cycle_ = max_cycle;
    until_ = cycle_;
  }

  uint32_t n_;
  std::vector<uint32_t> dist_, count_;
  uint32_t total_ = 0, cycle_ = 0, until_ = 0;
};

class ArithmeticEncoder {
 public:
  void encode(uint32_t s, AdaptiveModel &m) {
    const uint32_t before = base_;
    uint32_t x;
    if (s == m.symbols() - 1) {  // last symbol: the interval's top end
      x = m.lo(s) * (length_ >> kLengthShift);
      base_ += x;
      length_ -= x;
    } else {
      length_ >>= kLengthShift;
      x = m.lo(s) * length_;
      base_ += x;
      length_ = m.hi(s) * length_ - x;
    }
    if (before > base_) carry();
    if (length_ < kMinLength) renormalise();
    m.seen(s);
  }
  // Final bytes; returns the code.
  std::vector<uint8_t> &finish() {
    const uint32_t before = base_;
    if (length_ > 2 * kMinLength) {
      base_ += kMinLength;
      length_ = kMinLength >> 1;
    } else {
      base_ += kMinLength >> 1;
      length_ = kMinLength >> 9;
    }
    if (before > base_) carry();
    renormalise();
    return out_;
  }

 private:
  void carry() {
    for (size_t p = out_.size(); p-- > 0;) {
      if (out_[p] != 0xFF) {
        ++out_[p];
        return;
      }
      out_[p] = 0;
    }
  }
  void renormalise() {
    do {
      out_.push_back((uint8_t)(base_ >> 24));
      base_ <<= 8;
    } while ((length_ <<= 8) < kMinLength);
  }

  uint32_t base_ = 0, length_ = kMaxLength;
  std::vector<uint8_t> out_;
};

// A byte sequence through a fresh 257-symbol adaptive model.
std::vector<uint8_t> code_bytes(const uint8_t *data, size_t n) {
  AdaptiveModel m(257);
  ArithmeticEncoder enc;
  for (size_t i = 0; i < n; ++i) enc.encode(data[i], m);
  return enc.finish();
}

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
};

extern "C" {

mptc_status mptc_stream_writer_create(int32_t width, int32_t height, int32_t search_area, int32_t unique_interval,
                                      int32_t total_frames, mptc_stream_writer **out) {
  if (!out || width <= 0 || height <= 0 || (width % 256) || (height % 256) || unique_interval <= 0 ||
      unique_interval > 255 || total_frames < 0 || search_area < 1 || search_area > 63)
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
  put_u32(w->stream, (uint32_t)height);
  put_u32(w->stream, (uint32_t)width);
  w->stream.push_back((uint8_t)unique_interval);
  w->stream.push_back((uint8_t)search_area);
  put_u32(w->stream, (uint32_t)(total_frames / unique_interval));
  for (int k = 0; k < 5; ++k) put_u32(w->stream, 0);
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
  const size_t n = (size_t)w->bw * w->bh;
  if (n_unique > n) return MPTC_EINVAL;
  std::vector<uint8_t> rec;
  // frame record: unique count, motion codes (codec/codec.cpp:1119-1153)
  const std::vector<uint8_t> mo = code_bytes(motion, 2 * n);
  put_u32(rec, n_unique);
  put_u32(rec, (uint32_t)mo.size());
  rec.insert(rec.end(), mo.begin(), mo.end());
  w->max_motion = std::max(w->max_motion, (uint32_t)mo.size());
  w->last_motion = (uint32_t)mo.size();
  // endpoint images (CompressEndpoint, codec/codec.cpp:804-899)
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
    const std::vector<uint8_t> cy = plane_coefficients(Y, w->bw, w->bh);
    std::vector<uint8_t> cc = plane_coefficients(Co, w->bw, w->bh);
    const std::vector<uint8_t> ccg = plane_coefficients(Cg, w->bw, w->bh);
    cc.insert(cc.end(), ccg.begin(), ccg.end());
    const std::vector<uint8_t> zy = code_bytes(cy.data(), cy.size());
    const std::vector<uint8_t> zc = code_bytes(cc.data(), cc.size());
    put_u32(rec, (uint32_t)zy.size());
    rec.insert(rec.end(), zy.begin(), zy.end());
    put_u32(rec, (uint32_t)zc.size());
    rec.insert(rec.end(), zc.begin(), zc.end());
    w->max_ep_y = std::max(w->max_ep_y, (uint32_t)zy.size());
    w->max_ep_c = std::max(w->max_ep_c, (uint32_t)zc.size());
    w->last_ep[2 * e] = (uint32_t)zy.size();
    w->last_ep[2 * e + 1] = (uint32_t)zc.size();
  }
  w->group_records.insert(w->group_records.end(), rec.begin(), rec.end());
  // unique palette of the group (codec/codec.cpp:1471-1505): u32 entries as bytes
  const uint8_t *pb = reinterpret_cast<const uint8_t *>(unique);
  w->group_palette.insert(w->group_palette.end(), pb, pb + 4 * (size_t)n_unique);
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
  return MPTC_OK;
}

mptc_status mptc_stream_writer_finish(mptc_stream_writer *w, uint8_t *out, uint64_t *size) {
  if (!w || !size) return MPTC_EINVAL;
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
