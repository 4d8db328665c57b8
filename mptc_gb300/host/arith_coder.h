// Adaptive arithmetic coder of the MPTC stream.
//
// The 32-bit multiplication-based coder with adaptive multi-symbol models of
// A. Said's "FastAC" as the reference vendors it (entropy/arithmetic_codec.cpp:
// carry :81-86, renormalisation :90-96 and :100-105, adaptive encode :360-388,
// adaptive decode :391-440, start/stop :498-573, model update/reset :781-826):
// the interval [base, base + length) shrinks by each symbol's share of a
// cumulative distribution of 2^15; the distribution is rebuilt from symbol
// counts on a cycle that grows by 5/4 up to 8 * (symbols + 6) symbols; counts
// are halved once their total passes 2^15. Every stream part (motion codes,
// each endpoint plane pair, a group's palette) starts a fresh coder and model.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace mptc_host {

constexpr uint32_t kMinLength = 0x01000000u;  // renormalise below this length
constexpr uint32_t kMaxLength = 0xFFFFFFFFu;
constexpr uint32_t kLengthShift = 15;         // distribution resolution (bits)
constexpr uint32_t kMaxCount = 1u << kLengthShift;

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
  // Largest s with lo(s) <= v (lo(0) == 0).
  uint32_t find(uint32_t v) const {
    uint32_t s = 0, e = n_;
    while (e - s > 1) {
      const uint32_t m = (s + e) >> 1;
      if (dist_[m] > v) e = m;
      else s = m;
    }
    return s;
  }
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
  // Final bytes (one or two more); returns the code.
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

// Reads past the end of the code as zero bytes.
class ArithmeticDecoder {
 public:
  ArithmeticDecoder(const uint8_t *code, size_t size) : code_(code), size_(size) {
    for (int k = 0; k < 4; ++k) value_ = (value_ << 8) | next();
  }
  uint32_t decode(AdaptiveModel &m) {
    const uint32_t unit = length_ >> kLengthShift;
    const uint32_t s = m.find(value_ / unit);
    const uint32_t x = m.lo(s) * unit;
    const uint32_t y = s == m.symbols() - 1 ? length_ : m.hi(s) * unit;
    value_ -= x;
    length_ = y - x;
    if (length_ < kMinLength) {
      do {
        value_ = (value_ << 8) | next();
      } while ((length_ <<= 8) < kMinLength);
    }
    m.seen(s);
    return s;
  }

 private:
  uint32_t next() { return pos_ < size_ ? code_[pos_++] : (++pos_, 0u); }

  const uint8_t *code_;
  size_t size_, pos_ = 0;
  uint32_t value_ = 0, length_ = kMaxLength;
};

// A byte sequence through a fresh 257-symbol adaptive model (the reference's
// EntropyEncode of a byte vector, codec/codec.cpp:186-201).
inline std::vector<uint8_t> code_bytes(const uint8_t *data, size_t n) {
  AdaptiveModel m(257);
  ArithmeticEncoder enc;
  for (size_t i = 0; i < n; ++i) enc.encode(data[i], m);
  return enc.finish();
}

// Inverse of code_bytes for n symbols (EntropyDecode, codec/decoder.cpp:44-65).
// Returns false if a decoded symbol is not a byte (256, the model's escape).
inline bool decode_bytes(const uint8_t *code, size_t size, uint8_t *out, size_t n) {
  AdaptiveModel m(257);
  ArithmeticDecoder dec(code, size);
  for (size_t i = 0; i < n; ++i) {
    const uint32_t s = dec.decode(m);
    if (s > 255) return false;
    out[i] = (uint8_t)s;
  }
  return true;
}

}  // namespace mptc_host
