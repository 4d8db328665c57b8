// Host-side MPTC stream reader (include/mptc_host.h): walks the container the
// writer produces (codec/codec.cpp:1354-1505 layout) and arithmetic-decodes
// each frame's parts, as the reference decoder's GetFrame does
// (codec/decoder.cpp:256-414), without its rewind after the last group's
// palette. The five parts of a frame decode concurrently on large frames.
#include "../../include/mptc_host.h"
#include "arith_coder.h"
#include "parallel.h"

#include <cstring>
#include <new>
#include <thread>
#include <vector>

namespace {

constexpr size_t kParallelBlocks = 16384;

uint32_t get_u32(const uint8_t *p) { return (uint32_t)p[0] | (uint32_t)p[1] << 8 | (uint32_t)p[2] << 16 | (uint32_t)p[3] << 24; }

}  // namespace

struct mptc_stream_reader {
  std::vector<uint8_t> data;
  mptc_stream_info info{};
  size_t nblk = 0;
  size_t pos = 34;               // next unread byte
  uint32_t frame = 0;            // frames returned
  std::vector<uint8_t> palette;  // decoded palette bytes of the current group
  size_t palette_used = 0;

  bool take(size_t n, const uint8_t **p) {
    if (n > data.size() - pos) return false;
    *p = data.data() + pos;
    pos += n;
    return true;
  }
  bool take_u32(uint32_t *v) {
    const uint8_t *p;
    if (!take(4, &p)) return false;
    *v = get_u32(p);
    return true;
  }
};

extern "C" {

mptc_status mptc_stream_reader_open(const uint8_t *data, uint64_t size, mptc_stream_reader **out) {
  if (!out || (!data && size) || size < 34) return MPTC_EINVAL;
  mptc_stream_info in{};
  in.height = (int32_t)get_u32(data);
  in.width = (int32_t)get_u32(data + 4);
  in.unique_interval = data[8];
  in.search_area = data[9];
  in.groups = get_u32(data + 10);
  in.max_unique_count = get_u32(data + 14);
  in.max_compressed_palette = get_u32(data + 18);
  in.max_compressed_motion_indices = get_u32(data + 22);
  in.max_compressed_ep_y = get_u32(data + 26);
  in.max_compressed_ep_c = get_u32(data + 30);
  if (in.width <= 0 || in.height <= 0 || in.width % 256 || in.height % 256 || in.unique_interval < 1 ||
      in.search_area < 1 || in.search_area > 63 || (int64_t)in.width * in.height > (int64_t)1 << 30)
    return MPTC_EINVAL;
  in.frames = in.groups * (uint32_t)in.unique_interval;
  mptc_stream_reader *r = new (std::nothrow) mptc_stream_reader();
  if (!r) return MPTC_ENOMEM;
  try {
    r->data.assign(data, data + size);
  } catch (...) {
    delete r;
    return MPTC_ENOMEM;
  }
  r->info = in;
  r->nblk = (size_t)(in.width / 4) * (in.height / 4);
  *out = r;
  return MPTC_OK;
}

mptc_status mptc_stream_reader_destroy(mptc_stream_reader *r) {
  if (!r) return MPTC_EINVAL;
  delete r;
  return MPTC_OK;
}

mptc_status mptc_stream_reader_info(const mptc_stream_reader *r, mptc_stream_info *info) {
  if (!r || !info) return MPTC_EINVAL;
  *info = r->info;
  return MPTC_OK;
}

}  // extern "C"

namespace {

// One frame record parsed: its five coded parts, not yet decoded.
struct FrameParts {
  const uint8_t *code[5];
  uint32_t size[5];
};

// Reads the next frame's record (and its group's palette first, at a group
// start), copies the frame's palette slice to `unique`; the parts stay coded.
mptc_status parse_frame(mptc_stream_reader *r, FrameParts *fp, uint32_t *unique, uint32_t *n_unique) {
  if (r->frame >= r->info.frames) return MPTC_ESTATE;
  const size_t n = r->nblk;
  if (r->frame % (uint32_t)r->info.unique_interval == 0) {
    // group start: [u32 palette_size][palette code][u32 palette bytes] (decoder.cpp:341-357)
    uint32_t psz, count;
    const uint8_t *pc;
    if (!r->take_u32(&psz) || !r->take(psz, &pc) || !r->take_u32(&count)) return MPTC_EINVAL;
    if (count > 4 * n * (size_t)r->info.unique_interval) return MPTC_EINVAL;
    try {
      r->palette.assign(count, 0);
    } catch (...) {
      return MPTC_ENOMEM;
    }
    if (!mptc_host::decode_bytes(pc, psz, r->palette.data(), count)) return MPTC_EINVAL;
    r->palette_used = 0;
  }
  // frame record: [u32 n_unique][u32 size][motion] then 4 x [u32 size][part] (decoder.cpp:361-401)
  uint32_t nu;
  if (!r->take_u32(&nu)) return MPTC_EINVAL;
  for (int k = 0; k < 5; ++k)
    if (!r->take_u32(&fp->size[k]) || !r->take(fp->size[k], &fp->code[k])) return MPTC_EINVAL;
  if (nu > n || 4 * (size_t)nu > r->palette.size() - r->palette_used) return MPTC_EINVAL;
  std::memcpy(unique, r->palette.data() + r->palette_used, 4 * (size_t)nu);
  r->palette_used += 4 * (size_t)nu;
  *n_unique = nu;
  ++r->frame;
  return MPTC_OK;
}

// Decodes part k of a parsed frame into the frame's motion / coefficient buffers.
bool decode_part(const FrameParts &fp, size_t n, int k, uint8_t *motion, uint8_t *coeff) {
  uint8_t *dst[5] = {motion, coeff, coeff + n, coeff + 3 * n, coeff + 4 * n};
  const size_t len[5] = {2 * n, n, 2 * n, n, 2 * n};
  return mptc_host::decode_bytes(fp.code[k], fp.size[k], dst[k], len[k]);
}

}  // namespace

extern "C" {

mptc_status mptc_stream_reader_next(mptc_stream_reader *r, uint8_t *motion, uint8_t *coeff, uint32_t *unique,
                                    uint32_t *n_unique) {
  if (!r || !motion || !coeff || !unique || !n_unique) return MPTC_EINVAL;
  FrameParts fp;
  uint32_t nu = 0;
  const mptc_status st = parse_frame(r, &fp, unique, &nu);
  if (st != MPTC_OK) return st;
  // the five parts on five threads when the frame is large
  const size_t n = r->nblk;
  if (!mptc_host::parallel_for(5, n >= kParallelBlocks ? 5 : 1,
                               [&](size_t k) { return decode_part(fp, n, (int)k, motion, coeff); }))
    return MPTC_EINVAL;
  *n_unique = nu;
  return MPTC_OK;
}

mptc_status mptc_stream_reader_next_frames(mptc_stream_reader *r, int32_t max_frames, uint8_t *motion, uint8_t *coeff,
                                           uint32_t *unique, uint32_t *n_unique, int32_t *n_read) {
  if (!r || max_frames < 0 || !n_read || (max_frames > 0 && (!motion || !coeff || !unique || !n_unique)))
    return MPTC_EINVAL;
  *n_read = 0;
  const size_t n = r->nblk;
  std::vector<FrameParts> parts;
  try {
    parts.reserve((size_t)max_frames);
  } catch (...) {
    return MPTC_ENOMEM;
  }
  // records are parsed in order (their sizes locate the next one), then every
  // part of every parsed frame is decoded on all the host's cores
  while ((int32_t)parts.size() < max_frames) {
    const size_t f = parts.size();
    FrameParts fp;
    const mptc_status st = parse_frame(r, &fp, unique + f * n, &n_unique[f]);
    if (st == MPTC_ESTATE) break;
    if (st != MPTC_OK) return st;
    parts.push_back(fp);
  }
  if (parts.empty() && max_frames > 0) return MPTC_ESTATE;
  if (!mptc_host::parallel_for(5 * parts.size(), mptc_host::host_threads(), [&](size_t j) {
        const size_t f = j / 5;
        return decode_part(parts[f], n, (int)(j % 5), motion + 2 * f * n, coeff + 6 * f * n);
      }))
    return MPTC_EINVAL;
  *n_read = (int32_t)parts.size();
  return MPTC_OK;
}

}  // extern "C"
