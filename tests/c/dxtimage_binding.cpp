// The binding a maintainer adds beside the reference codec: a DXTImage filled
// by the GPU encoder (libmptc_gb300) instead of by the PNG constructor and
// DXTImage::Reencode, then handed to the reference's own EntropyEncode. It is
// compiled against the reference's headers and linked with the reference's
// codec/codec.cpp and codec/dxt_image.cpp (tests/test_reference_binding.py),
// so the fields it fills are the ones the reference codec reads.
//
// Reference call site replaced (codec/codec.cpp:1388-1394):
//   curr_frame.reset(new DXTImage(file, set_intra, search_area, vErrThreshold));
//   curr_frame->Reencode(prev_frame, -1);
#include <cstdint>
#include <iostream>
#include <memory>
#include <tuple>
#include <vector>

#include "codec.h"
#include "dxt_image.h"
#include "mptc_gb300.h"

namespace mptc_binding {

// One frame of RGB8 (width x height, multiples of 4) through the GPU encoder;
// the context keeps the previous frame's final blocks, so successive calls
// form the stream (is_intra as CompressMultiUnique's set_intra,
// codec/codec.cpp:1462-1469). Returns nullptr on an error (printed).
std::unique_ptr<MPTC::DXTImage> EncodeFrameOnGpu(mptc_ctx *gpu, const uint8_t *rgb, int width, int height,
                                                 bool is_intra) {
  // DXTImage(int, int, bool, unique_indices) sizes the block grid
  // (codec/dxt_image.cpp:437-450); the encoder fills the rest.
  std::unique_ptr<MPTC::DXTImage> img(new MPTC::DXTImage(width, height, is_intra, std::vector<uint32_t>()));
  const size_t n = static_cast<size_t>(img->_blocks_width) * img->_blocks_height;
  std::vector<uint64_t> fin(n);
  std::vector<uint8_t> motion(2 * n);
  img->_unique_palette.resize(n);
  uint32_t n_unique = 0;
  const mptc_status st = mptc_encode_frame_host(gpu, rgb, is_intra ? 1 : 0, nullptr, fin.data(), motion.data(),
                                                img->_unique_palette.data(), &n_unique, nullptr);
  if (st != MPTC_OK) {
    std::cerr << "mptc_encode_frame_host: " << mptc_last_error(gpu) << std::endl;
    return nullptr;
  }
  img->_unique_palette.resize(n_unique);
  img->_physical_blocks.resize(n);
  for (size_t i = 0; i < n; ++i) img->_physical_blocks[i].dxt_block = fin[i];
  img->_motion_indices.clear();
  img->_motion_indices.reserve(n);
  for (size_t i = 0; i < n; ++i) img->_motion_indices.emplace_back(motion[2 * i], motion[2 * i + 1]);
  // only PSNR() and the image views read the logical blocks and the source
  img->_logical_blocks.resize(n);
  for (size_t i = 0; i < n; ++i) img->_logical_blocks[i] = MPTC::PhysicalToLogical(img->_physical_blocks[i]);
  img->_src_img.assign(rgb, rgb + static_cast<size_t>(width) * height * 3);
  return img;
}

// The per-frame motion record of the reference stream for a run of frames,
// coded by the reference's EntropyEncode (codec/codec.cpp:1115-1158) from the
// GPU-encoded frames. Returns false on an error.
bool EncodeRecordsOnGpu(const mptc_config &cfg, const uint8_t *frames, int n_frames, int width, int height,
                        std::vector<std::vector<uint8_t>> &records) {
  mptc_ctx *gpu = nullptr;
  if (mptc_ctx_create(&cfg, width, height, &gpu) != MPTC_OK) return false;
  bool set_intra = true;
  uint32_t intra_num = 1;
  const size_t frame_bytes = static_cast<size_t>(width) * height * 3;
  bool ok = true;
  for (int f = 0; f < n_frames && ok; ++f) {
    std::unique_ptr<MPTC::DXTImage> curr = EncodeFrameOnGpu(gpu, frames + f * frame_bytes, width, height, set_intra);
    if (!curr) {
      ok = false;
      break;
    }
    std::vector<uint8_t> rec;
    MPTC::EntropyEncode(curr, rec);
    records.push_back(std::move(rec));
    // the reference's intra schedule (codec/codec.cpp:1462-1469)
    if (intra_num <= static_cast<uint32_t>(cfg.intra_interval)) {
      set_intra = false;
      if (intra_num == static_cast<uint32_t>(cfg.intra_interval)) {
        set_intra = true;
        intra_num = 1;
      } else {
        ++intra_num;
      }
    }
  }
  mptc_ctx_destroy(gpu);
  return ok;
}

}  // namespace mptc_binding
