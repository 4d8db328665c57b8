// Test infrastructure: drives the UNMODIFIED reference hot path
// (MPTC::DXTImage constructor + DXTImage::Reencode, codec/dxt_image.cpp:385-436
// and :868-957) over a raw RGB8 frame sequence and dumps what it produced.
//
// The reference constructor only accepts a PNG path, so each frame is written
// as a temporary PNG with stb_image_write (linked from the reference's own
// dxt_image.cpp) and loaded back by the constructor; PNG is lossless.
//
// Frame sequencing follows CompressMultiUnique (codec/codec.cpp:1379-1508):
// frame 1 is intra, then every `intra_interval`-th frame; prev_frame is the
// previous frame's final state.
//
// usage: hotpath_harness frames.rgb W H N search_area threshold intra_interval out.bin tmpdir
// out.bin, per frame: u64 stb[nblk] | u64 final[nblk] | u8 motion[2*nblk] |
//                     u32 n_unique | u32 unique[n_unique] | f64 psnr
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "dxt_image.h"
#include "stb_image_write.h"

int main(int argc, char **argv) {
  if (argc != 10) {
    std::fprintf(stderr, "usage: %s frames.rgb W H N sa thr intra_interval out.bin tmpdir\n", argv[0]);
    return 2;
  }
  const std::string in_path = argv[1];
  const int W = std::atoi(argv[2]), H = std::atoi(argv[3]), N = std::atoi(argv[4]);
  const int sa = std::atoi(argv[5]), thr = std::atoi(argv[6]), intra_interval = std::atoi(argv[7]);
  const std::string out_path = argv[8], tmpdir = argv[9];

  std::ifstream in(in_path, std::ios::binary);
  std::ofstream out(out_path, std::ios::binary);
  if (!in || !out) { std::fprintf(stderr, "cannot open files\n"); return 2; }

  const size_t fsz = static_cast<size_t>(W) * H * 3;
  std::vector<uint8_t> frame(fsz);
  std::unique_ptr<MPTC::DXTImage> prev, cur;
  bool set_intra = true;
  uint32_t curr_intra_num = 1;
  const std::string png = tmpdir + "/frame.png";

  for (int f = 0; f < N; ++f) {
    in.read(reinterpret_cast<char *>(frame.data()), fsz);
    if (!in) { std::fprintf(stderr, "short input\n"); return 2; }
    if (!stbi_write_png(png.c_str(), W, H, 3, frame.data(), W * 3)) {
      std::fprintf(stderr, "png write failed\n");
      return 2;
    }
    cur.reset(new MPTC::DXTImage(png, set_intra, sa, thr));
    const size_t nblk = cur->_physical_blocks.size();
    std::vector<uint64_t> stb(nblk);
    for (size_t i = 0; i < nblk; ++i) stb[i] = cur->_physical_blocks[i].dxt_block;

    cur->Reencode(prev, -1);

    std::vector<uint64_t> fin(nblk);
    for (size_t i = 0; i < nblk; ++i) fin[i] = cur->_physical_blocks[i].dxt_block;
    std::vector<uint8_t> motion;
    motion.reserve(2 * nblk);
    for (auto &m : cur->_motion_indices) {
      motion.push_back(std::get<0>(m));
      motion.push_back(std::get<1>(m));
    }
    if (motion.size() != 2 * nblk) { std::fprintf(stderr, "motion size mismatch\n"); return 3; }
    uint32_t nu = static_cast<uint32_t>(cur->_unique_palette.size());
    double psnr = cur->PSNR();

    out.write(reinterpret_cast<const char *>(stb.data()), nblk * 8);
    out.write(reinterpret_cast<const char *>(fin.data()), nblk * 8);
    out.write(reinterpret_cast<const char *>(motion.data()), 2 * nblk);
    out.write(reinterpret_cast<const char *>(&nu), 4);
    out.write(reinterpret_cast<const char *>(cur->_unique_palette.data()), 4 * nu);
    out.write(reinterpret_cast<const char *>(&psnr), 8);

    // intra-interval toggle, codec/codec.cpp:1462-1469
    if (curr_intra_num <= static_cast<uint32_t>(intra_interval)) {
      set_intra = false;
      if (curr_intra_num == static_cast<uint32_t>(intra_interval)) {
        set_intra = true;
        curr_intra_num = 1;
      } else {
        curr_intra_num++;
      }
    }
    prev = std::move(cur);
  }
  std::remove(png.c_str());
  return 0;
}
