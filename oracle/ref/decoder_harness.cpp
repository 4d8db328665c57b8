// Test infrastructure: drives the UNMODIFIED reference decoder's GetFrame
// (codec/decoder.cpp:256-414) sequentially over an MPTC stream file and dumps
// the decoded physical blocks of each frame, for golden vectors of the GPU
// decoder. GetFrame is called the way a sequential player would: frame k
// decodes into curr with prev = frame k-1.
//
// GetFrame rewinds to the first group right after decoding the first frame of
// the last group (decoder.cpp:404-409), so only the first
// (groups - 1) * unique_interval + 1 frames are the stream's frames; the
// caller asks for no more than that.
//
// usage: decoder_harness stream.mptc n_frames out.bin
// out.bin: n_frames x (u64 blocks[width/4 * height/4])
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <vector>

#include "decoder.h"

int main(int argc, char **argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s stream.mptc n_frames out.bin\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1], std::ifstream::binary);
  if (!in.is_open()) return 3;
  uint32_t hw[2];
  in.read(reinterpret_cast<char *>(hw), 8);
  in.seekg(0);
  const size_t nblk = (size_t)(hw[0] / 4) * (hw[1] / 4);
  const int n = std::atoi(argv[2]);
  std::vector<PhysicalDXTBlock> a(nblk), b(nblk);
  PhysicalDXTBlock *prev = a.data(), *curr = b.data();
  MPTCDecodeInfo info;
  info.is_start = true;
  FILE *out = std::fopen(argv[3], "wb");
  if (!out) return 4;
  for (int k = 0; k < n; ++k) {
    if (GetFrame(in, prev, curr, &info) != 0) return 5;
    std::fwrite(curr, sizeof(PhysicalDXTBlock), nblk, out);
    std::swap(prev, curr);
  }
  std::fclose(out);
  return 0;
}
