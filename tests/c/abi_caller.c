/* A plain C caller of the public headers (C99, built with -pedantic -Werror by
 * tests/test_c_abi_caller.py, and as C++): the GPU library's GPU-free calls,
 * then one frame through the host stream writer and back through the reader.
 * The exit code names the first failing step. */
#include "mptc_gb300.h"
#include "mptc_host.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
int main(void) {
  enum { W = 256, H = 256, N = (W / 4) * (H / 4) };
  static uint64_t blocks[N];
  static uint8_t motion[2 * N], coeff[6 * N], motion2[2 * N];
  static uint32_t unique[N], unique2[N];
  mptc_stream_writer *w = NULL;
  mptc_stream_reader *r = NULL;
  mptc_stream_info info;
  uint64_t size = 0;
  uint8_t *bytes;
  uint32_t nu = 0;
  int i;
  if (mptc_version() <= 0 || mptc_built_arch() != 1030) return 1;
  for (i = 0; i < N; ++i) {
    blocks[i] = (uint64_t)(0xF800u + (unsigned)i % 31u) | (uint64_t)0x001Fu << 16 | (uint64_t)0x55555555u << 32;
    motion[2 * i] = 255;
    motion[2 * i + 1] = 255;
    unique[i] = 0x55555555u;
  }
  if (mptc_stream_writer_create(W, H, 8, 1, 1, &w) != MPTC_OK) return 2;
  if (mptc_stream_writer_add_frame(w, blocks, motion, unique, N) != MPTC_OK) return 3;
  if (mptc_stream_writer_finish(w, NULL, &size) != MPTC_OK || size < 34) return 4;
  bytes = (uint8_t *)malloc((size_t)size);
  if (!bytes || mptc_stream_writer_finish(w, bytes, &size) != MPTC_OK) return 5;
  mptc_stream_writer_destroy(w);
  if (mptc_stream_reader_open(bytes, size, &r) != MPTC_OK) return 6;
  if (mptc_stream_reader_info(r, &info) != MPTC_OK || info.width != W || info.height != H || info.frames != 1) return 7;
  if (mptc_stream_reader_next(r, motion2, coeff, unique2, &nu) != MPTC_OK || nu != N) return 8;
  if (memcmp(motion, motion2, sizeof motion) || memcmp(unique, unique2, sizeof unique)) return 9;
  if (mptc_stream_reader_next(r, motion2, coeff, unique2, &nu) != MPTC_ESTATE) return 10;
  mptc_stream_reader_destroy(r);
  free(bytes);
  printf("ok %llu\n", (unsigned long long)size);
  return 0;
}
