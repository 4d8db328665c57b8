/*
 * mptc_host — host-side MPTC stream writer and reader (no GPU). The writer
 * turns the arrays the encoder returns per frame (final DXT1 blocks, motion codes, unique index
 * palette) into the MPTC container bytes, exactly as the reference encoder's
 * CompressMultiUnique (codec/codec.cpp:1307-1532) writes them:
 *
 *   header (34 bytes): u32 height, u32 width, u8 unique_interval,
 *     u8 search_area, u32 groups (= frames / unique_interval), then u32
 *     max_unique_count, max_compressed_palette, max_compressed_motion_indices,
 *     max_compressed_ep_Y, max_compressed_ep_C (patched when the stream ends);
 *   per group of unique_interval frames: u32 palette_size, the arithmetic-coded
 *     palette bytes of the group, u32 palette byte count, then every frame record;
 *   frame record (EntropyEncode, codec/codec.cpp:1115-1158): u32 n_unique,
 *     u32 motion_size, arithmetic-coded motion codes (x then y per block), then
 *     the endpoint images (CompressEndpoint, :804-899): for ep1 then ep2,
 *     RGB565 -> YCoCg-667, a 6-level integer 5/3 wavelet per 64x64 tile and
 *     per plane, coefficients + 128, arithmetic coding of the Y plane and of
 *     the Co plane followed by the Cg plane, each with a u32 size prefix.
 *
 * Like the reference, frames after the last complete group are coded (they
 * count towards the maximum sizes) but not written, and the endpoint images
 * must be multiples of 64 blocks in each direction (frame sizes multiples of
 * 256 pixels): other sizes are rejected here, where the reference would write
 * out of bounds. A writer or reader object is not thread-safe; separate
 * objects may be used from separate threads.
 */
#ifndef MPTC_HOST_H_
#define MPTC_HOST_H_

#include <stdint.h>

#include "mptc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mptc_stream_writer mptc_stream_writer;

/* `total_frames` is the number of frames the caller will add (it fixes the
 * header's group count, codec/codec.cpp:1357). Frames are at most 2^30
 * pixels. If host memory runs out while a frame is added, the call returns
 * MPTC_ENOMEM and every later add or finish call MPTC_ESTATE. */
mptc_status mptc_stream_writer_create(int32_t width, int32_t height, int32_t search_area,
                                      int32_t unique_interval, int32_t total_frames,
                                      mptc_stream_writer **out_writer);
mptc_status mptc_stream_writer_destroy(mptc_stream_writer *writer);

/* One encoded frame: blocks (width/4 * height/4 u64, the final physical
 * blocks), motion (2 bytes per block), the unique palette and its length. */
mptc_status mptc_stream_writer_add_frame(mptc_stream_writer *writer, const uint64_t *final_blocks,
                                         const uint8_t *motion, const uint32_t *unique_palette,
                                         uint32_t n_unique);

/* The same frame with its endpoint images already transformed (for instance by
 * mptc_endpoint_coefficients on the GPU): `coeff` holds the six coefficient
 * planes [Y1 | Co1 | Cg1 | Y2 | Co2 | Cg2] of blocks bytes each, the byte
 * vectors that CompressEndpoint codes (codec/codec.cpp:838-846). */
mptc_status mptc_stream_writer_add_frame_coefficients(mptc_stream_writer *writer, const uint8_t *coeff,
                                                      const uint8_t *motion, const uint32_t *unique_palette,
                                                      uint32_t n_unique);

/* A run of frames in one call, in the layout of mptc_encode_stream_host's
 * outputs: frame f's blocks at final_blocks + f * blocks, its motion codes at
 * motion + 2 * f * blocks, its palette at unique_palette + f * blocks with
 * n_unique[f] entries. The frames' endpoint transforms and coded parts are
 * computed on all the host's cores and appended in frame order: the bytes are
 * those of n_frames mptc_stream_writer_add_frame calls. The run is coded in
 * chunks of 2 x (host threads) frames; if host memory runs out part way, the
 * call returns MPTC_ENOMEM after the earlier chunks' records were appended,
 * and the writer is unusable from then on (every later add or finish call
 * returns MPTC_ESTATE), as after a failed single-frame call. The host threads
 * are the hardware threads, or MPTC_HOST_THREADS from the environment. */
mptc_status mptc_stream_writer_add_frames(mptc_stream_writer *writer, int32_t n_frames,
                                          const uint64_t *final_blocks, const uint8_t *motion,
                                          const uint32_t *unique_palette, const uint32_t *n_unique);

/* The same with the endpoint images already transformed: frame f's six
 * coefficient planes at coeff + 6 * f * blocks. */
mptc_status mptc_stream_writer_add_frames_coefficients(mptc_stream_writer *writer, int32_t n_frames,
                                                       const uint8_t *coeff, const uint8_t *motion,
                                                       const uint32_t *unique_palette, const uint32_t *n_unique);

/* Finishes the stream: *size receives its byte count; if `out` is not NULL
 * (room for *size bytes when called with out == NULL first) the bytes are
 * copied there. */
mptc_status mptc_stream_writer_finish(mptc_stream_writer *writer, uint8_t *out, uint64_t *size);

/* Sizes in bytes of the last added frame's coded parts: motion codes, the four
 * endpoint streams (Y1, C1, Y2, C2). Any pointer may be NULL. */
mptc_status mptc_stream_writer_frame_sizes(const mptc_stream_writer *writer, uint32_t *motion_bytes,
                                           uint32_t *endpoint_bytes);

/* ---- reader: the host half of the reference decoder's GetFrame
 * (codec/decoder.cpp:256-414): header, group palettes and per-frame parts,
 * arithmetic-decoded (EntropyDecode, decoder.cpp:44-65). The frame's blocks
 * are then rebuilt by mptc_decode_frame (include/mptc_gb300.h).
 *
 * Unlike GetFrame, which rewinds to the first group as soon as it has read
 * the last group's palette (decoder.cpp:404-409, so the later frames of that
 * group are never returned), the reader returns every frame of every
 * complete group, in order, then reports the end. */
typedef struct mptc_stream_info {
  int32_t width, height, search_area, unique_interval;
  uint32_t groups, frames; /* frames = groups * unique_interval */
  uint32_t max_unique_count, max_compressed_palette, max_compressed_motion_indices;
  uint32_t max_compressed_ep_y, max_compressed_ep_c;
} mptc_stream_info;

typedef struct mptc_stream_reader mptc_stream_reader;

/* Copies `size` bytes of stream; checks the header (sizes multiples of 256
 * pixels, at most 2^30 pixels, search area 1..63, unique interval >= 1). */
mptc_status mptc_stream_reader_open(const uint8_t *data, uint64_t size, mptc_stream_reader **out_reader);
mptc_status mptc_stream_reader_destroy(mptc_stream_reader *reader);
mptc_status mptc_stream_reader_info(const mptc_stream_reader *reader, mptc_stream_info *info);

/* Next frame's parts: motion (2 bytes per block), coeff (6 planes of blocks
 * bytes, the layout mptc_decode_frame reads), its slice of the group palette
 * (room for blocks entries) and the slice length. MPTC_ESTATE after the last
 * frame; MPTC_EINVAL on a truncated or inconsistent stream. */
mptc_status mptc_stream_reader_next(mptc_stream_reader *reader, uint8_t *motion, uint8_t *coeff,
                                    uint32_t *unique_palette, uint32_t *n_unique);

/* Up to max_frames next frames in one call, their parts decoded on all the
 * host's cores: frame f's motion codes at motion + 2 * f * blocks, its
 * coefficient planes at coeff + 6 * f * blocks, its palette slice at
 * unique_palette + f * blocks (n_unique[f] entries); *n_read frames were
 * read (fewer than max_frames at the end of the stream). MPTC_ESTATE when no
 * frame is left; MPTC_EINVAL on a truncated or inconsistent stream. The call
 * parses all the records it reads before decoding their parts, so an error in
 * any of them (or in decoding any part) returns MPTC_EINVAL with *n_read = 0
 * after the reader has moved past the parsed records: the frames of that call
 * are lost and the reader is unusable from then on (destroy it). */
mptc_status mptc_stream_reader_next_frames(mptc_stream_reader *reader, int32_t max_frames, uint8_t *motion,
                                           uint8_t *coeff, uint32_t *unique_palette, uint32_t *n_unique,
                                           int32_t *n_read);

#ifdef __cplusplus
}
#endif
#endif
