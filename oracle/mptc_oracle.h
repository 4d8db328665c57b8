/*
 * ORACLE — test infrastructure only.
 *
 * A CPU restatement of the MPTC encoder hot path (stb_dxt DXT1 block encode
 * and the index-block search of DXTImage::Reencode). Only tests/, the smoke
 * check and the CPU-baseline leg of bench.py may load it, and only as the
 * checker. The product path never calls it.
 *
 * Parity is pinned against the unmodified reference encoder (built from its
 * own sources by oracle/ref/Makefile) through the golden vectors under
 * tests/golden/.
 */
#ifndef MPTC_ORACLE_H_
#define MPTC_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Per-frame decision counters (what the reference loop visits and decides). */
typedef struct mo_stats {
  int64_t inter_visited;    /* candidate positions evaluated by the inter search */
  int64_t intra_visited;    /* candidate positions evaluated by the intra search */
  int64_t refits;           /* candidates that needed an endpoint refit */
  int32_t n_inter, n_intra, n_unique;
} mo_stats;

/* stb_dxt DXT1 encode (alpha=0, STB_DXT_HIGHQUAL) of one 4x4 RGBA block.
 * Returns the 8-byte block as a little-endian u64: ep1 | ep2<<16 | mask<<32. */
uint64_t mo_stb_encode_block(const uint8_t rgba[64]);

/* DXT1 encode of a whole RGB8 frame (width, height multiples of 4). */
int mo_dxt1_encode_frame(const uint8_t *rgb, int width, int height, uint64_t *blocks);

/* floor(SSE/48) of a DXT1 block against its 4x4 pixels (48 bytes RGB). */
int mo_block_error(const uint8_t px[48], uint64_t block);

/* Least-squares endpoint refit for candidate indices `interp`.
 * Writes the 8-bit endpoints (after the 5/6-bit snap) and returns floor(SSE/48)
 * of the refit palette; *valid = Pack565(ep1) > Pack565(ep2). */
int mo_refit(const uint8_t px[48], uint32_t interp, uint8_t ep1[3], uint8_t ep2[3], int *valid);

/* One frame of DXTImage::Reencode. prev_final == NULL means an intra frame.
 * Outputs: final blocks (nblk u64), motion (2*nblk bytes), unique palette
 * (up to nblk u32) with its length. `stats` may be NULL. */
int mo_reencode_frame(const uint8_t *rgb, int width, int height, const uint64_t *stb_blocks,
                      const uint64_t *prev_final, int search_area, int32_t err_threshold,
                      uint64_t *final_blocks, uint8_t *motion, uint32_t *unique_palette,
                      uint32_t *n_unique, mo_stats *stats);

/* Same, with the inter search split over `threads` POSIX threads (the inter
 * search is independent per block; the intra search stays sequential). */
int mo_reencode_frame_mt(const uint8_t *rgb, int width, int height, const uint64_t *stb_blocks,
                         const uint64_t *prev_final, int search_area, int32_t err_threshold,
                         uint64_t *final_blocks, uint8_t *motion, uint32_t *unique_palette,
                         uint32_t *n_unique, mo_stats *stats, int threads);

/* DXTImage::PSNR over the frame's final logical blocks. */
double mo_frame_psnr(const uint8_t *rgb, int width, int height, const uint64_t *final_blocks,
                     const uint64_t *stb_blocks);

/* Squared error of the frame against the decoded DXT1 blocks (RGB565 endpoints
 * expanded, PhysicalToLogical palettes), summed over every pixel and channel. */
uint64_t mo_decoded_sse(const uint8_t *rgb, int width, int height, const uint64_t *blocks);

#ifdef __cplusplus
}
#endif
#endif
