/*
 * mptc_gb300 — GB300 (sm_103a) MPTC encoder hot path behind a C ABI.
 *
 * The reference encoder's hot path is the C++ class MPTC::DXTImage
 * (codec/dxt_image.h:46-198): its constructor DXT1-encodes a frame with
 * stb_dxt and DXTImage::Reencode runs the index-block search. This library
 * replaces those two steps with CUDA kernels and returns exactly the data the
 * rest of the reference codec reads from a DXTImage: the final physical
 * blocks (_physical_blocks), the motion codes (_motion_indices) and the unique
 * index palette (_unique_palette). Results are bit-identical to the reference.
 *
 * Conventions: every call returns an mptc_status; buffers are caller-owned;
 * `_dev` pointers are device memory, `_host` pointers host memory; `stream` is
 * a cudaStream_t passed as void* (NULL = legacy default stream). Frame width
 * and height must be multiples of 4 (the reference reads past the frame
 * otherwise, codec/dxt_image.cpp:128-139). A context, batch, model or decoder
 * is used by one host thread at a time; separate ones may be used from
 * separate threads at once (the shared per-device tables are uploaded under a
 * lock), except mptc_encode_frame_noalloc, whose calls share one scratch area.
 *
 * Layouts (little-endian, raster order of 4x4 blocks, blocks_wide = width/4):
 *   block  u64 = ep1 | ep2 << 16 | interp << 32   (PhysicalDXTBlock, dxt_image.h:16-23)
 *   motion u8[2] per block = (x, y); (255,255) marks a unique block,
 *          x|0x80,y|0x80 an inter match, plain x,y an intra match
 *          (codec/dxt_image.cpp:701, :761, :892-894, :953)
 *   unique u32 interp per unique block, in raster order (codec/dxt_image.cpp:954)
 */
#ifndef MPTC_GB300_H_
#define MPTC_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mptc_status {
  MPTC_OK = 0,
  MPTC_EINVAL = 1,    /* bad argument: size, search area, NULL pointer */
  MPTC_ENOMEM = 2,    /* device or pinned allocation failed */
  MPTC_ETIMEOUT = 3,  /* a bounded device-side wait expired; results invalid */
  MPTC_ECUDA = 4,     /* a CUDA runtime call failed */
  MPTC_ESTATE = 5     /* call order: e.g. an inter frame without a previous frame */
} mptc_status;

/* Encoder parameters. The reference takes them as required command-line
 * arguments (codec/encoder.cpp:467-470): search_area in blocks (1..63; 64
 * would collide with the unique sentinel), err_threshold on the per-block
 * error increase (DXTImage::DXTImage err_threshold, codec/dxt_image.cpp:385-394),
 * intra_interval as in CompressMultiUnique (codec/codec.cpp:1462-1469). */
typedef struct mptc_config {
  int32_t search_area;
  int32_t err_threshold;
  int32_t intra_interval;
  /* Fixed-point sweeps of an inter frame's intra pass before the exact
   * dataflow pass takes over (results are identical either way): 0 = the
   * default (6), negative = none (dataflow only), at most 32. */
  int32_t intra_sweeps;
} mptc_config;

typedef struct mptc_ctx mptc_ctx;

/* Per-frame counters of the last reencode on a context (host-side copy). */
typedef struct mptc_frame_stats {
  uint32_t n_inter, n_intra, n_unique;
  uint32_t is_intra;
  uint32_t n_fallback;  /* learned proposal: blocks that needed the exhaustive search */
} mptc_frame_stats;

/* Replaces the state the reference keeps in DXTImage statics and in the
 * constructor's arguments (codec/dxt_image.cpp:25, :357-358, :385-394) with an
 * explicit context for frames of `width` x `height`; allocates the device
 * scratch the kernels need. */
mptc_status mptc_ctx_create(const mptc_config *cfg, int32_t width, int32_t height,
                            mptc_ctx **out_ctx);
mptc_status mptc_ctx_destroy(mptc_ctx *ctx);

/* Stage 1, the DXTImage constructor's stb_dxt pass: CompressRGB + the block
 * loop, codec/dxt_image.cpp:123-149 and :419-431 (stb_compress_dxt_block with
 * alpha=0, STB_DXT_HIGHQUAL, Include/stb_dxt.h:613-627).
 * rgb_dev: width*height*3 bytes, row-major RGB8. blocks_dev: blocks u64.
 * orig_err_dev: per block floor(SSE/48) of the stb block (CompressedBlock::Error,
 * codec/dxt_image.cpp:258-276), consumed by mptc_reencode; may be NULL. */
mptc_status mptc_dxt1_encode(mptc_ctx *ctx, const uint8_t *rgb_dev, uint64_t *blocks_dev,
                             int32_t *orig_err_dev, void *stream);

/* Stage 2, DXTImage::Reencode(prev, ref) (codec/dxt_image.cpp:868-957): the
 * inter search over prev_final_dev (the previous frame's final blocks; NULL
 * makes this an intra frame), the causal intra search over this frame, and the
 * unique palette. stb_dev / orig_err_dev come from mptc_dxt1_encode on the same
 * frame. Writes final_dev (blocks), motion_dev (2 bytes/block), unique_dev
 * (up to blocks u32) and *n_unique_dev (device u32). */
mptc_status mptc_reencode(mptc_ctx *ctx, const uint8_t *rgb_dev, const uint64_t *stb_dev,
                          const int32_t *orig_err_dev, const uint64_t *prev_final_dev,
                          uint64_t *final_dev, uint8_t *motion_dev, uint32_t *unique_dev,
                          uint32_t *n_unique_dev, void *stream);

/* Stage 1 + 2 on one device-resident frame, using context-owned stb/orig_err
 * scratch. stb_dev may be NULL when the caller does not need the stb blocks. */
mptc_status mptc_encode_frame(mptc_ctx *ctx, const uint8_t *rgb_dev, const uint64_t *prev_final_dev,
                              uint64_t *stb_dev, uint64_t *final_dev, uint8_t *motion_dev,
                              uint32_t *unique_dev, uint32_t *n_unique_dev, void *stream);

/* The DXTImage(file, is_intra, ...) + Reencode pair on HOST buffers, the call a
 * host encoder loop makes per frame (codec/codec.cpp:1388-1394). The context
 * keeps the previous frame's final blocks on the device, so successive calls
 * form a stream; is_intra=1 starts (or restarts) it. Copies in on `stream`
 * through pinned staging, runs both stages and copies the outputs back before
 * returning. stb_host may be NULL. Returns the number of unique blocks in
 * *n_unique_host. */
mptc_status mptc_encode_frame_host(mptc_ctx *ctx, const uint8_t *rgb_host, int32_t is_intra,
                                   uint64_t *stb_host, uint64_t *final_host, uint8_t *motion_host,
                                   uint32_t *unique_host, uint32_t *n_unique_host, void *stream);

/* A run of n_frames frames from HOST buffers, the host encoder loop of
 * codec/codec.cpp:1383-1394 in one call: the same results as n_frames
 * successive mptc_encode_frame_host calls (the stream continues across
 * calls). frames_host holds the frames back to back (width*height*3 bytes
 * each), is_intra[k] flags frame k; frame k's outputs go to
 * final_host + k*nblk, motion_host + k*2*nblk, unique_host + k*nblk (its
 * n_unique_host[k] first entries; the copy covers all nblk) with
 * nblk = (width/4)*(height/4). With every buffer pinned, the frames pass
 * through a ring of device frame slots of the context, uploads and downloads
 * on two copy streams overlap the encodes, and intra frames after the first
 * are encoded on a second lane concurrently with the inter frames before
 * them (see mptc_encode_stream_device); pageable buffers go frame by frame
 * through the pinned staging. Returns once every output is in host memory. */
mptc_status mptc_encode_stream_host(mptc_ctx *ctx, const uint8_t *frames_host, int32_t n_frames,
                                    const int32_t *is_intra, uint64_t *final_host, uint8_t *motion_host,
                                    uint32_t *unique_host, uint32_t *n_unique_host, void *stream);

/* The same run on DEVICE buffers: frames_dev holds the frames back to back,
 * frame k's outputs go to final_dev + k*nblk, motion_dev + k*2*nblk,
 * unique_dev + k*nblk and n_unique_dev[k]. Intra frames depend on no earlier
 * frame, so the call encodes them on a second context of its own and a second
 * CUDA stream, concurrently with the inter frames before them; each inter
 * frame that follows an intra frame waits for it. The results are those of
 * n_frames successive mptc_encode_frame calls; the run's last final blocks
 * become the context's previous frame (a later call or mptc_encode_frame_host
 * continues the stream). Returns after `stream` has completed the run. */
mptc_status mptc_encode_stream_device(mptc_ctx *ctx, const uint8_t *frames_dev, int32_t n_frames,
                                      const int32_t *is_intra, uint64_t *final_dev, uint8_t *motion_dev,
                                      uint32_t *unique_dev, uint32_t *n_unique_dev, void *stream);

/* Largest frame, in 4x4 blocks, that mptc_encode_frame_noalloc accepts
 * (131072 blocks: 1920x1080 is 129600, 2048x1024 is 131072). */
#define MPTC_NOALLOC_MAX_BLOCKS 131072

/* mptc_encode_frame without any allocation. This entry point has no
 * counterpart in the reference, whose encoder allocates freely.
 *
 * For callers that may not allocate device memory: host applications that
 * reserve the whole device memory budget up front and forbid plugins from
 * calling cudaMalloc, and frame loops with a latency budget that cannot absorb
 * the allocator (cudaFree synchronises the whole device). It takes no context:
 * the caller passes the configuration, the frame size, the input frame and
 * every output buffer; the kernels' scratch (per-block completion words, the
 * stb error of each block, the wavefront order, pending list and sweep
 * estimates and stored statistics of the intra search, the refit weight sums
 * of the previous frame's blocks, work counters and scan tile states) lives in
 * one file-scope device array of about 8.1 MiB inside the library, which every GPU
 * that loads the library holds until the process exits.
 *
 * Frames larger than MPTC_NOALLOC_MAX_BLOCKS blocks are rejected with
 * MPTC_EINVAL. The first call on a device sets that device up (looks up the
 * scratch array's device address and uploads the stb tables); make that first
 * call before any stream capture. The set-up is kept for the life of the
 * process: cudaDeviceReset on a device that has made a call is not supported
 * (the saved scratch address and tables would be stale afterwards). All calls
 * share the one scratch array, so
 * calls that overlap on the GPU (on different streams, or from several host
 * threads) race and corrupt each other's results: serialise them. Outputs and
 * their layouts are those of mptc_encode_frame; stb_dev may be NULL. If a
 * bounded device-side wait expired, *n_unique_dev reads 0xFFFFFFFF and the
 * outputs are invalid. */
mptc_status mptc_encode_frame_noalloc(const mptc_config *cfg, int32_t width, int32_t height,
                                      const uint8_t *rgb_dev, const uint64_t *prev_final_dev,
                                      uint64_t *stb_dev, uint64_t *final_dev, uint8_t *motion_dev,
                                      uint32_t *unique_dev, uint32_t *n_unique_dev, void *stream);

/* Batched encoding of many independent streams (resolutions may differ); the
 * multi-stream form of the reference's per-stream encoder loop
 * (codec/codec.cpp:1383-1509, and ThreadedCompressMultiUnique's one thread per
 * chunk, :1781-1856). One call encodes one frame of every stream. The batch
 * owns each stream's input buffer, its previous/current final blocks and its
 * outputs; the work of all streams is launched as one CUDA graph (captured on
 * first use of each intra/inter pattern) whose per-stream branches run
 * concurrently, so one stream's latency-bound intra search overlaps the other
 * streams' inter searches. */
typedef struct mptc_batch mptc_batch;
mptc_status mptc_batch_create(const mptc_config *cfg, int32_t n_streams, const int32_t *widths,
                              const int32_t *heights, mptc_batch **out_batch);
mptc_status mptc_batch_destroy(mptc_batch *batch);
/* Device buffer (width*height*3 bytes) that receives stream i's next frame. */
mptc_status mptc_batch_input(mptc_batch *batch, int32_t i, uint8_t **rgb_dev);
/* Device outputs of stream i's last encoded frame (valid until the next call). */
mptc_status mptc_batch_output(mptc_batch *batch, int32_t i, const uint64_t **final_dev,
                              const uint8_t **motion_dev, const uint32_t **unique_dev,
                              const uint32_t **n_unique_dev);
/* Copies a frame (host or device memory, width*height*3 bytes) into stream
 * i's input buffer on `stream`. */
mptc_status mptc_batch_upload(mptc_batch *batch, int32_t i, const uint8_t *rgb, void *stream);
/* Copies stream i's last outputs to host memory (synchronises `stream`);
 * unique_host needs room for blocks entries; any pointer may be NULL. */
mptc_status mptc_batch_fetch(mptc_batch *batch, int32_t i, uint64_t *final_host, uint8_t *motion_host,
                             uint32_t *unique_host, uint32_t *n_unique_host, void *stream);
/* Encodes the frame in every stream's input buffer; is_intra: host array, one
 * flag per stream (a stream's first frame must be intra). Asynchronous on
 * `stream`. */
mptc_status mptc_batch_encode(mptc_batch *batch, const int32_t *is_intra, void *stream);
/* A run of n_frames frames of every stream in one call, from device memory:
 * stream i's frames back to back at frames_dev[i] (its width*height*3 bytes
 * each), its intra flags at is_intra[i * n_frames .. +n_frames] (a stream's
 * first frame ever must be intra), its outputs for frame k at
 * final_dev[i] + k*nblk_i, motion_dev[i] + 2*k*nblk_i, unique_dev[i] + k*nblk_i
 * and n_unique_dev[i][k]. The streams continue across calls (the run's last
 * frame becomes each stream's previous frame, for this call or
 * mptc_batch_encode). The results equal n_frames calls of mptc_batch_encode.
 * All the run's intra frames are encoded first, each stream's on an intra lane
 * of its own (they depend on no earlier frame), overlapping the inter frames;
 * the inter frames follow frame by frame, and with a model attached each phase
 * of their learned search is one launch over all streams. Returns after
 * `stream` has completed the run. The multi-stream form of the reference's
 * per-stream encoder loop (codec/codec.cpp:1383-1509) for whole runs. */
mptc_status mptc_batch_encode_run(mptc_batch *batch, int32_t n_frames, const uint8_t *const *frames_dev,
                                  const int32_t *is_intra, uint64_t *const *final_dev, uint8_t *const *motion_dev,
                                  uint32_t *const *unique_dev, uint32_t *const *n_unique_dev, void *stream);
/* Autotuner: times the candidate launch shapes on the current inputs and the
 * given intra/inter pattern (without advancing the streams) and keeps the
 * fastest: warps (blocks) per CTA of the exhaustive inter search (2, 4; with a
 * model attached the current value is kept), the CTA count of each stream's
 * intra dataflow (all, 8, 4, 2 or 1 per SM) and, with a model attached, the
 * dictionary slice per pipeline stage of the window scoring (4 or 8: 64 or
 * 128 words, mptc_ctx_set_learned_shape). Writes the
 * chosen values (any pointer may be NULL; synchronises). The number of
 * proposals K is set with the model (mptc_batch_set_model): it changes the
 * encoder's output, so it is chosen against the exhaustive search's quality,
 * not by time alone. */
mptc_status mptc_batch_autotune(mptc_batch *batch, const int32_t *is_intra, int32_t *inter_warps,
                                int32_t *intra_ctas, int32_t *score_rows, void *stream);

/* ---- Learned candidate proposal (no counterpart in the reference) -------
 * A block MLP f (54 -> 128 -> 128 -> 64 over the 48 pixel bytes, normalised
 * per channel to the block's range, and the stb endpoints) and a candidate MLP
 * g (32 -> 128 -> 64 over an index word's bits) score window candidates by
 * f(block) . g(candidate). With a model attached, the inter search scores
 * each block against the distinct index words of its window on the tcgen05
 * tensor cores (per tile of 16 x 8 blocks, against the words of the tile's
 * window union), tests only the K best-scored words exactly, applies the reference's selection
 * rule to those K positions and accepts under the error threshold; a block
 * none of whose K proposals passes goes to the exhaustive search. Every
 * accepted block meets the reference's acceptance rule and the stream stays a
 * valid MPTC stream, but it is no longer bit-identical to the reference's.
 * BF16 operands, FP32 accumulate; trained on the GPU with AdamW on
 * (block, accepted candidate) pairs. */
typedef struct mptc_model mptc_model;
int64_t mptc_model_num_params(void);
mptc_status mptc_model_create(uint64_t seed, mptc_model **out_model);
mptc_status mptc_model_destroy(mptc_model *model);
/* Flat fp32 parameter vector (layer weights [in x out] then biases, for f1,
 * f2, f3, g1, g2; f1's input padded to 64 rows). */
mptc_status mptc_model_get_params(mptc_model *model, float *host);
mptc_status mptc_model_set_params(mptc_model *model, const float *host);
/* One AdamW step on a batch of B blocks of one frame (block indices
 * blocks_dev) with C candidate index words each (cands_dev, B x C, the
 * accepted candidate first): sampled softmax cross-entropy. With loss_host
 * the call waits for the step and returns MPTC_ETIMEOUT if a bounded
 * device-side wait of this or an earlier unread step expired; with
 * loss_host NULL it returns once the step is queued. */
mptc_status mptc_model_train_step(mptc_model *model, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                                  const uint32_t *blocks_dev, const uint32_t *cands_dev, int32_t B, int32_t C,
                                  float lr, float weight_decay, float *loss_host, void *stream);
/* Loss and gradient (flat, like the parameters) of the same objective, no update. */
mptc_status mptc_model_grads(mptc_model *model, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                             const uint32_t *blocks_dev, const uint32_t *cands_dev, int32_t B, int32_t C,
                             float *grads_host, float *loss_host, void *stream);
/* Embeddings: n_blocks rows of f (blocks_dev NULL = the first n_blocks blocks
 * in raster order) and n_words rows of g (words_dev[i * word_stride]). */
mptc_status mptc_model_embed(mptc_model *model, const uint8_t *rgb_dev, int32_t width, const uint64_t *stb_dev,
                             const uint32_t *blocks_dev, int32_t n_blocks, float *emb_blocks_dev,
                             const uint32_t *words_dev, int32_t word_stride, int32_t n_words,
                             float *emb_words_dev, void *stream);
/* Checkpoint / resume: parameters, AdamW moments and step count. */
mptc_status mptc_model_save(mptc_model *model, const char *path);
mptc_status mptc_model_load(mptc_model *model, const char *path);
/* Attaches (k = 4, 8 or 16 proposals per block) or detaches (model NULL or
 * k <= 0) a model to a context's inter search. Needs search_area <= 8. The
 * context keeps a pointer: the model must outlive the attachment, and a
 * training step between frames changes the proposals of later frames. */
mptc_status mptc_ctx_set_model(mptc_ctx *ctx, const mptc_model *model, int32_t k);
/* The learned proposal's window scoring of one inter frame on its own: the
 * embeddings of the frame's blocks (rgb_dev, stb_dev) and of the previous
 * frame's final blocks, then for every block the K best-scored distinct index
 * words of its inter window (K of the attached model), best first, each at its
 * first window position in the reference's scan order (row-major from
 * (bx-sa, by-sa), codec/dxt_image.cpp:731-735); unused slots 0xFFFF.
 * topk_dev: blocks x 16 u16. Synchronises `stream`. */
mptc_status mptc_learned_proposals(mptc_ctx *ctx, const uint8_t *rgb_dev, const uint64_t *stb_dev,
                                   const uint64_t *prev_final_dev, uint16_t *topk_dev, void *stream);
/* The dictionary slice of a pipeline stage of the scoring kernel, as 4 or 8
 * (the default): each stage scores a tile's 128 blocks against 16 x that many
 * distinct words of the tile's window union (64 or 128 words per tcgen05 MMA);
 * a union with more words takes more stages. Results do not depend on it. */
mptc_status mptc_ctx_set_learned_shape(mptc_ctx *ctx, int32_t rows_per_stage);
/* Attaches (or detaches) a model to every stream of a batch. */
mptc_status mptc_batch_set_model(mptc_batch *batch, const mptc_model *model, int32_t k);
/* Exact err_diff of C candidate index words for each of B blocks of a frame:
 * the refit, validity and error the inter search computes for a window
 * candidate (CompressedBlock::RecalculateEndpoints + Error against the block's
 * stb error, codec/dxt_image.cpp:258-349, as InterBlockSearch uses them,
 * :739-757). blocks_dev: B block indices; cands_dev: B x C index words;
 * err_dev: B x C int32, 2^31-1 where the refit would swap the endpoints (the
 * reference skips such a candidate). The learned proposal's training examples
 * are labelled with it. */
mptc_status mptc_candidate_errors(const uint8_t *rgb_dev, int32_t width, int32_t height, const uint64_t *stb_dev,
                                  const uint32_t *blocks_dev, const uint32_t *cands_dev, int32_t B, int32_t C,
                                  int32_t *err_dev, void *stream);

/* Squared error between a frame and the decoded DXT1 blocks (RGB565 endpoints
 * expanded as a decoder does), into *sse_dev (device u64). */
mptc_status mptc_decoded_sse(const uint8_t *rgb_dev, int32_t width, int32_t height, const uint64_t *blocks_dev,
                             uint64_t *sse_dev, void *stream);

/* Counters of the last frame reencoded on this context (synchronises `stream`). */
mptc_status mptc_last_frame_stats(mptc_ctx *ctx, mptc_frame_stats *out, void *stream);

/* Opt-in CUDA-event timing of every kernel this context launches (off by
 * default). Timing brackets each launch with events on the launching stream. */
typedef struct mptc_kernel_time {
  char name[32];
  int32_t launches;
  double total_ms;
} mptc_kernel_time;
mptc_status mptc_set_kernel_timing(mptc_ctx *ctx, int32_t enable);
/* Sums the recorded launches per kernel (synchronises on the recorded events)
 * and clears the record. Writes up to max_entries entries and their count. */
mptc_status mptc_kernel_times(mptc_ctx *ctx, mptc_kernel_time *out, int32_t max_entries,
                              int32_t *n_entries);

/* Number of kernels the library launched for this context since the last
 * call (or since creation); clears the count. */
mptc_status mptc_kernel_launches(mptc_ctx *ctx, uint64_t *count);

/* Scalar-ALU throughput probe: `threads` x `iters` x 32 dependent-chain-free
 * fp32 add/int32 add pairs. Writes a checksum to *sink_dev (device int32) so
 * nothing is optimised away; the caller times the launch. Returns the op count
 * per launch in *ops (2 ops per pair). */
mptc_status mptc_alu_probe(int32_t blocks, int32_t iters, int32_t *sink_dev, double *ops, void *stream);

/* ---- endpoint images and GPU decode (the stream's endpoint half) ----
 * Frame sizes must be multiples of 256 pixels (64 blocks) in both directions:
 * the reference transforms the endpoint images in 64x64-block tiles and
 * writes out of bounds otherwise (codec/image_processing.h:293-294).
 *
 * Coefficient layout: 6 planes of blocks bytes each,
 *   [Y1 | Co1 | Cg1 | Y2 | Co2 | Cg2]
 * i.e. exactly the byte vectors CompressEndpoint arithmetic-codes
 * (codec/codec.cpp:804-846: the Y plane of endpoint 1, its Co plane followed
 * by its Cg plane, then the same for endpoint 2). */

/* The transform half of CompressEndpoint (codec/codec.cpp:804-838: RGB565 ->
 * YCoCg-667, ImageSplit, RunDXTEndpointPipeline = per-tile 6-level 5/3
 * wavelet, int8 wrap, +128) for the final blocks of one frame. */
mptc_status mptc_endpoint_coefficients(int32_t width, int32_t height, const uint64_t *blocks_dev,
                                       uint8_t *coeff_dev, void *stream);

/* GPU half of the reference's GetFrame (codec/decoder.cpp:256-414): from one
 * frame's entropy-decoded parts (coefficients as above, motion codes, the
 * frame's slice of the group palette) and the previous decoded frame, the
 * frame's physical blocks: ReconstructDXTFrame (decoder.cpp:203-254) and
 * ReconstructEndpoints with the inverse wavelet (decoder.cpp:68-201). */
typedef struct mptc_decoder mptc_decoder;
mptc_status mptc_decoder_create(int32_t width, int32_t height, int32_t search_area,
                                mptc_decoder **out_decoder);
mptc_status mptc_decoder_destroy(mptc_decoder *dec);
/* prev_blocks_dev may be NULL for a frame without inter copies (the first).
 * Asynchronous on `stream`; invalid references are recorded, see below. */
mptc_status mptc_decode_frame(mptc_decoder *dec, const uint8_t *coeff_dev, const uint8_t *motion_dev,
                              const uint32_t *unique_dev, uint32_t n_unique,
                              const uint64_t *prev_blocks_dev, uint64_t *out_blocks_dev, void *stream);
/* Synchronises `stream` and returns MPTC_EINVAL if any frame decoded since the
 * last check held an invalid motion code (a copy from outside the previous
 * frame or from a block not yet decoded) or a unique count that differs from
 * n_unique; *flags (may be NULL) gets bit 0 / bit 1 for those. Clears them. */
mptc_status mptc_decoder_check(mptc_decoder *dec, void *stream, uint32_t *flags);
const char *mptc_decoder_last_error(const mptc_decoder *dec);

/* Human-readable text of the last error on this context (never NULL). */
const char *mptc_last_error(const mptc_ctx *ctx);

/* Library version and the device architecture it was built for (e.g. 1030). */
int32_t mptc_version(void);
int32_t mptc_built_arch(void);

#ifdef __cplusplus
}
#endif
#endif
