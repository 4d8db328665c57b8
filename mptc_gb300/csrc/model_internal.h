// Library-internal interface between the encoder (mptc_api.cu) and the
// learned-proposal model (mptc_model.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mptc_gb300.h"
#include "learned_common.cuh"

namespace mptc_internal {

// One embedding job: the f network over `n` blocks of a frame (rgb, width a
// multiple of 4, 4-byte aligned frame; stb endpoints; blocks NULL = blocks
// 0 .. n-1 in raster order) or the g network over n index words
// (words[i * word_stride]); bf16 output n x 64, row i at out_rows[i] when
// out_rows is set. With n_dev set the job has min(n, *n_dev) rows (a count
// written on the device by an earlier launch). An expired device-side wait
// ORs kDevTimeout into *status.
struct EmbedJob {
  const uint8_t *rgb = nullptr;
  int width = 0;
  const uint64_t *stb = nullptr;
  const uint32_t *blocks = nullptr;
  const uint32_t *words = nullptr;
  int word_stride = 1;
  int n = 0;
  __nv_bfloat16 *out = nullptr;
  uint32_t *status = nullptr;
  const uint32_t *n_dev = nullptr;
  const uint32_t *out_rows = nullptr;
};

// Jobs a single embedding launch takes (the streams of a batch).
constexpr int kMaxEmbedJobs = mptc::kMaxBatch;

// One persistent launch of the f (blocks = true) or g network over up to
// kMaxEmbedJobs jobs with the model's current weights; `next` is a zeroed
// device counter the launch's CTAs draw tiles from.
mptc_status model_embed(const mptc_model *m, bool blocks, const EmbedJob *jobs, int n_jobs, uint32_t *next,
                        cudaStream_t s);

}  // namespace mptc_internal
