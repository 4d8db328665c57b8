// Library-internal interface between the encoder (mptc_api.cu) and the
// learned-proposal model (mptc_model.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mptc_gb300.h"

namespace mptc_internal {

// Tensor-core embeddings (bf16, n x 64, row-major) with the model's current
// weights: the f network over the frame's blocks (blocks NULL = blocks 0 ..
// n-1 in raster order; width a multiple of 4, the frame 4-byte aligned) and
// the g network over index words (words[i * word_stride]). An expired
// device-side wait ORs kDevTimeout into *status (NULL: the model's own word).
mptc_status model_embed_blocks(const mptc_model *m, const uint8_t *rgb, int width, const uint64_t *stb,
                               const uint32_t *blocks, int n, __nv_bfloat16 *F, uint32_t *status, cudaStream_t s);
mptc_status model_embed_words(const mptc_model *m, const uint32_t *words, int word_stride, int n, __nv_bfloat16 *G,
                              uint32_t *status, cudaStream_t s);

}  // namespace mptc_internal
