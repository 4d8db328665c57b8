// Library-internal interface between the encoder (mptc_api.cu) and the
// learned-proposal model (mptc_model.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/mptc_gb300.h"

namespace mptc_internal {

// Activation scratch of one embedding pass over up to `cap` rows; owned by
// the caller so that concurrent encoders never share it.
struct EmbedWorkspace {
  int cap = 0;
  __nv_bfloat16 *x = nullptr, *h1b = nullptr, *h2b = nullptr;
  float *h1 = nullptr, *h2 = nullptr;
  __nv_bfloat16 *wt = nullptr;  // transposed bf16 weights of the current model
};

mptc_status embed_workspace_alloc(EmbedWorkspace &ws, int rows);
void embed_workspace_free(EmbedWorkspace &ws);

// F[n x 64] = f(features of blocks 0..n-1 of a frame); G[n x 64] = g(words).
// Kernels model_embed_frame launches per call (5 weight transposes, block
// and candidate features, 5 GEMMs).
constexpr int kEmbedLaunches = 12;
mptc_status model_embed_frame(const mptc_model *m, EmbedWorkspace &ws, const uint8_t *rgb, int width,
                              const uint64_t *stb, int n, float *F, const uint32_t *words, int word_stride,
                              float *G, cudaStream_t s);

}  // namespace mptc_internal
