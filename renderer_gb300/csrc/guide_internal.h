// guide_internal.h — the path-guiding network object shared by guide.cu (its
// kernels and entry points) and pathtrace.cu (the guided render).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/gbrt.h"
#include "gbrt_internal.h"
#include "guide_net.cuh"

struct gbrt_guide {
  gbrt_ctx* ctx = nullptr;
  int device = 0;
  float bounds[6] = {0, 0, 0, 1, 1, 1};  // lo.xyz, hi.xyz
  float* d_p = nullptr;                  // FP32 master parameters
  float* d_m = nullptr;                  // Adam first moments
  float* d_v = nullptr;                  // Adam second moments
  float* d_g = nullptr;                  // gradient accumulator
  __nv_bfloat16* d_w = nullptr;          // BF16 copy read by the kernels
  // While a render trains asynchronously (GBRT_GUIDE_ASYNC_TRAINING): the
  // BF16 copy that training reads and Adam writes, on the training stream;
  // d_w then points at the snapshot the current pass infers with. Null
  // otherwise.
  __nv_bfloat16* d_wt = nullptr;
  float* d_loss = nullptr;
  int* d_err = nullptr;
  int step = 0;                          // optimizer steps taken
  bool ready = false;                    // trained or given weights: renders may sample it
  int infer_grid = 0, train_grid = 0;
};

namespace gbrt {
namespace guide {

GuideNet view(const gbrt_guide* g);

// Mixture of every row of a queue: rows are three float4 (point, -), (normal
// facing the viewer, -), (outgoing direction, -); the row count is *count on
// the device (or n_rows when count is null). Writes kMixStride float4 per row.
cudaError_t launch_infer(const gbrt_guide* g, const float4* in, const int* count, int n_rows, float4* mix,
                         cudaStream_t stream);

// Gradient of the loss over n training samples (four float4 each: (point,
// weight), (normal, -), (outgoing, -), (sampled direction, -)) into d_g and
// d_loss (zeroed first); with step, also one Adam step.
cudaError_t train(gbrt_guide* g, const float4* samples, int n, float lr, bool step, cudaStream_t stream);

// The same over step k's window of a sample buffer whose fill count
// (capped at cap) is read on the device: samples [k batch mod n, ... + batch).
cudaError_t train_window(gbrt_guide* g, const float4* samples, const int* avail, int cap, int k, int batch,
                         float lr, bool step, cudaStream_t stream);

}  // namespace guide
}  // namespace gbrt
