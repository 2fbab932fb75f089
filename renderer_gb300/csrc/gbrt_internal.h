// gbrt_internal.h — host-side objects behind the C ABI handles.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "gbrt_scene.h"

struct gbrt_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  // Scratch for the ray-query entry points: one work counter and one error
  // word, reused by every call on this context.
  unsigned long long* d_work = nullptr;
  int* d_err = nullptr;
  // The context's own stream-ordered memory pool: every per-call buffer
  // (wavefront state, films, queries) comes from it, and it keeps freed
  // memory reserved (release threshold unlimited), so that repeated renders
  // with gigabyte-sized wavefronts do not go back to the driver each time.
  cudaMemPool_t pool = nullptr;
  // Streams of gbrt_render_batch and the tuned batch settings.
  std::vector<cudaStream_t> batch_streams;
  int batch_streams_tuned = 4;
  long long batch_paths_tuned = 1ll << 22;
  // Tuned schedule of gbrt_render_batch_fused.
  gbrt_batch_schedule fused_tuned{1ll << 24, 2, 128, 256, 0};
  // Device address of the no-allocation entry point's file-scope scratch
  // array, looked up by the first gbrt_render_device_noalloc call on this
  // context (with its device current).
  unsigned char* noalloc_scratch = nullptr;
  // Host-side fault injection for the tests of the failure paths
  // (gbrt_debug_fault); everything off by default.
  mutable long long fault_alloc_countdown = -1;  // device allocations that still succeed (-1: off)
  unsigned long long fault_nan_every = 0;        // every n-th camera sample's radiance becomes NaN
  bool fault_small_stack = false;                // traversal kernels with a kFaultStack-entry stack
  unsigned long long fault_guide_wait_ns = 0;    // guide kernels skip their products and wait this long
};

struct gbrt_scene {
  gbrt_ctx* ctx = nullptr;
  int device = 0;
  bool watertight = false;  // GBRT_SCENE_WATERTIGHT
  gbrt::DeviceScene view{};
  std::vector<void*> allocations;
  int64_t n_leaves = 0;
  int32_t max_depth = 0;   // binary tree
  int32_t max_depth4 = 0;  // 4-wide tree traversed on the device
  double sah_cost = 0;
  double build_ms = 0;
  int32_t n_prims = 0;  // primitive ids in use
  float bounds[6] = {0, 0, 0, 0, 0, 0};  // box of the bounded primitives: lo.xyz, hi.xyz
};

namespace gbrt {

// Records a failure message on ctx (or the global slot) and returns status.
gbrt_status fail(gbrt_ctx* ctx, gbrt_status st, const std::string& msg);
gbrt_status cuda_fail(gbrt_ctx* ctx, cudaError_t e, const char* what);
void clear_error(gbrt_ctx* ctx);

// The injected allocation failure of gbrt_debug_fault: cudaErrorMemoryAllocation
// for the allocation the countdown reaches, cudaSuccess otherwise. Called
// before every device allocation the library makes for a context.
inline cudaError_t fault_alloc(const gbrt_ctx* ctx) {
  if (!ctx || ctx->fault_alloc_countdown < 0) return cudaSuccess;
  if (ctx->fault_alloc_countdown == 0) {
    ctx->fault_alloc_countdown = -1;
    return cudaErrorMemoryAllocation;
  }
  --ctx->fault_alloc_countdown;
  return cudaSuccess;
}

// Stream-ordered allocation from the context's pool (cudaFreeAsync frees).
inline cudaError_t ctx_alloc(const gbrt_ctx* ctx, void** p, size_t bytes, cudaStream_t stream) {
  if (cudaError_t f = fault_alloc(ctx)) {
    *p = nullptr;
    return f;
  }
  return cudaMallocFromPoolAsync(p, bytes, ctx->pool, stream);
}
template <typename T>
inline cudaError_t ctx_alloc(const gbrt_ctx* ctx, T** p, size_t bytes, cudaStream_t stream) {
  return ctx_alloc(ctx, reinterpret_cast<void**>(p), bytes, stream);
}

#define GBRT_CUDA_TRY(ctx, expr)                              \
  do {                                                        \
    cudaError_t e_ = (expr);                                  \
    if (e_ != cudaSuccess) return gbrt::cuda_fail(ctx, e_, #expr); \
  } while (0)

}  // namespace gbrt
