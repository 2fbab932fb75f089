// bvh_gpu.h — the GPU builder of the 4-wide BVH (bvh_gpu.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "bvh_build.h"

namespace gbrt {

// Levels of 4-wide nodes the traversal stack supports (3 depth + 1 <= 190).
constexpr int kGpuBuildMaxDepth4 = 63;

struct GpuBuild {
  float4* nodes;     // n_nodes Node4 (eight float4 each), cudaMalloc'ed, root at 0
  unsigned* order;   // sorted position -> input primitive, cudaMalloc'ed
  int64_t n_nodes;
  int depth4;        // levels of 4-wide nodes
  int64_t leaves;
  bool too_deep;     // the tree would not fit the traversal stack: build on the host
};

// Builds over boxes (all finite). On success with too_deep false the caller
// owns nodes and order.
cudaError_t gpu_build_bvh4(const std::vector<Box>& boxes, int max_leaf, cudaStream_t stream, GpuBuild* out);

// Records (three float4) and meta (int4) from input order into leaf order.
cudaError_t gpu_gather_records(const float4* rin, const int4* min_, const unsigned* order, int64_t n, float4* rout,
                               int4* mout, cudaStream_t stream);

}  // namespace gbrt
