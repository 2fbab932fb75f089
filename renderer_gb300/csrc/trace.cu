// trace.cu — batched ray queries of the C ABI (gbrt_trace_closest/_any and
// their device-pointer variants): the GPU counterpart of calling
// Intersectable::intersect (src/intersectable.h:40) on the scene root for each
// ray, and of the shadow tests inside Light::getIntensity
// (src/arealight.cpp:41-46, src/pointlight.cpp:55-60,
// src/environmentmap.cpp:44-50).
//
// Persistent kernel: a grid of (SMs x resident blocks) in which each warp
// fetches 32 rays at a time from a global counter until the batch is done.
#include <cuda_runtime.h>

#include <algorithm>

#include "gbrt_internal.h"
#include "traverse.cuh"

namespace gbrt {

template <bool ANY, bool WT, int STACK, bool GEN>
__global__ void __launch_bounds__(kTraceBlock)
    k_trace_api(DeviceScene S, const float4* __restrict__ rays, int64_t n, const int32_t* __restrict__ ignore,
                gbrt_hit* __restrict__ hits, uint8_t* __restrict__ occluded, unsigned long long* work, int* err) {
  const int lane = threadIdx.x & 31;
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned long long)n) break;
    int64_t i = int64_t(base) + lane;
    if (i >= n) continue;
    float4 a = __ldg(rays + 2 * i), b = __ldg(rays + 2 * i + 1);
    TRay r = make_tray(a, b);
    float t, u, v;
    int ign = (ANY && ignore) ? ignore[i] : -1;
    int32_t inst = -1;
    int32_t rec = trace_ray<ANY, false, WT, STACK, GEN>(S, r, ign, t, u, v, err, nullptr, &inst);
    if (ANY) {
      occluded[i] = rec != -1 ? 1 : 0;
    } else {
      gbrt_hit h;
      h.t = t; h.u = u; h.v = v;
      if (rec >= 0) {
        h.prim = __ldg(&S.meta[rec]).x;
        if (GEN && __float_as_int(__ldg(S.recs + 3 * int64_t(rec)).w) == kRecCSG) h.u = h.v = 0.f;
        if (GEN && inst >= 0) h.prim = __float_as_int(__ldg(S.inst + 4 * int64_t(inst) + 3).y);
      }
      else if (rec <= -2) h.prim = S.plane_meta[-2 - rec].x;
      else if (S.env_light >= 0 && isinf(r.tmax) && r.tmax > 0.f) {
        h.t = CUDART_INF_F; h.prim = S.env_light; h.u = 0.f; h.v = 0.f;
      } else {
        h.prim = -1; h.t = CUDART_NAN_F;
      }
      hits[i] = h;
    }
  }
}

int trace_grid(gbrt_ctx* ctx, const void* kernel) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTraceBlock, 0);
  return std::max(1, per_sm) * std::max(1, ctx->num_sms);
}

// The ray-query kernel for a scene: any / closest hit, watertight triangles,
// short stack, general leaves (CSG objects, instances).
template <bool G>
static decltype(&k_trace_api<false, false, kStackSize, false>) pick_api(bool any, bool wt, bool shortStack) {
  if (any) {
    if (shortStack) return wt ? k_trace_api<true, true, kShortStack, G> : k_trace_api<true, false, kShortStack, G>;
    return wt ? k_trace_api<true, true, kStackSize, G> : k_trace_api<true, false, kStackSize, G>;
  }
  if (shortStack) return wt ? k_trace_api<false, true, kShortStack, G> : k_trace_api<false, false, kShortStack, G>;
  return wt ? k_trace_api<false, true, kStackSize, G> : k_trace_api<false, false, kStackSize, G>;
}

static gbrt_status launch_api(gbrt_scene* s, bool any, const gbrt_ray* d_rays, const int32_t* d_ignore, int64_t n,
                              gbrt_hit* d_hits, uint8_t* d_occ, cudaStream_t st) {
  gbrt_ctx* ctx = s->ctx;
  GBRT_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_work, 0, sizeof(unsigned long long), st));
  const float4* rays = reinterpret_cast<const float4*>(d_rays);
  // The short stack when the tree is shallow enough for it.
  const bool shortStack = stack_need(s->max_depth4) <= kShortStack;
  const bool gen = s->view.csg_prog != nullptr || s->view.inst != nullptr;
  decltype(&k_trace_api<false, false, kStackSize, false>) k;
  if (gen) k = pick_api<true>(any, s->watertight, shortStack);
  else k = pick_api<false>(any, s->watertight, shortStack);
  const int grid = trace_grid(ctx, (const void*)k);
  k<<<grid, kTraceBlock, 0, st>>>(s->view, rays, n, any ? d_ignore : nullptr, any ? nullptr : d_hits,
                                  any ? d_occ : nullptr, ctx->d_work, ctx->d_err);
  GBRT_CUDA_TRY(ctx, cudaGetLastError());
  return GBRT_OK;
}

static gbrt_status check_err_word(gbrt_ctx* ctx) {
  int err = 0;
  GBRT_CUDA_TRY(ctx, cudaMemcpyAsync(&err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  GBRT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (err & kErrIndex) return fail(ctx, GBRT_ERR_NUMERIC, "trace: index out of range (checked build)");
  if (err) return fail(ctx, GBRT_ERR_NUMERIC, "traversal stack overflow (BVH deeper than supported)");
  return GBRT_OK;
}

}  // namespace gbrt

using namespace gbrt;

extern "C" {

gbrt_status gbrt_trace_closest_device(gbrt_scene* s, const gbrt_ray* d_rays, int64_t n, gbrt_hit* d_hits,
                                      void* stream) {
  if (!s || n < 0 || (n > 0 && (!d_rays || !d_hits)))
    return fail(s ? s->ctx : nullptr, GBRT_ERR_INVALID_ARG, "gbrt_trace_closest_device: bad argument");
  if (n == 0) return GBRT_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->ctx->stream;
  return launch_api(s, false, d_rays, nullptr, n, d_hits, nullptr, st);
}

gbrt_status gbrt_trace_any_device(gbrt_scene* s, const gbrt_ray* d_rays, const int32_t* d_ignore, int64_t n,
                                  uint8_t* d_occ, void* stream) {
  if (!s || n < 0 || (n > 0 && (!d_rays || !d_occ)))
    return fail(s ? s->ctx : nullptr, GBRT_ERR_INVALID_ARG, "gbrt_trace_any_device: bad argument");
  if (n == 0) return GBRT_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : s->ctx->stream;
  return launch_api(s, true, d_rays, d_ignore, n, nullptr, d_occ, st);
}

gbrt_status gbrt_trace_closest(gbrt_scene* s, const gbrt_ray* rays, int64_t n, gbrt_hit* hits) {
  if (!s || n < 0 || (n > 0 && (!rays || !hits)))
    return fail(s ? s->ctx : nullptr, GBRT_ERR_INVALID_ARG, "gbrt_trace_closest: bad argument");
  if (n == 0) return GBRT_OK;
  gbrt_ctx* ctx = s->ctx;
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  gbrt_ray* d_r = nullptr;
  gbrt_hit* d_h = nullptr;
  GBRT_CUDA_TRY(ctx, ctx_alloc(ctx, &d_r, size_t(n) * sizeof(gbrt_ray), ctx->stream));
  cudaError_t e = ctx_alloc(ctx, &d_h, size_t(n) * sizeof(gbrt_hit), ctx->stream);
  if (e != cudaSuccess) { cudaFreeAsync(d_r, ctx->stream); return cuda_fail(ctx, e, "cudaMallocAsync(hits)"); }
  gbrt_status st = GBRT_OK;
  if ((e = cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream)) != cudaSuccess ||
      (e = cudaMemcpyAsync(d_r, rays, size_t(n) * sizeof(gbrt_ray), cudaMemcpyHostToDevice, ctx->stream)) !=
          cudaSuccess) {
    st = cuda_fail(ctx, e, "upload rays");
  }
  if (st == GBRT_OK) st = launch_api(s, false, d_r, nullptr, n, d_h, nullptr, ctx->stream);
  if (st == GBRT_OK &&
      (e = cudaMemcpyAsync(hits, d_h, size_t(n) * sizeof(gbrt_hit), cudaMemcpyDeviceToHost, ctx->stream)) !=
          cudaSuccess)
    st = cuda_fail(ctx, e, "download hits");
  cudaFreeAsync(d_r, ctx->stream);
  cudaFreeAsync(d_h, ctx->stream);
  if (st == GBRT_OK) st = check_err_word(ctx);
  else cudaStreamSynchronize(ctx->stream);
  return st;
}

gbrt_status gbrt_trace_any(gbrt_scene* s, const gbrt_ray* rays, const int32_t* ignore, int64_t n, uint8_t* occ) {
  if (!s || n < 0 || (n > 0 && (!rays || !occ)))
    return fail(s ? s->ctx : nullptr, GBRT_ERR_INVALID_ARG, "gbrt_trace_any: bad argument");
  if (n == 0) return GBRT_OK;
  gbrt_ctx* ctx = s->ctx;
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  gbrt_ray* d_r = nullptr;
  int32_t* d_i = nullptr;
  uint8_t* d_o = nullptr;
  cudaError_t e;
  gbrt_status st = GBRT_OK;
  if ((e = ctx_alloc(ctx, &d_r, size_t(n) * sizeof(gbrt_ray), ctx->stream)) != cudaSuccess ||
      (e = ctx_alloc(ctx, &d_o, size_t(n), ctx->stream)) != cudaSuccess ||
      (ignore && (e = ctx_alloc(ctx, &d_i, size_t(n) * sizeof(int32_t), ctx->stream)) != cudaSuccess))
    st = cuda_fail(ctx, e, "cudaMallocAsync(trace_any)");
  if (st == GBRT_OK &&
      ((e = cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream)) != cudaSuccess ||
       (e = cudaMemcpyAsync(d_r, rays, size_t(n) * sizeof(gbrt_ray), cudaMemcpyHostToDevice, ctx->stream)) !=
           cudaSuccess ||
       (ignore && (e = cudaMemcpyAsync(d_i, ignore, size_t(n) * sizeof(int32_t), cudaMemcpyHostToDevice,
                                       ctx->stream)) != cudaSuccess)))
    st = cuda_fail(ctx, e, "upload rays");
  if (st == GBRT_OK) st = launch_api(s, true, d_r, d_i, n, nullptr, d_o, ctx->stream);
  if (st == GBRT_OK &&
      (e = cudaMemcpyAsync(occ, d_o, size_t(n), cudaMemcpyDeviceToHost, ctx->stream)) != cudaSuccess)
    st = cuda_fail(ctx, e, "download occlusion");
  if (d_r) cudaFreeAsync(d_r, ctx->stream);
  if (d_o) cudaFreeAsync(d_o, ctx->stream);
  if (d_i) cudaFreeAsync(d_i, ctx->stream);
  if (st == GBRT_OK) st = check_err_word(ctx);
  else cudaStreamSynchronize(ctx->stream);
  return st;
}

}  // extern "C"
