// guide.cu — neural path guiding: fused tcgen05 kernels for the network's
// inference and training, Adam, and the gbrt_guide_* entry points.
//
// No counterpart in the renderer (its integrators sample the BSDF only,
// src/unidipathtracingintegrator.cpp:34-46); the network and its loss are
// those of neural path guiding: a small MLP maps (position, normal,
// outgoing direction) to a mixture of von Mises-Fisher lobes, trained online
// by minimising the KL divergence from the incident-radiance distribution,
// estimated by the tracer's own radiance samples:
//   loss = -(1/N) sum_s w_s log q(wi_s),   w_s = target_s / pdf_s.
//
// Both kernels process tiles of 128 rows. Per layer: the threads write the
// layer input (BF16) into shared memory; one thread issues the tcgen05.mma
// chain (M = 128, N = layer width, K in steps of 16) into TMEM and commits it
// to an mbarrier; after the wait every warp reads its 32 TMEM lanes back
// (tcgen05.ld 32x32b), applies the activation and writes the next layer's
// input.
//
// Training keeps, for the backward pass, the encoded input, the hidden
// activations and the deltas once each, row-wise, and reads the same tiles
// in the operand order each product needs:
//   forward  X_l     = ReLU(X_{l-1} W_l^T)    A = X rows, B = W (K-major)
//   dX_l   = delta_{l+1} W_{l+1}              A = delta rows (K-major),
//                                             B = W read MN-major
//   dW_l^T += X_{l-1}^T delta_l               A = X rows, B = delta rows,
//                                             both MN-major (the batch rows
//                                             are the reduction; M = 128)
// The weight-gradient accumulators stay in TMEM across all tiles of a block
// and are added to global memory once at the end.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "guide_internal.h"

namespace gbrt {
namespace guide {

// ------------------------------------------------------------ layouts ----
// Shared by both kernels: the four weight matrices (49,152 B).
constexpr int kSW1 = 0, kSW2 = 26624, kSW3 = 34816, kSW4 = 43008, kSWEnd = 49152;

// Inference: one block per SM of kInferWG warpgroups that share the weights;
// each warpgroup runs its own 128-row tile through the network with its own
// 28,672-byte activation buffer, TMEM columns, mbarrier and named barrier.
// Layer 1 takes the 208 input features in two halves (112 + 96) so that the
// buffer holds one half at a time.
constexpr int kInferWG = 6;
constexpr int kEncA = 14, kEncB = 12;  // groups of 8 features in the two halves
constexpr int kInferBuf = kRows * kEncA * 8 * 2;
constexpr int kInferMisc = kSWEnd + kInferWG * kInferBuf, kInferSmem = kInferMisc + 8 * kInferWG + 16;
constexpr uint32_t kInferCols = 512;  // 64 per warpgroup, rounded up to a power of two

// Training: the weights, the activation rows X1..X3, the region R (the
// encoded input X0 rows, 53,248 bytes, kept for the weight gradient of
// layer 1), the delta rows and the exchange of the loss's lobe terms
// between the two halves of a row. Every tile is stored once: the weight
// gradients read the activation and delta rows MN-major (gemm_mn), the dX
// products the weights MN-major (gemm_k_wmn).
constexpr int kTX1 = 49152, kTX2 = 65536, kTX3 = 81920, kTR = 98304, kTDR = 151552, kTXchg = 167936;
constexpr int kTMisc = kTXchg + 2 * kRows * 16, kTrainSmem = kTMisc + 64;
constexpr uint32_t kTrainCols = 512;
constexpr int kTrainThreads = 2 * kRows;  // two threads per row of a tile
// TMEM columns of the training kernel.
constexpr uint32_t kColScratch = 0, kColW1lo = 64, kColW1hi = 128, kColW2 = 192, kColW3 = 256, kColW4 = 320;

static_assert(kTrainSmem <= 232448, "training tile exceeds the shared memory of a block");
static_assert(kInferSmem <= 232448, "inference block exceeds the shared memory of a block");
static_assert(64 * kInferWG <= int(kInferCols), "TMEM columns of the inference block");
static_assert(kEncA + kEncB == kIn / 8, "encoding halves");

// Layer input ReLU(TMEM columns [0, 64)) of row r into an interleaved
// [128][64] tile at s.
__device__ __forceinline__ void hidden_to_smem(uint32_t lane_taddr, uint32_t s, int r) {
#pragma unroll
  for (int c = 0; c < kHid; c += 32) {
    float v[32];
    tmem_ld32(lane_taddr + c, v);
#pragma unroll
    for (int q = 0; q < 4; ++q)
      st_shared_v4(s + ik_off(r, c + 8 * q, kHid), pack_relu_bf16(v[8 * q], v[8 * q + 1]),
                   pack_relu_bf16(v[8 * q + 2], v[8 * q + 3]), pack_relu_bf16(v[8 * q + 4], v[8 * q + 5]),
                   pack_relu_bf16(v[8 * q + 6], v[8 * q + 7]));
  }
}

// Block-wide hand-over between the threads' shared-memory writes / TMEM
// reads and the next tcgen05 operation.
__device__ __forceinline__ void handoff() {
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// The same within one warpgroup (named barrier id, 128 threads).
__device__ __forceinline__ void wg_sync(int id) { asm volatile("bar.sync %0, 128;" ::"r"(id) : "memory"); }
__device__ __forceinline__ bool wg_sync_or(int id, bool pred) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred q, p;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, %2, 128, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(r)
      : "r"(uint32_t(pred)), "r"(id)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void wg_handoff(int id) {
  fence_async_smem();
  tc_fence_before();
  wg_sync(id);
  tc_fence_after();
}

// Encoding groups [G0, G1) of row r into an interleaved [128][8 (G1 - G0)]
// tile. Unrolled, so that every group's coordinate, band and bin are
// compile-time constants (no division, no indexing of the input by a
// run-time value).
template <int G0, int G1>
__device__ __forceinline__ void write_enc_range(uint32_t s, int r, const EncIn& e) {
  constexpr int K = 8 * (G1 - G0);
#pragma unroll
  for (int g = G0; g < G1; ++g) {
    float f[8];
    enc_group(e, g, f);
    st_shared_v4(s + ik_off(r, 8 * (g - G0), K), pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]),
                 pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
  }
}

// ------------------------------------------------------------ inference ----
__global__ void __launch_bounds__(128 * kInferWG, 1) k_guide_infer(GuideNet net, const float4* __restrict__ in,
                                                                   const int* __restrict__ count, int n_rows,
                                                                   float4* __restrict__ mix, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int wg = threadIdx.x >> 7, t = threadIdx.x & 127, warp = threadIdx.x >> 5;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kInferMisc) + wg;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kInferMisc + 8 * kInferWG);
  const uint32_t sW1 = smem_u32(sm + kSW1), sW2 = smem_u32(sm + kSW2), sW3 = smem_u32(sm + kSW3),
                 sW4 = smem_u32(sm + kSW4), sX = smem_u32(sm + kSWEnd + wg * kInferBuf), bar = smem_u32(mbar);
  const int bid = 1 + wg;  // named barrier of this warpgroup
  load_weights(sm + kSW1, net.w + kOffW1, kHid, kIn, kHid);
  load_weights(sm + kSW2, net.w + kOffW2, kHid, kHid, kHid);
  load_weights(sm + kSW3, net.w + kOffW3, kHid, kHid, kHid);
  load_weights(sm + kSW4, net.w + kOffW4, kOut, kHid, kOutPad);
  if (t == 0) mbar_init(bar, 1);
  if (warp == 0) tmem_alloc(smem_u32(tslot), kInferCols);
  handoff();
  const uint32_t tbase = *tslot;
  const uint32_t tmem = tbase + 64 * wg;
  const uint32_t lane = tmem + (uint32_t((warp & 3) * 32) << 16);
  const int n = count ? *count : n_rows;
  const int ntiles = (n + kRows - 1) / kRows;
  uint32_t phase = 0;
  bool ok = true;
  // One chain of products committed to this warpgroup's barrier, then the
  // wait; false (for the whole warpgroup) when the wait timed out. One thread
  // polls the mbarrier; the other 127 block at the named barrier, which
  // issues nothing while the tensor cores work, so the warpgroups still
  // encoding keep the issue slots.
  auto chain_wait = [&]() -> bool {
    bool fine = true;
    if (t == 0) {
      if (net.issue) mma_commit(bar);
      fine = mbar_wait(bar, phase, net.wait_ns);
    }
    phase ^= 1;
    if (wg_sync_or(bid, !fine)) return false;
    tc_fence_after();
    return true;
  };
  for (int tile = blockIdx.x * kInferWG + wg; tile < ntiles; tile += gridDim.x * kInferWG) {
    const int r = tile * kRows + t;
    EncIn e;
    if (r < n) {
      float4 a = in[3 * size_t(r)], b = in[3 * size_t(r) + 1], c = in[3 * size_t(r) + 2];
      e = make_enc(net, a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z);
    } else {
      e = make_enc(net, net.lo[0], net.lo[1], net.lo[2], 0.f, 0.f, 1.f, 0.f, 0.f, 1.f);
    }
    // Layer 1 in two halves of the input.
    write_enc_range<0, kEncA>(sX, t, e);
    wg_handoff(bid);
    if (t == 0 && net.issue) gemm_k(tmem, sX, 8 * kEncA, sW1, kIn, 8 * kEncA, kHid, false);
    if (!(ok = chain_wait())) break;
    write_enc_range<kEncA, kEncA + kEncB>(sX, t, e);
    wg_handoff(bid);
    if (t == 0 && net.issue) gemm_k(tmem, sX, 8 * kEncB, sW1 + kEncA * 128, kIn, 8 * kEncB, kHid, true);
    if (!(ok = chain_wait())) break;
    hidden_to_smem(lane, sX, t);
    // Layers 2 and 3, then the output layer (N = 48, 40 used).
    for (int layer = 1; layer < 4; ++layer) {
      wg_handoff(bid);
      if (t == 0) {
        if (layer == 1) gemm_k(tmem, sX, kHid, sW2, kHid, kHid, kHid, false);
        else if (layer == 2) gemm_k(tmem, sX, kHid, sW3, kHid, kHid, kHid, false);
        else gemm_k(tmem, sX, kHid, sW4, kHid, kHid, kOutPad, false);
      }
      if (!(ok = chain_wait())) break;
      if (layer < 3) {
        hidden_to_smem(lane, sX, t);
      } else {
        float o[kOutPad];
        tmem_ld32(lane, o);
        tmem_ld16(lane + 32, o + 32);
        if (r < n) {
          Mixture m;
          decode_mixture(o, m);
          store_mixture(mix + kMixStride * size_t(r), m);
        }
      }
    }
    if (!ok) break;
    tc_fence_before();
    wg_sync(bid);
  }
  if (!ok) {
    if (t == 0) atomicExch(err, 1);
    mbar_wait(bar, phase ^ 1, net.wait_ns);  // the chain that timed out, once more (bounded)
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tbase, kInferCols);
  }
}

// ------------------------------------------------------------- training ----
// dLoss/d(raw outputs) of one sample, loss = -w log q(wi), with
//   log q = logsumexp_k lp_k,
//   lp_k = (o_k - logsumexp_j o_j) + log(kappa_k / (2 pi (1 - exp(-2 kappa_k))))
//          + kappa_k (mu_k . wi - 1),
// mu_k the normalised mean outputs and kappa_k = exp(clamp(o_{32+k}, -4, 9));
// with r_k = exp(lp_k - log q) and p_k the softmax weight:
//   d/do_k = -w (r_k - p_k),  d/dmean_k = -w r_k kappa_k / |mean_k| (wi - (mu_k . wi) mu_k),
//   d/do_{32+k} = -w r_k (1 - 2 kappa_k / (exp(2 kappa_k) - 1) + kappa_k (mu_k . wi - 1))
// inside the clamp (0 outside). The two threads of a row share the lobes:
// thread half H takes lobes 4H .. 4H + 3. Phase 1 evaluates the weights'
// normaliser (over all eight) and lp_k of the thread's lobes, and publishes
// those (four floats per row and half); after a block barrier, phase 2 forms
// log q from all eight and the gradients of the thread's lobes and writes
// them, as bfloat16, into its columns of the [128][48] delta row tile.
struct LossHalf {
  float lse_a;
  float lp[4], mx[4], my[4], mz[4], kap[4], cw[4], il[4];
};

template <int H>
__device__ __forceinline__ void loss_phase1(const float* o, float wx, float wy, float wz, LossHalf& L,
                                            float* published) {
  float amax = o[0];
#pragma unroll
  for (int k = 1; k < kLobes; ++k) amax = fmaxf(amax, o[k]);
  float se = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) se += expf(o[k] - amax);
  L.lse_a = amax + logf(se);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = 4 * H + j;
    float x = o[8 + 3 * k], y = o[9 + 3 * k], z = o[10 + 3 * k];
    float l = sqrtf(x * x + y * y + z * z);
    if (l > 1e-12f) {
      L.il[j] = 1.f / l;
      L.mx[j] = x * L.il[j]; L.my[j] = y * L.il[j]; L.mz[j] = z * L.il[j];
    } else {
      L.il[j] = 0.f;
      L.mx[j] = 0.f; L.my[j] = 0.f; L.mz[j] = 1.f;
    }
    L.kap[j] = expf(fminf(fmaxf(o[32 + k], kLogKappaMin), kLogKappaMax));
    L.cw[j] = L.mx[j] * wx + L.my[j] * wy + L.mz[j] * wz;
    L.lp[j] = (o[k] - L.lse_a) + vmf_log_norm(L.kap[j]) + L.kap[j] * (L.cw[j] - 1.f);
  }
  *reinterpret_cast<float4*>(published) = make_float4(L.lp[0], L.lp[1], L.lp[2], L.lp[3]);
}

__device__ __forceinline__ void st_shared_v2(uint32_t saddr, uint32_t a, uint32_t b) {
  asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(saddr), "r"(a), "r"(b) : "memory");
}

template <int H>
__device__ __forceinline__ float loss_phase2(const float* o, float wx, float wy, float wz, float w, const LossHalf& L,
                                             const float* other, uint32_t s_rows, int r) {
  const float4 q = *reinterpret_cast<const float4*>(other);
  float lp[kLobes];
#pragma unroll
  for (int j = 0; j < 4; ++j) lp[4 * H + j] = L.lp[j];
  lp[4 * (1 - H) + 0] = q.x; lp[4 * (1 - H) + 1] = q.y; lp[4 * (1 - H) + 2] = q.z; lp[4 * (1 - H) + 3] = q.w;
  float lmax = -INFINITY;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) lmax = fmaxf(lmax, lp[k]);
  float sq = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) sq += expf(lp[k] - lmax);
  const float lq = lmax + logf(sq);
  float gw[4], gm[12], gk[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = 4 * H + j;
    float rk = expf(L.lp[j] - lq);
    float pk = expf(o[k] - L.lse_a);
    gw[j] = -w * (rk - pk);
    float s = -w * rk * L.kap[j] * L.il[j];
    gm[3 * j] = s * (wx - L.cw[j] * L.mx[j]);
    gm[3 * j + 1] = s * (wy - L.cw[j] * L.my[j]);
    gm[3 * j + 2] = s * (wz - L.cw[j] * L.mz[j]);
    bool inside = o[32 + k] > kLogKappaMin && o[32 + k] < kLogKappaMax;
    float dk = 1.f - 2.f * L.kap[j] / expm1f(2.f * L.kap[j]) + L.kap[j] * (L.cw[j] - 1.f);
    gk[j] = inside ? -w * rk * dk : 0.f;
  }
  // Columns: weights 0-7, means 8-31 (three per lobe), kappas 32-39, 40-47
  // zero; 16-byte chunks of eight columns, the halves' shares aligned to 8 bytes.
  const uint32_t row = s_rows + ik_off(r, 0, kOutPad);
  if (H == 0) {
    st_shared_v2(row, pack_bf16(gw[0], gw[1]), pack_bf16(gw[2], gw[3]));                  // cols 0-3
    st_shared_v4(row + 128, pack_bf16(gm[0], gm[1]), pack_bf16(gm[2], gm[3]), pack_bf16(gm[4], gm[5]),
                 pack_bf16(gm[6], gm[7]));                                                  // cols 8-15
    st_shared_v2(row + 256, pack_bf16(gm[8], gm[9]), pack_bf16(gm[10], gm[11]));          // cols 16-19
    st_shared_v2(row + 512, pack_bf16(gk[0], gk[1]), pack_bf16(gk[2], gk[3]));            // cols 32-35
  } else {
    st_shared_v2(row + 8, pack_bf16(gw[0], gw[1]), pack_bf16(gw[2], gw[3]));              // cols 4-7
    st_shared_v2(row + 256 + 8, pack_bf16(gm[0], gm[1]), pack_bf16(gm[2], gm[3]));        // cols 20-23
    st_shared_v4(row + 384, pack_bf16(gm[4], gm[5]), pack_bf16(gm[6], gm[7]), pack_bf16(gm[8], gm[9]),
                 pack_bf16(gm[10], gm[11]));                                                // cols 24-31
    st_shared_v2(row + 512 + 8, pack_bf16(gk[0], gk[1]), pack_bf16(gk[2], gk[3]));        // cols 36-39
    st_shared_v4(row + 640, 0u, 0u, 0u, 0u);                                                // cols 40-47
  }
  return -w * lq;
}


// Half of a hidden layer's input for row r: ReLU(TMEM columns [c0, c0 + 32))
// into an interleaved [128][64] tile at s.
__device__ __forceinline__ void hidden_half_to_smem(uint32_t lane_taddr, uint32_t s, int r, int c0) {
  float v[32];
  tmem_ld32(lane_taddr + c0, v);
#pragma unroll
  for (int q = 0; q < 4; ++q)
    st_shared_v4(s + ik_off(r, c0 + 8 * q, kHid), pack_relu_bf16(v[8 * q], v[8 * q + 1]),
                 pack_relu_bf16(v[8 * q + 2], v[8 * q + 3]), pack_relu_bf16(v[8 * q + 4], v[8 * q + 5]),
                 pack_relu_bf16(v[8 * q + 6], v[8 * q + 7]));
}

// delta = ReLU'(X) * dX for row r, features [c0, c0 + 32): dX from TMEM
// scratch, X from the row tile; the delta rows go to the tile at s_rows.
__device__ __forceinline__ void backprop_delta_half(uint32_t lane_taddr, const uint8_t* xrow, uint32_t s_rows, int r,
                                                    int c0) {
  float x[32], d[32];
#pragma unroll
  for (int c = 0; c < 32; c += 8) {
    uint4 q = *reinterpret_cast<const uint4*>(xrow + ik_off(r, c0 + c, kHid));
    const __nv_bfloat162* hv = reinterpret_cast<const __nv_bfloat162*>(&q);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float2 f = __bfloat1622float2(hv[i]);
      x[c + 2 * i] = f.x;
      x[c + 2 * i + 1] = f.y;
    }
  }
  tmem_ld32(lane_taddr + c0, d);
#pragma unroll
  for (int k = 0; k < 32; ++k) d[k] = x[k] > 0.f ? d[k] : 0.f;
#pragma unroll
  for (int c = 0; c < 32; c += 8)
    st_shared_v4(s_rows + ik_off(r, c0 + c, kHid), pack_bf16(d[c], d[c + 1]), pack_bf16(d[c + 2], d[c + 3]),
                 pack_bf16(d[c + 4], d[c + 5]), pack_bf16(d[c + 6], d[c + 7]));
}

// Encoding groups [G0, G1) of row r into the full [128][208] row tile (at
// the groups' own feature offsets).
template <int G0, int G1>
__device__ __forceinline__ void write_enc_rows(uint32_t s, int r, const EncIn& e) {
#pragma unroll
  for (int g = G0; g < G1; ++g) {
    float f[8];
    enc_group(e, g, f);
    st_shared_v4(s + ik_off(r, 8 * g, kIn), pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                 pack_bf16(f[6], f[7]));
  }
}
// One optimizer step's gradient over a window of the sample buffer: with
// n_avail = min(*avail, cap) samples written (n_avail = cap when avail is
// null), step k uses samples [start, start + n) with start = k * batch mod
// n_avail and n = min(batch, n_avail - start), read on the device so that
// the host never waits for the sample count.
//
// Two threads per row (threads t and t + 128, halves 0 and 1, in warps w and
// w + 4, which read the same TMEM lanes): each encodes 13 of the 26 feature
// groups, reads back and activates 32 of a hidden layer's 64 columns, and
// back-propagates 32 of its deltas; the output layer's loss and gradient are
// computed by half 0. Eight warps per SM instead of four hide more of the
// per-tile chain's latency. Weight gradients dW^T = X^T delta read the
// activation and delta rows MN-major (gemm_mn): the batch rows are the
// reduction, and the products accumulate in TMEM across the block's tiles.
__global__ void __launch_bounds__(kTrainThreads, 1) k_guide_train(GuideNet net, const float4* __restrict__ base,
                                                                  const int* __restrict__ avail, int cap, int k,
                                                                  int batch, float* __restrict__ grad,
                                                                  float* __restrict__ loss_sum, int* err) {
  extern __shared__ __align__(1024) uint8_t sm[];
  const int t = threadIdx.x, warp = t >> 5, r = t & (kRows - 1), half = t >> 7, c0 = 32 * half;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kTMisc);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(sm + kTMisc + 8);
  const uint32_t bar = smem_u32(mbar);
  const uint32_t sW1 = smem_u32(sm + kSW1), sW2 = smem_u32(sm + kSW2), sW3 = smem_u32(sm + kSW3),
                 sW4 = smem_u32(sm + kSW4), sX1 = smem_u32(sm + kTX1), sX2 = smem_u32(sm + kTX2),
                 sX3 = smem_u32(sm + kTX3), sR = smem_u32(sm + kTR), sDR = smem_u32(sm + kTDR);
  load_weights(sm + kSW1, net.w + kOffW1, kHid, kIn, kHid);
  load_weights(sm + kSW2, net.w + kOffW2, kHid, kHid, kHid);
  load_weights(sm + kSW3, net.w + kOffW3, kHid, kHid, kHid);
  load_weights(sm + kSW4, net.w + kOffW4, kOut, kHid, kOutPad);
  if (t == 0) mbar_init(bar, 1);
  if (warp == 0) tmem_alloc(smem_u32(tslot), kTrainCols);
  handoff();
  const uint32_t tmem = *tslot;
  const uint32_t lane = tmem + (uint32_t((warp & 3) * 32) << 16);
  const int n_avail = avail ? min(*avail, cap) : cap;
  const int start = n_avail > 0 ? int((long long)k * batch % n_avail) : 0;
  const int n = min(batch, n_avail - start);
  const float inv_n = n > 0 ? 1.f / float(n) : 0.f;
  const float4* samples = base + 4 * size_t(start);
  const int ntiles = (n + kRows - 1) / kRows;
  uint32_t phase = 0;
  bool ok = true, first = true;
  float loss = 0.f;

  // One chain of products, then the wait; false when the wait timed out.
  auto sync_chain = [&]() -> bool {
    bool fine = true;
    if (t == 0) {  // one thread polls; the block waits at the barrier
      if (net.issue) mma_commit(bar);
      fine = mbar_wait(bar, phase, net.wait_ns);
    }
    phase ^= 1;
    if (__syncthreads_or(!fine)) return false;
    tc_fence_after();
    return true;
  };

  for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
    const int row = tile * kRows + r;
    float4 s0 = make_float4(net.lo[0], net.lo[1], net.lo[2], 0.f), s1 = make_float4(0.f, 0.f, 1.f, 0.f),
           s2 = make_float4(0.f, 0.f, 1.f, 0.f), s3 = make_float4(0.f, 0.f, 1.f, 0.f);
    if (row < n) {
      s0 = samples[4 * size_t(row)];
      s1 = samples[4 * size_t(row) + 1];
      s2 = samples[4 * size_t(row) + 2];
      s3 = samples[4 * size_t(row) + 3];
    }
    const float w = row < n ? s0.w * inv_n : 0.f;
    const EncIn e = make_enc(net, s0.x, s0.y, s0.z, s1.x, s1.y, s1.z, s2.x, s2.y, s2.z);
    if (half == 0) write_enc_rows<0, kIn / 16>(sR, r, e);
    else write_enc_rows<kIn / 16, kIn / 8>(sR, r, e);
    // ---- forward
    handoff();
    if (t == 0 && net.issue) gemm_k(tmem + kColScratch, sR, kIn, sW1, kIn, kIn, kHid, false);
    if (!(ok = sync_chain())) break;
    hidden_half_to_smem(lane + kColScratch, sX1, r, c0);
    handoff();
    if (t == 0 && net.issue) gemm_k(tmem + kColScratch, sX1, kHid, sW2, kHid, kHid, kHid, false);
    if (!(ok = sync_chain())) break;
    hidden_half_to_smem(lane + kColScratch, sX2, r, c0);
    handoff();
    if (t == 0 && net.issue) gemm_k(tmem + kColScratch, sX2, kHid, sW3, kHid, kHid, kHid, false);
    if (!(ok = sync_chain())) break;
    hidden_half_to_smem(lane + kColScratch, sX3, r, c0);
    handoff();
    if (t == 0 && net.issue) gemm_k(tmem + kColScratch, sX3, kHid, sW4, kHid, kHid, kOutPad, false);
    if (!(ok = sync_chain())) break;
    {
      // the loss and the output layer's delta, lobes split between the halves
      float o[kOutPad];
      tmem_ld32(lane + kColScratch, o);
      tmem_ld16(lane + kColScratch + 32, o + 32);
      float* xchg = reinterpret_cast<float*>(sm + kTXchg);
      float* mine = xchg + 4 * (half * kRows + r);
      const float* other = xchg + 4 * ((1 - half) * kRows + r);
      LossHalf L;
      if (half == 0) loss_phase1<0>(o, s3.x, s3.y, s3.z, L, mine);
      else loss_phase1<1>(o, s3.x, s3.y, s3.z, L, mine);
      __syncthreads();
      float ls;
      if (half == 0) ls = loss_phase2<0>(o, s3.x, s3.y, s3.z, w, L, other, sDR, r);
      else ls = loss_phase2<1>(o, s3.x, s3.y, s3.z, w, L, other, sDR, r);
      if (half == 0 && row < n) loss += ls;
    }
    // ---- backward: output layer
    handoff();
    if (t == 0 && net.issue) {
      gemm_mn(tmem + kColW4, sX3, kHid, sDR, kOutPad, kRows, kOutPad, !first);
      gemm_k_wmn(tmem + kColScratch, sDR, kOutPad, sW4, kHid, kOutPad, kHid, false);
    }
    if (!(ok = sync_chain())) break;
    backprop_delta_half(lane + kColScratch, sm + kTX3, sDR, r, c0);
    // ---- layer 3
    handoff();
    if (t == 0 && net.issue) {
      gemm_mn(tmem + kColW3, sX2, kHid, sDR, kHid, kRows, kHid, !first);
      gemm_k_wmn(tmem + kColScratch, sDR, kHid, sW3, kHid, kHid, kHid, false);
    }
    if (!(ok = sync_chain())) break;
    backprop_delta_half(lane + kColScratch, sm + kTX2, sDR, r, c0);
    // ---- layer 2
    handoff();
    if (t == 0 && net.issue) {
      gemm_mn(tmem + kColW2, sX1, kHid, sDR, kHid, kRows, kHid, !first);
      gemm_k_wmn(tmem + kColScratch, sDR, kHid, sW2, kHid, kHid, kHid, false);
    }
    if (!(ok = sync_chain())) break;
    backprop_delta_half(lane + kColScratch, sm + kTX1, sDR, r, c0);
    // ---- layer 1: input features 0..127 and 128..207 (M = 128 each)
    handoff();
    if (t == 0 && net.issue) {
      gemm_mn(tmem + kColW1lo, sR, kIn, sDR, kHid, kRows, kHid, !first);
      gemm_mn(tmem + kColW1hi, sR + 16 * 128, kIn, sDR, kHid, kRows, kHid, !first);
    }
    if (!(ok = sync_chain())) break;
    first = false;
    tc_fence_before();
    __syncthreads();
  }
  if (ok && !first) {
    // Weight gradients out of TMEM: lane = input feature, column = output;
    // half h takes columns [32 h, 32 h + 32) of each block (W4: half 0 the
    // first 32 of its 48, half 1 the rest).
    float v[16];
    for (int c = c0; c < c0 + 32; c += 16) {
      tmem_ld16(lane + kColW1lo + c, v);
      for (int i = 0; i < 16; ++i) atomicAdd(&grad[kOffW1 + (c + i) * kIn + r], v[i]);
      tmem_ld16(lane + kColW1hi + c, v);
      if (kRows + r < kIn)
        for (int i = 0; i < 16; ++i) atomicAdd(&grad[kOffW1 + (c + i) * kIn + kRows + r], v[i]);
      tmem_ld16(lane + kColW2 + c, v);
      if (r < kHid)
        for (int i = 0; i < 16; ++i) atomicAdd(&grad[kOffW2 + (c + i) * kHid + r], v[i]);
      tmem_ld16(lane + kColW3 + c, v);
      if (r < kHid)
        for (int i = 0; i < 16; ++i) atomicAdd(&grad[kOffW3 + (c + i) * kHid + r], v[i]);
    }
    for (int c = half ? 32 : 0; c < (half ? kOutPad : 32); c += 16) {
      tmem_ld16(lane + kColW4 + c, v);
      if (r < kHid)
        for (int i = 0; i < 16; ++i)
          if (c + i < kOut) atomicAdd(&grad[kOffW4 + (c + i) * kHid + r], v[i]);
    }
    if (half == 0) atomicAdd(loss_sum, loss);
  }
  if (!ok) {
    if (t == 0) atomicExch(err, 1);
    mbar_wait(bar, phase ^ 1, net.wait_ns);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, kTrainCols);
  }
}

// ----------------------------------------------------------------- Adam ----
__global__ void k_guide_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                             const float* __restrict__ g, __nv_bfloat16* __restrict__ w, int n, float lr, float b1,
                             float b2, float eps, float bc1, float bc2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  if (!isfinite(gi)) gi = 0.f;
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  p[i] = pi;
  w[i] = __float2bfloat16_rn(pi);
}

__global__ void k_to_bf16(const float* __restrict__ p, __nv_bfloat16* __restrict__ w, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) w[i] = __float2bfloat16_rn(p[i]);
}

// ------------------------------------------------------------- host side ----
GuideNet view(const gbrt_guide* g) {
  GuideNet v;
  v.w = g->d_w;
  // An injected fault (gbrt_debug_fault) issues nothing and waits briefly.
  v.wait_ns = g->ctx->fault_guide_wait_ns ? g->ctx->fault_guide_wait_ns : 1000000000ull;
  v.issue = g->ctx->fault_guide_wait_ns ? 0 : 1;
  for (int k = 0; k < 3; ++k) {
    v.lo[k] = g->bounds[k];
    float ext = g->bounds[3 + k] - g->bounds[k];
    v.inv_ext[k] = ext > 0.f ? 1.f / ext : 0.f;
  }
  return v;
}

cudaError_t launch_infer(const gbrt_guide* g, const float4* in, const int* count, int n_rows, float4* mix,
                         cudaStream_t stream) {
  k_guide_infer<<<g->infer_grid, kRows * kInferWG, kInferSmem, stream>>>(view(g), in, count, n_rows, mix,
                                                                         g->d_err);
  return cudaGetLastError();
}

cudaError_t train_window(gbrt_guide* g, const float4* samples, const int* avail, int cap, int k, int batch,
                         float lr, bool step, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(g->d_g, 0, kParams * sizeof(float), stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->d_loss, 0, sizeof(float), stream);
  if (e != cudaSuccess) return e;
  if (cap > 0 && batch > 0) {
    int tiles = (std::min(batch, cap) + kRows - 1) / kRows;
    int grid = std::min(g->train_grid, tiles);
    // Training reads (and Adam writes) the training copy of the BF16
    // weights when a render trains asynchronously, else the only copy.
    GuideNet tv = view(g);
    if (g->d_wt) tv.w = g->d_wt;
    k_guide_train<<<grid, kTrainThreads, kTrainSmem, stream>>>(tv, samples, avail, cap, k, batch, g->d_g, g->d_loss,
                                                       g->d_err);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (step) {
    g->step += 1;
    g->ready = true;
    const float b1 = 0.9f, b2 = 0.999f;
    float bc1 = float(1.0 - std::pow(double(b1), g->step)), bc2 = float(1.0 - std::pow(double(b2), g->step));
    k_guide_adam<<<(kParams + 255) / 256, 256, 0, stream>>>(g->d_p, g->d_m, g->d_v, g->d_g,
                                                            g->d_wt ? g->d_wt : g->d_w, kParams, lr, b1, b2, 1e-8f,
                                                            bc1, bc2);
    e = cudaGetLastError();
  }
  return e;
}

cudaError_t train(gbrt_guide* g, const float4* samples, int n, float lr, bool step, cudaStream_t stream) {
  return train_window(g, samples, nullptr, n, 0, n, lr, step, stream);
}

}  // namespace guide
}  // namespace gbrt

using namespace gbrt;
using namespace gbrt::guide;

namespace {

// Seeded initial parameters: uniform in +-sqrt(6 / fan_in) (He et al. for
// the ReLU layers), the output layer scaled by 0.1 so that the initial
// mixture is close to eight broad lobes of equal weight.
void init_params(std::vector<float>& p, unsigned long long seed) {
  p.assign(kParams, 0.f);
  unsigned long long s = seed ^ 0x5DEECE66Dull;
  auto next = [&]() {
    s += 0x9E3779B97F4A7C15ull;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return double(z >> 11) * (1.0 / 9007199254740992.0);
  };
  struct M { int off, n, fan; double scale; } ms[4] = {
      {kOffW1, kW1, kIn, 1.0}, {kOffW2, kW2, kHid, 1.0}, {kOffW3, kW3, kHid, 1.0}, {kOffW4, kW4, kHid, 0.1}};
  for (auto& m : ms) {
    double a = std::sqrt(6.0 / m.fan) * m.scale;
    for (int i = 0; i < m.n; ++i) p[m.off + i] = float((2.0 * next() - 1.0) * a);
  }
}

gbrt_status check_guide(gbrt_guide* g) {
  if (!g) return fail(nullptr, GBRT_ERR_INVALID_ARG, "guide: NULL handle");
  cudaError_t e = cudaSetDevice(g->device);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "cudaSetDevice");
  return GBRT_OK;
}

gbrt_status read_err(gbrt_guide* g, cudaStream_t stream) {
  int err = 0;
  cudaError_t e = cudaMemcpyAsync(&err, g->d_err, sizeof err, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "guide");
  if (err) {
    cudaMemsetAsync(g->d_err, 0, sizeof(int), stream);
    return fail(g->ctx, GBRT_ERR_TIMEOUT, "guide: a tensor-core wait timed out");
  }
  return GBRT_OK;
}

}  // namespace

extern "C" {

gbrt_status gbrt_guide_create(gbrt_ctx* ctx, const float bounds[6], uint64_t seed, gbrt_guide** out) {
  if (!ctx || !bounds || !out) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_create: NULL argument");
  *out = nullptr;
  for (int k = 0; k < 3; ++k)
    if (!(bounds[3 + k] >= bounds[k]) || !std::isfinite(bounds[k]) || !std::isfinite(bounds[3 + k]))
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_create: bounds must be finite with hi >= lo");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  auto* g = new gbrt_guide();
  g->ctx = ctx;
  g->device = ctx->device;
  std::memcpy(g->bounds, bounds, sizeof g->bounds);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(cudaMalloc(&g->d_p, kParams * sizeof(float)));
  A(cudaMalloc(&g->d_m, kParams * sizeof(float)));
  A(cudaMalloc(&g->d_v, kParams * sizeof(float)));
  A(cudaMalloc(&g->d_g, kParams * sizeof(float)));
  A(cudaMalloc(&g->d_w, kParams * sizeof(__nv_bfloat16)));
  A(cudaMalloc(&g->d_loss, sizeof(float)));
  A(cudaMalloc(&g->d_err, sizeof(int)));
  A(cudaFuncSetAttribute(k_guide_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, kInferSmem));
  A(cudaFuncSetAttribute(k_guide_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem));
  g->infer_grid = ctx->num_sms;
  g->train_grid = ctx->num_sms;
  std::vector<float> p;
  init_params(p, seed);
  if (e == cudaSuccess) {
    A(cudaMemcpy(g->d_p, p.data(), kParams * sizeof(float), cudaMemcpyHostToDevice));
    A(cudaMemset(g->d_m, 0, kParams * sizeof(float)));
    A(cudaMemset(g->d_v, 0, kParams * sizeof(float)));
    A(cudaMemset(g->d_err, 0, sizeof(int)));
    k_to_bf16<<<(kParams + 255) / 256, 256>>>(g->d_p, g->d_w, kParams);
    A(cudaGetLastError());
    A(cudaDeviceSynchronize());
  }
  if (e != cudaSuccess) {
    gbrt_guide_destroy(g);
    return cuda_fail(ctx, e, "gbrt_guide_create");
  }
  *out = g;
  return GBRT_OK;
}

gbrt_status gbrt_guide_destroy(gbrt_guide* g) {
  if (!g) return GBRT_OK;
  cudaSetDevice(g->device);
  cudaDeviceSynchronize();
  for (void* p : {(void*)g->d_p, (void*)g->d_m, (void*)g->d_v, (void*)g->d_g, (void*)g->d_w, (void*)g->d_loss,
                  (void*)g->d_err})
    if (p) cudaFree(p);
  delete g;
  return GBRT_OK;
}

gbrt_status gbrt_guide_get_weights(gbrt_guide* g, float* out, size_t n) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!out || n < size_t(kParams)) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_get_weights: buffer");
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(out, g->d_p, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return GBRT_OK;
}

gbrt_status gbrt_guide_set_weights(gbrt_guide* g, const float* w, size_t n) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!w || n != size_t(kParams)) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_set_weights: size");
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(w[i])) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_set_weights: non-finite");
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(g->d_p, w, kParams * sizeof(float), cudaMemcpyHostToDevice));
  GBRT_CUDA_TRY(g->ctx, cudaMemset(g->d_m, 0, kParams * sizeof(float)));
  GBRT_CUDA_TRY(g->ctx, cudaMemset(g->d_v, 0, kParams * sizeof(float)));
  k_to_bf16<<<(kParams + 255) / 256, 256>>>(g->d_p, g->d_w, kParams);
  GBRT_CUDA_TRY(g->ctx, cudaGetLastError());
  GBRT_CUDA_TRY(g->ctx, cudaDeviceSynchronize());
  g->step = 0;
  g->ready = true;
  return GBRT_OK;
}

gbrt_status gbrt_guide_get_state(gbrt_guide* g, float* params, float* adam_m, float* adam_v, int64_t* step) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!params || !adam_m || !adam_v || !step) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_get_state: NULL");
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(params, g->d_p, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(adam_m, g->d_m, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(adam_v, g->d_v, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  *step = int64_t(g->step);
  return GBRT_OK;
}

gbrt_status gbrt_guide_set_state(gbrt_guide* g, const float* params, const float* adam_m, const float* adam_v,
                                 int64_t step) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!params || !adam_m || !adam_v || step < 0 || step > 0x7fffffff)
    return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_set_state: bad argument");
  for (int i = 0; i < kParams; ++i)
    if (!std::isfinite(params[i]) || !std::isfinite(adam_m[i]) || !(adam_v[i] >= 0.f) || !std::isfinite(adam_v[i]))
      return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_set_state: non-finite or negative value");
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(g->d_p, params, kParams * sizeof(float), cudaMemcpyHostToDevice));
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(g->d_m, adam_m, kParams * sizeof(float), cudaMemcpyHostToDevice));
  GBRT_CUDA_TRY(g->ctx, cudaMemcpy(g->d_v, adam_v, kParams * sizeof(float), cudaMemcpyHostToDevice));
  k_to_bf16<<<(kParams + 255) / 256, 256>>>(g->d_p, g->d_w, kParams);
  GBRT_CUDA_TRY(g->ctx, cudaGetLastError());
  GBRT_CUDA_TRY(g->ctx, cudaDeviceSynchronize());
  g->step = int(step);
  g->ready = true;
  return GBRT_OK;
}

gbrt_status gbrt_guide_eval(gbrt_guide* g, const float* inputs, size_t n, float* out) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!inputs || !out) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_eval: NULL argument");
  if (n == 0) return GBRT_OK;
  if (n > (1u << 26)) return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_eval: too many rows");
  cudaStream_t s = g->ctx->stream;
  std::vector<float4> h(3 * n);
  for (size_t i = 0; i < n; ++i) {
    const float* r = inputs + 9 * i;
    h[3 * i] = make_float4(r[0], r[1], r[2], 0.f);
    h[3 * i + 1] = make_float4(r[3], r[4], r[5], 0.f);
    h[3 * i + 2] = make_float4(r[6], r[7], r[8], 0.f);
  }
  float4 *d_in = nullptr, *d_mix = nullptr;
  cudaError_t e = ctx_alloc(g->ctx, &d_in, h.size() * sizeof(float4), s);
  if (e == cudaSuccess) e = ctx_alloc(g->ctx, &d_mix, kMixStride * n * sizeof(float4), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_in, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = launch_infer(g, d_in, nullptr, int(n), d_mix, s);
  if (e == cudaSuccess)
    e = cudaMemcpy2DAsync(out, 10 * sizeof(float4), d_mix, kMixStride * sizeof(float4), 10 * sizeof(float4), n,
                          cudaMemcpyDeviceToHost, s);
  if (d_in) cudaFreeAsync(d_in, s);
  if (d_mix) cudaFreeAsync(d_mix, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "gbrt_guide_eval");
  return read_err(g, s);
}

static gbrt_status upload_samples(gbrt_guide* g, const float* samples, size_t n, float4** d_out) {
  std::vector<float4> h(4 * n);
  for (size_t i = 0; i < n; ++i) {
    const float* r = samples + 13 * i;
    h[4 * i] = make_float4(r[0], r[1], r[2], r[12]);
    h[4 * i + 1] = make_float4(r[3], r[4], r[5], 0.f);
    h[4 * i + 2] = make_float4(r[6], r[7], r[8], 0.f);
    h[4 * i + 3] = make_float4(r[9], r[10], r[11], 0.f);
  }
  cudaStream_t s = g->ctx->stream;
  cudaError_t e = ctx_alloc(g->ctx, d_out, h.size() * sizeof(float4), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(*d_out, h.data(), h.size() * sizeof(float4), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "guide samples");
  return GBRT_OK;
}

gbrt_status gbrt_guide_gradient(gbrt_guide* g, const float* samples, size_t n, float* grad, float* loss) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!samples || !grad || n == 0 || n > (1u << 26))
    return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_gradient: bad argument");
  float4* d = nullptr;
  if ((st = upload_samples(g, samples, n, &d)) != GBRT_OK) return st;
  cudaStream_t s = g->ctx->stream;
  cudaError_t e = train(g, d, int(n), 0.f, false, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad, g->d_g, kParams * sizeof(float), cudaMemcpyDeviceToHost, s);
  float l = 0.f;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&l, g->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "gbrt_guide_gradient");
  if (loss) *loss = l;
  return read_err(g, s);
}

gbrt_status gbrt_guide_train_step(gbrt_guide* g, const float* samples, size_t n, float learning_rate, float* loss) {
  gbrt_status st = check_guide(g);
  if (st != GBRT_OK) return st;
  if (!samples || n == 0 || n > (1u << 26) || !(learning_rate > 0.f))
    return fail(g->ctx, GBRT_ERR_INVALID_ARG, "gbrt_guide_train_step: bad argument");
  float4* d = nullptr;
  if ((st = upload_samples(g, samples, n, &d)) != GBRT_OK) return st;
  cudaStream_t s = g->ctx->stream;
  cudaError_t e = train(g, d, int(n), learning_rate, true, s);
  float l = 0.f;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&l, g->d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(d, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(g->ctx, e, "gbrt_guide_train_step");
  if (loss) *loss = l;
  return read_err(g, s);
}

}  // extern "C"
