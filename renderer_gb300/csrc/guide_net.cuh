// guide_net.cuh — the path-guiding network: input encoding, von Mises-Fisher
// mixture, and the tcgen05 building blocks of its fused kernels.
//
// Network (no counterpart in the renderer, which samples BSDFs only):
//   input  208 = position (scene box -> [0,1]^3) and normal ((n+1)/2), each
//                coordinate as sin/cos(2^j pi v), j = 0..11 (2 x 72), and the
//                outgoing direction as a one-blob encoding of theta / pi and
//                phi / 2pi with 32 Gaussian bins each (64)
//   layers 208 -> 64 -> 64 -> 64 -> 40, ReLU between, no biases, BF16
//          operands with FP32 accumulation on the tensor cores (tcgen05)
//   output 8 lobes: softmax weights (8), mean directions (8 x 3, normalised),
//          concentrations kappa = exp(clamp(b, -4, 9)) (8)
// Parameters, FP32 master copy and BF16 copy alike, are four row-major
// matrices [out][in] one after the other: W1 64x208, W2 64x64, W3 64x64,
// W4 40x64 (24,064 values).
//
// Shared-memory operand layout (tcgen05 "no swizzle"): an R x K BF16 tile is
// stored as 8 x 8 core matrices of 128 contiguous bytes; the K/8 core
// matrices of one 8-row group are adjacent (leading byte offset 128) and row
// groups follow each other (stride byte offset 16 K). Read K-major, the rows
// are M or N; read MN-major (gemm_mn, gemm_k_wmn), the same tile's rows are
// the reduction and its K columns are M or N.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace gbrt {
namespace guide {

constexpr int kIn = 208, kHid = 64, kOut = 40, kOutPad = 48, kLobes = 8, kRows = 128;
constexpr int kBands = 12, kBlob = 32;
constexpr int kW1 = kHid * kIn, kW2 = kHid * kHid, kW3 = kHid * kHid, kW4 = kOut * kHid;
constexpr int kOffW1 = 0, kOffW2 = kW1, kOffW3 = kW1 + kW2, kOffW4 = kW1 + kW2 + kW3;
constexpr int kParams = kW1 + kW2 + kW3 + kW4;
constexpr float kLogKappaMin = -4.f, kLogKappaMax = 9.f;
// A stored mixture: (pi0..3), (pi4..7), (mean, kappa) per lobe, then the
// normalised lobe weights c_k = pi_k kappa_k / (2 pi (1 - exp(-2 kappa_k)))
// in two float4, so that q(w) = sum_k c_k exp(kappa_k (mean_k . w - 1)).
constexpr int kMixStride = 12;
constexpr float kPi = 3.14159265358979323846f;

// Device view of a network.
struct GuideNet {
  const __nv_bfloat16* w;  // kParams BF16 values, layout above
  float lo[3], inv_ext[3];  // position normalisation: (p - lo) * inv_ext
  unsigned long long wait_ns;  // limit of every wait for the tensor cores (1 s)
  int issue;                   // 0 only under an injected fault: no products are issued or committed
};

// ------------------------------------------------------------ layout ----
__host__ __device__ constexpr uint32_t ik_off(int r, int k, int K) {
  return uint32_t((r >> 3) * (K * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (all >> 4), descriptor version 1 (bits 46-47), no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return uint64_t((saddr >> 4) & 0x3FFFu) | (uint64_t((lbo >> 4) & 0x3FFFu) << 16) |
         (uint64_t((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits
// 4-5 = 1), BF16 A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit
// 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// ----------------------------------------------------------- tcgen05 ----
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A * B^T, one instruction (M x N x 16).
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint32_t mbar_saddr) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar_saddr)
               : "memory");
}

// A (128 x K at sa) times B^T (N x K at sb), K a multiple of 16, into TMEM
// columns starting at d_tmem. Issued by one thread.
__device__ __forceinline__ void gemm_k(uint32_t d_tmem, uint32_t sa, int Ka, uint32_t sb, int Kb, int K, int N,
                                       bool accumulate) {
  const uint32_t idesc = idesc_bf16(128, N);
  for (int kk = 0; kk < K / 16; ++kk) {
    uint64_t da = smem_desc(sa + kk * 256, 128, uint32_t(Ka) * 16);
    uint64_t db = smem_desc(sb + kk * 256, 128, uint32_t(Kb) * 16);
    mma_bf16(d_tmem, da, db, idesc, (accumulate || kk > 0) ? 1u : 0u);
  }
}

// A^T B for two interleaved row tiles whose rows are the reduction (the
// batch): A at sa holds K rows of Ma features, B at sb K rows of Nb features
// (both laid out by ik_off). Both operands are read MN-major (instruction
// descriptor bits 15 and 16): a core matrix is 8 rows x 8 consecutive
// features, the next 8 features 128 bytes on (stride byte offset), the next
// 8 rows one row group of the tile on (leading byte offset, features x 16).
// D[m][n] = sum_k A[k][m] B[k][n] with M = 128: rows m >= Ma read the
// following row group and are not used. Issued by one thread.
__device__ __forceinline__ void gemm_mn(uint32_t d_tmem, uint32_t sa, int Ma, uint32_t sb, int Nb, int K, int N,
                                        bool accumulate) {
  const uint32_t idesc = idesc_bf16(128, N) | (1u << 15) | (1u << 16);
  for (int kk = 0; kk < K / 16; ++kk) {
    uint64_t da = smem_desc(sa + kk * 2 * uint32_t(Ma) * 16, uint32_t(Ma) * 16, 128);
    uint64_t db = smem_desc(sb + kk * 2 * uint32_t(Nb) * 16, uint32_t(Nb) * 16, 128);
    mma_bf16(d_tmem, da, db, idesc, (accumulate || kk > 0) ? 1u : 0u);
  }
}

// A (128 x K at sa, K-major as in gemm_k) times B, where B is a weight row
// tile W [K rows][Nw features] read MN-major: D[m][n] = sum_k A[m][k] W[k][n]
// (the product with W itself rather than its transpose), N = Nw columns.
__device__ __forceinline__ void gemm_k_wmn(uint32_t d_tmem, uint32_t sa, int Ka, uint32_t sw, int Nw, int K, int N,
                                           bool accumulate) {
  const uint32_t idesc = idesc_bf16(128, N) | (1u << 16);
  for (int kk = 0; kk < K / 16; ++kk) {
    uint64_t da = smem_desc(sa + kk * 256, 128, uint32_t(Ka) * 16);
    uint64_t db = smem_desc(sw + kk * 2 * uint32_t(Nw) * 16, uint32_t(Nw) * 16, 128);
    mma_bf16(d_tmem, da, db, idesc, (accumulate || kk > 0) ? 1u : 0u);
  }
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for the phase of an mbarrier to complete, for at most limit_ns.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// 16 consecutive FP32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive FP32 columns as two loads and one wait: the wait names the
// loaded registers, so that no use of them can be scheduled before it.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];"
      : "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr + 16));
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                 "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                 "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}
// ReLU and the bfloat16 rounding of two values in one conversion (a in the
// low half, as pack_bf16).
__device__ __forceinline__ uint32_t pack_relu_bf16(float a, float b) {
  uint32_t d;
  asm("cvt.rn.relu.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
  return d;
}
__device__ __forceinline__ void st_shared_v4(uint32_t saddr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(saddr), "r"(a), "r"(b), "r"(c), "r"(d) : "memory");
}
__device__ __forceinline__ void st_shared_u16(uint32_t saddr, uint16_t v) {
  asm volatile("st.shared.u16 [%0], %1;" ::"r"(saddr), "h"(v) : "memory");
}
__device__ __forceinline__ uint16_t bf16_bits(float a) {
  __nv_bfloat16 h = __float2bfloat16_rn(a);
  return *reinterpret_cast<uint16_t*>(&h);
}

// Copies a row-major [N][K] BF16 matrix from global memory into the
// interleaved layout at sbase (rows N..Npad-1 zero). All threads of the block
// take part.
__device__ __forceinline__ void load_weights(uint8_t* sbase, const __nv_bfloat16* g, int N, int K, int Npad) {
  const uint32_t s = smem_u32(sbase);
  const int chunks = Npad * (K / 8);
  for (int c = threadIdx.x; c < chunks; c += blockDim.x) {
    int n = c / (K / 8), k8 = c % (K / 8);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (n < N) v = *reinterpret_cast<const uint4*>(g + size_t(n) * K + k8 * 8);
    st_shared_v4(s + ik_off(n, k8 * 8, K), v.x, v.y, v.z, v.w);
  }
}

// ---------------------------------------------------------- encoding ----
// One row's 208 features, in groups of 8 (group g = features 8g..8g+7).
struct EncIn {
  float v[6];         // normalised position (3) and normal (3), in [0, 1]
  float theta, phi;   // outgoing direction: theta / pi, phi / (2 pi), in [0, 1]
};

__device__ __forceinline__ EncIn make_enc(const GuideNet& net, float px, float py, float pz, float nx, float ny,
                                          float nz, float wx, float wy, float wz) {
  EncIn e;
  e.v[0] = fminf(fmaxf((px - net.lo[0]) * net.inv_ext[0], 0.f), 1.f);
  e.v[1] = fminf(fmaxf((py - net.lo[1]) * net.inv_ext[1], 0.f), 1.f);
  e.v[2] = fminf(fmaxf((pz - net.lo[2]) * net.inv_ext[2], 0.f), 1.f);
  e.v[3] = 0.5f * (nx + 1.f);
  e.v[4] = 0.5f * (ny + 1.f);
  e.v[5] = 0.5f * (nz + 1.f);
  e.theta = acosf(fminf(fmaxf(wz, -1.f), 1.f)) * (1.f / kPi);
  e.phi = atan2f(wy, wx) * (0.5f / kPi) + 0.5f;
  return e;
}

// Eight features of group g. A frequency group holds bands j0 .. j0 + 3 of one
// coordinate (j0 = 0, 4, 8): band j0 is evaluated directly, the next three by
// the double-angle identities sin 2a = 2 sin a cos a, cos 2a = 1 - 2 sin^2 a.
// Each doubling about doubles the absolute error of the one before, so the
// features stay within ~1e-6 of the exact values (sincospif is within 1 ulp),
// far below the bfloat16 rounding the layer input gets.
__device__ __forceinline__ void enc_group(const EncIn& e, int g, float* out) {
  if (g < 18) {
    const int c = g / 3, j0 = 4 * (g % 3);
    float s, co;
    sincospif(e.v[c] * float(1 << j0), &s, &co);
    out[0] = s;
    out[1] = co;
#pragma unroll
    for (int q = 1; q < 4; ++q) {
      const float sc = s * co;
      co = fmaf(-2.f * s, s, 1.f);
      s = sc + sc;
      out[2 * q] = s;
      out[2 * q + 1] = co;
    }
  } else {
    // One-blob bins b0 .. b0 + 7: exp(-(D - q)^2 / 2) with D the distance in
    // bins from bin b0's centre. Consecutive bins differ by the factor
    // exp(D - q - 1/2), itself divided by e from one bin to the next, so a
    // group takes two exponentials. phi wraps around: its distance is taken
    // from the group's middle, wrapped to [-16, 16] bins (a bin that wraps
    // the other way lies more than 12.5 bins off, below 1e-33).
    const int f0 = 8 * g - 144, b0 = f0 & 31;
    float D = (f0 < 32 ? e.theta : e.phi) * float(kBlob) - (float(b0) + 0.5f);
    if (f0 >= 32) {
      const float m = D - 3.5f;
      D = m - float(kBlob) * rintf(m * (1.f / kBlob)) + 3.5f;
    }
    float gq = __expf(-0.5f * D * D), r = __expf(D - 0.5f);
    out[0] = gq;
#pragma unroll
    for (int q = 1; q < 8; ++q) {
      gq *= r;
      r *= 0.36787944117144233f;  // 1 / e
      out[q] = gq;
    }
  }
}

// Writes row r's encoding into an interleaved [128][208] tile (unrolled:
// every group's coordinate, band and bin are compile-time constants).
__device__ __forceinline__ void write_enc_row(uint32_t s, int r, const EncIn& e) {
#pragma unroll
  for (int g = 0; g < kIn / 8; ++g) {
    float f[8];
    enc_group(e, g, f);
    st_shared_v4(s + ik_off(r, 8 * g, kIn), pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]),
                 pack_bf16(f[6], f[7]));
  }
}

// ------------------------------------------------------ vMF mixture ----
// Decoded mixture of one vertex: weights, unit means, concentrations.
struct Mixture {
  float pi[kLobes];
  float mx[kLobes], my[kLobes], mz[kLobes];
  float kappa[kLobes];
};

// log of the vMF normalisation kappa / (2 pi (1 - exp(-2 kappa))).
__device__ __forceinline__ float vmf_log_norm(float k) {
  return logf(k) - logf(2.f * kPi) - logf(-expm1f(-2.f * k));
}

// Decodes the 40 raw outputs with the fast intrinsics (__expf, rsqrtf,
// __frcp_rn): relative errors of a few 1e-7, below the bfloat16 rounding of
// the layers that produced the outputs.
__device__ __forceinline__ void decode_mixture(const float* o, Mixture& m) {
  float mx = o[0];
#pragma unroll
  for (int k = 1; k < kLobes; ++k) mx = fmaxf(mx, o[k]);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    m.pi[k] = __expf(o[k] - mx);
    s += m.pi[k];
  }
  const float is = __frcp_rn(s);
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    m.pi[k] *= is;
    float x = o[8 + 3 * k], y = o[9 + 3 * k], z = o[10 + 3 * k];
    float l2 = x * x + y * y + z * z;
    if (l2 > 1e-24f) {
      float il = rsqrtf(l2);
      m.mx[k] = x * il; m.my[k] = y * il; m.mz[k] = z * il;
    } else {
      m.mx[k] = 0.f; m.my[k] = 0.f; m.mz[k] = 1.f;
    }
    m.kappa[k] = __expf(fminf(fmaxf(o[32 + k], kLogKappaMin), kLogKappaMax));
  }
}

// 1 - exp(-x) for x >= 0: its Taylor series to x^4 below 1/8 (relative error
// under x^4 / 120 = 2e-6), else with __expf (absolute error ~1e-7 on a
// result above 0.11).
__device__ __forceinline__ float one_minus_exp_neg(float x) {
  if (x < 0.125f) return x * (1.f - x * (0.5f - x * (1.f / 6.f - x * (1.f / 24.f))));
  return 1.f - __expf(-x);
}

// Writes a decoded mixture in the stored layout (kMixStride float4).
__device__ __forceinline__ void store_mixture(float4* out, const Mixture& m) {
  float c[kLobes];
#pragma unroll
  for (int k = 0; k < kLobes; ++k)
    c[k] = m.pi[k] * m.kappa[k] * __frcp_rn((2.f * kPi) * one_minus_exp_neg(2.f * m.kappa[k]));
  out[0] = make_float4(m.pi[0], m.pi[1], m.pi[2], m.pi[3]);
  out[1] = make_float4(m.pi[4], m.pi[5], m.pi[6], m.pi[7]);
#pragma unroll
  for (int k = 0; k < kLobes; ++k) out[2 + k] = make_float4(m.mx[k], m.my[k], m.mz[k], m.kappa[k]);
  out[10] = make_float4(c[0], c[1], c[2], c[3]);
  out[11] = make_float4(c[4], c[5], c[6], c[7]);
}

// Mixture pdf (solid angle) of the unit direction (x, y, z).
__device__ __forceinline__ float mixture_pdf(const float4* M, float x, float y, float z) {
  float4 c0 = M[10], c1 = M[11];
  float cs[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
  float q = 0.f;
#pragma unroll
  for (int k = 0; k < kLobes; ++k) {
    float4 l = M[2 + k];
    float d = l.x * x + l.y * y + l.z * z;
    q += cs[k] * __expf(l.w * (d - 1.f));
  }
  return q;
}

// Samples the mixture with u0 (lobe) and u1, u2 (direction about the mean).
__device__ __forceinline__ void mixture_sample(const float4* M, float u0, float u1, float u2, float& x, float& y,
                                               float& z) {
  float4 p0 = M[0], p1 = M[1];
  float pis[8] = {p0.x, p0.y, p0.z, p0.w, p1.x, p1.y, p1.z, p1.w};
  int k = kLobes - 1;
  float acc = 0.f;
#pragma unroll
  for (int j = 0; j < kLobes; ++j) {
    acc += pis[j];
    if (u0 < acc) { k = j; break; }
  }
  float4 l = M[2 + k];
  float kap = l.w;
  // cos of the angle to the mean (inversion of the vMF marginal)
  float w = 1.f + logf(u1 + (1.f - u1) * expf(-2.f * kap)) / kap;
  w = fminf(fmaxf(w, -1.f), 1.f);
  float sw = sqrtf(fmaxf(0.f, 1.f - w * w));
  float sn, cs;
  sincospif(2.f * u2, &sn, &cs);
  // orthonormal basis about the mean (Duff et al. 2017)
  float sg = copysignf(1.f, l.z);
  float a = -1.f / (sg + l.z);
  float b = l.x * l.y * a;
  float tx = 1.f + sg * l.x * l.x * a, ty = sg * b, tz = -sg * l.x;
  float bx = b, by = sg + l.y * l.y * a, bz = -l.y;
  x = sw * (cs * tx + sn * bx) + w * l.x;
  y = sw * (cs * ty + sn * by) + w * l.y;
  z = sw * (cs * tz + sn * bz) + w * l.z;
}

}  // namespace guide
}  // namespace gbrt
