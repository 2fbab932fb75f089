// chains.cuh — the Markov-chain renderers: MetropolisRenderer
// (src/metropolisrenderer.cpp:56-201) and EnergyRedistributionRenderer
// (src/energyredistributionrenderer.cpp:38-135) with MetropolisSample's
// mutations (src/metropolissample.cpp:33-121). Included by pathtrace.cu: the
// chains reuse its wavefront (extend / shade / shadow) with the shade kernel
// reading each path's random numbers from a stored primary-sample vector
// (PssSrc) instead of the counter-based stream.
//
// GB300 layout: one chain per wavefront slot, all chains advanced one
// mutation per wavefront. Sample vectors are structure-of-arrays floats,
// dimension d of chain c at [d * stride + c], so the mutation kernels and the
// shade kernel's reads of a dimension are coalesced across a warp. The film
// is an FP64 sum written with atomics (deposits land anywhere on the image).
//
// A sample has 3 + 5 D dimensions (D = max depth): camera point over the
// image (0, 1), path-length number (2), direction sample i (3 + 2i, 4 + 2i),
// light sample k (3 + 2D + 3k, +1) and light choice (3 + 2D + 3k + 2) — the
// dimension layout of the per-pixel renderer. The renderer's
// lightPathSamples and lightSample2 feed nothing in the unidirectional
// integrator and are not kept. Keys of the counter-based stream: tag << 56 |
// index, with the tags below (the oracle uses the same keys).

namespace gbrt {
namespace chain {

enum : unsigned long long { kBoot = 1, kMutate = 2, kPick = 3, kEd = 4, kInit = 5, kFlow = 6 };
__host__ __device__ __forceinline__ unsigned long long tag(unsigned long long t, unsigned long long id) {
  return (t << 56) | id;
}
__host__ __device__ __forceinline__ int dims(int D) { return 3 + 5 * D; }
// Dimensions a small step moves (MetropolisSample::smallStep, src/metropolissample.cpp:86-96):
// the camera point and the direction and light samples; not the path length
// (drawn afresh by every mutation) nor the light choice (large steps only).
__device__ __forceinline__ bool moves(int d, int D) {
  if (d == 2) return false;
  if (d >= 3 + 2 * D) return (d - 3 - 2 * D) % 3 != 2;
  return true;
}
// mutate(qreal&, rng), src/metropolissample.cpp:62-78: a step of b exp(-log(b / a) u1)
// (a = 1/1024, b = 1/64), negative when u2 < 1/2, wrapped into [0, 1].
// -log(16) is rounded to float, as the renderer's static float holds it.
__device__ __forceinline__ float mutate_coord(float s, float ux, float uy) {
  const float b = 1.f / 64.f, logRatio = -2.772588722239781f;
  float delta = __fmul_rn(b, expf(__fmul_rn(logRatio, ux)));
  if (uy < 0.5f) delta = -delta;
  s = __fadd_rn(s, delta);
  if (s < 0.f) s = __fadd_rn(s, 1.f);
  if (s > 1.f) s = __fadd_rn(s, -1.f);
  return s;
}
// lum() (src/mathhelper.cpp:102-105) of a BGR float4, the sum in double.
__host__ __device__ __forceinline__ float lum_bgr(float4 c) {
#ifdef __CUDA_ARCH__
  return __double2float_rn(__dadd_rn(__dadd_rn(__dmul_rn(0.299, double(c.z)), __dmul_rn(0.587, double(c.y))),
                                     __dmul_rn(0.114, double(c.x))));
#else
  return float(.299 * double(c.z) + .587 * double(c.y) + .114 * double(c.x));
#endif
}
// cv::norm of a Vec3f: the squares summed in double.
__device__ __forceinline__ double cv_norm(float4 c) {
  double s = __dmul_rn(double(c.x), double(c.x));
  s = __dadd_rn(s, __dmul_rn(double(c.y), double(c.y)));
  s = __dadd_rn(s, __dmul_rn(double(c.z), double(c.z)));
  return __dsqrt_rn(s);
}
// MetropolisSample::getPos (src/metropolissample.cpp:129-136): the pixel of a camera coordinate.
__device__ __forceinline__ int pixel_of(float u, int n) {
  return max(0, min(int(__dmul_rn(double(u), double(n))), n - 1));
}
__device__ __forceinline__ float4 finite_or_zero(float4 L, unsigned long long* bad) {
  if (isfinite(L.x) && isfinite(L.y) && isfinite(L.z)) return make_float4(L.x, L.y, L.z, 0.f);
  atomicAdd(bad, 1ull);
  return make_float4(0.f, 0.f, 0.f, 0.f);
}
__device__ __forceinline__ void deposit(double* sum, int W, int H, float ux, float uy, float w, float4 v) {
  const size_t o = (size_t(pixel_of(uy, H)) * W + pixel_of(ux, W)) * 3;
  atomicAdd(sum + o, double(__fmul_rn(w, v.x)));
  atomicAdd(sum + o + 1, double(__fmul_rn(w, v.y)));
  atomicAdd(sum + o + 2, double(__fmul_rn(w, v.z)));
}
__device__ __forceinline__ void count_warp(bool pred, unsigned long long* counter) {
  const unsigned m = __ballot_sync(__activemask(), pred);
  if (m && (threadIdx.x & 31) == __ffs(__activemask()) - 1) atomicAdd(counter, (unsigned long long)__popc(m));
}

// The camera ray of a sample (MetropolisSample::cameraPathFromSample,
// src/metropolissample.cpp:120-127: the point times the resolution) and the path length from its
// dimension 2 (D when P.term_p is 0), started in slot.
template <class R>
__device__ __forceinline__ void start_from(const PTParams& P, const PTState& st, int slot, const R& rs) {
  const float sxp = __fmul_rn(rs.u(0), float(P.cam.W)), syp = __fmul_rn(rs.u(1), float(P.cam.H));
  float dx, dy, dz;
  camera_dir(P, sxp, syp, dx, dy, dz);
  start_path(P, st, slot, ref_path_length(P, rs.u(2)), dx, dy, dz);
}

__device__ __forceinline__ void reset_queues(const PTParams& P, const PTState& st, int slot) {
  if (slot == 0) {
    st.counts[0] = P.nb;
    st.work[0] = 0;
  }
}

// Samples drawn whole from the stream of key (seed, g0 + slot): the
// bootstrap's large steps.
__global__ void __launch_bounds__(256) k_chain_raygen(PTParams P, PTState st) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  reset_queues(P, st, slot);
  if (slot >= P.nb) return;
  start_from(P, st, slot, StreamSrc(P, slot));
}

// Radiance of every slot (non-finite: zero, counted).
__global__ void __launch_bounds__(256) k_collect(PTParams P, PTState st, float4* out) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.nb) return;
  out[slot] = finite_or_zero(st.L[slot], &st.tally[2]);
}

// ------------------------------------------------------------------ MLT ----
struct MltArgs {
  float* cur;            // current samples, nd x N
  float* prop;           // proposals, nd x N
  float4* curV;          // current radiance
  double* sum;           // film sums, H x W x 3
  unsigned long long* accepted;
  const unsigned long long* t;  // mutation index of the iteration (device counter, advanced by k_tick)
  int N, nd;
  float large_p;
  float b;               // mean bootstrap luminance
  float mutations;       // numPixelSamples
};

// Chain c starts at bootstrap sample pick[c].
__global__ void __launch_bounds__(256) k_mlt_init(PTParams P, MltArgs A, const int* pick, const float4* bootL) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= A.N) return;
  const int bi = pick[c];
  const unsigned long long key = stream_key(P.seed, tag(kBoot, (unsigned long long)bi));
  for (int d = 0; d < A.nd; ++d) A.cur[size_t(d) * A.N + c] = stream_u(key, unsigned(d));
  A.curV[c] = bootL[bi];
}

// MetropolisSample::mutated (src/metropolissample.cpp:104-118): a fresh path length, then a
// large step (every dimension afresh) with probability large_p, else a small
// step; the proposal's path starts in slot c.
__global__ void __launch_bounds__(256) k_mlt_propose(PTParams P, PTState st, MltArgs A) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  reset_queues(P, st, c);
  if (c >= A.N) return;
  const unsigned long long key = stream_key(P.seed, tag(kMutate, *A.t * unsigned(A.N) + unsigned(c)));
  const bool large = stream_u(key, 0) < A.large_p;
  for (int d = 0; d < A.nd; ++d) {
    const size_t o = size_t(d) * A.N + c;
    float v;
    if (d == 2) v = stream_u(key, 2);
    else if (large) v = stream_u(key, 3u + 2u * d);
    else v = moves(d, P.D) ? mutate_coord(A.cur[o], stream_u(key, 3u + 2u * d), stream_u(key, 4u + 2u * d)) : A.cur[o];
    A.prop[o] = v;
  }
  start_from(P, st, c, PssSrc(P, c));
}

// src/metropolisrenderer.cpp:155-182: acceptance a = min(1, lum(new) / lum(cur)), the expected
// value deposits (1 - a) of the current and a of the proposal, each scaled
// to luminance b / mutations, then the move with probability a.
__global__ void __launch_bounds__(256) k_mlt_accept(PTParams P, PTState st, MltArgs A) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= A.N) return;
  const unsigned long long key = stream_key(P.seed, tag(kMutate, *A.t * unsigned(A.N) + unsigned(c)));
  const float4 nv = finite_or_zero(st.L[c], &st.tally[2]);
  const float4 cv = A.curV[c];
  const float lc = lum_bgr(cv), ln = lum_bgr(nv);
  const float ratio = __fdiv_rn(ln, lc);
  const float a = ratio < 1.f ? ratio : 1.f;  // std::min<float>(1, ratio): NaN gives 1
  const int W = P.cam.W, H = P.cam.H;
  if (lc > 0.f) {
    const float s = __fdiv_rn(__fmul_rn(__fdiv_rn(1.f, lc), A.b), A.mutations);
    const float4 v = make_float4(__fmul_rn(cv.x, s), __fmul_rn(cv.y, s), __fmul_rn(cv.z, s), 0.f);
    deposit(A.sum, W, H, A.cur[c], A.cur[size_t(A.N) + c], __fadd_rn(1.f, -a), v);
  }
  if (ln > 0.f) {
    const float s = __fdiv_rn(__fmul_rn(__fdiv_rn(1.f, ln), A.b), A.mutations);
    const float4 v = make_float4(__fmul_rn(nv.x, s), __fmul_rn(nv.y, s), __fmul_rn(nv.z, s), 0.f);
    deposit(A.sum, W, H, A.prop[c], A.prop[size_t(A.N) + c], a, v);
  }
  const bool acc = stream_u(key, 1) < a;
  count_warp(acc, A.accepted);
  if (acc) {
    for (int d = 0; d < A.nd; ++d) A.cur[size_t(d) * A.N + c] = A.prop[size_t(d) * A.N + c];
    A.curV[c] = nv;
  }
}

// ----------------------------------------------------------------- ERPT ----
struct ErptArgs {
  float* y;              // current samples of the chains of a batch, nd x B
  float* z;              // proposals, nd x B
  float4* yV;            // current radiance (w unused)
  double* dep;           // per chain: |depVal|
  double* sum;           // film sums
  int* count;            // per initial sample: chains
  float4* c0;            // per initial sample: its radiance
  double* dep0;          // per initial sample: |depVal|
  const long long* incl; // inclusive prefix sums of count
  unsigned long long* accepted;
  long long q0;          // first chain of the batch
  long long n_init;
  const unsigned long long* m;  // mutation of the chains (device counter, advanced by k_tick)
  int B, nd, xs, ys, M;
  float ed;
};

// Initial sample g: JitteredSampler(xs, ys) point of its pixel over the
// image (src/energyredistributionrenderer.cpp:63-76), MetropolisSample::initAtPixel's large step for the
// other dimensions.
__device__ __forceinline__ float erpt_init_dim(const PTParams& P, const ErptArgs& A, unsigned long long g,
                                               unsigned long long key, int d) {
  if (d >= 2) return stream_u(key, unsigned(d));
  const int spp = A.xs * A.ys;
  const long long pixel = (long long)(g / unsigned(spp));
  const int s = int(g - (unsigned long long)pixel * unsigned(spp));
  const int W = P.cam.W;
  if (d == 0) {
    const int a = s / A.ys, j = int(pixel % W);
    const double jx = __ddiv_rn(__dadd_rn(double(stream_u(key, 0)), double(a)), double(A.xs));
    return __double2float_rn(__ddiv_rn(__dadd_rn(double(j), jx), double(W)));
  }
  const int b = s % A.ys, i = int(pixel / W);
  const double jy = __ddiv_rn(__dadd_rn(double(stream_u(key, 1)), double(b)), double(A.ys));
  return __double2float_rn(__ddiv_rn(__dadd_rn(double(i), jy), double(P.cam.H)));
}

// computeEd (src/energyredistributionrenderer.cpp:120-135): one path through each pixel's corner with the
// integrator's termination probability 0.1. P.g0 = tag(kEd, first pixel).
__global__ void __launch_bounds__(256) k_erpt_corner_raygen(PTParams P, PTState st) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  reset_queues(P, st, slot);
  if (slot >= P.nb) return;
  const long long pixel = (long long)((P.g0 & ((1ull << 56) - 1)) + unsigned(slot));
  const StreamSrc rs(P, slot);
  float dx, dy, dz;
  camera_dir(P, float(pixel % P.cam.W), float(pixel / P.cam.W), dx, dy, dz);
  start_path(P, st, slot, ref_path_length(P, rs.u(2)), dx, dy, dz);
}

// Sum of the radiance of every slot (non-finite: dropped, counted).
__global__ void __launch_bounds__(256) k_sum_radiance(PTParams P, PTState st, double* acc) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  float4 L = make_float4(0.f, 0.f, 0.f, 0.f);
  if (slot < P.nb) L = finite_or_zero(st.L[slot], &st.tally[2]);
  double s0 = L.x, s1 = L.y, s2 = L.z;
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(acc, s0);
    atomicAdd(acc + 1, s1);
    atomicAdd(acc + 2, s2);
  }
}

// Initial samples g0 + slot: their vectors (in A.z) and paths (full length,
// no roulette: MetropolisSample starts with pathLength MAX_DEPTH and
// terminationProb 1).
__global__ void __launch_bounds__(256) k_erpt_init_raygen(PTParams P, PTState st, ErptArgs A) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  reset_queues(P, st, slot);
  if (slot >= P.nb) return;
  const unsigned long long g = P.g0 + unsigned(slot);
  const unsigned long long key = stream_key(P.seed, tag(kInit, g));
  for (int d = 0; d < A.nd; ++d) A.z[size_t(d) * A.B + slot] = erpt_init_dim(P, A, g, key, d);
  start_from(P, st, slot, PssSrc(P, slot));
}

// equalDispositionFlow's set-up (src/energyredistributionrenderer.cpp:85-91): (int)(u + |c| / (M ed))
// chains, each depositing |depVal| = |c ed / |c| / chains| per mutation.
__global__ void __launch_bounds__(256) k_erpt_count(PTParams P, PTState st, ErptArgs A) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.nb) return;
  const unsigned long long g = P.g0 + unsigned(slot);
  const unsigned long long key = stream_key(P.seed, tag(kInit, g));
  const float4 c = finite_or_zero(st.L[slot], &st.tally[2]);
  const double nc = cv_norm(c);
  const float me = __fmul_rn(float(A.M), A.ed);
  const double x = __dadd_rn(double(stream_u(key, unsigned(A.nd))), __ddiv_rn(nc, double(me)));
  const int n = x > 0.0 ? int(x) : 0;
  A.count[g] = n;
  A.c0[g] = c;
  double dn = 0.0;
  if (n > 0) {
    const double sc = __ddiv_rn(__ddiv_rn(double(A.ed), nc), double(n));
    const float4 dv = make_float4(__double2float_rn(__dmul_rn(double(c.x), sc)),
                                  __double2float_rn(__dmul_rn(double(c.y), sc)),
                                  __double2float_rn(__dmul_rn(double(c.z), sc)), 0.f);
    dn = cv_norm(dv);
  }
  A.dep0[g] = dn;
}

// Chain q0 + slot: its initial sample is the first g with incl[g] > q.
__global__ void __launch_bounds__(256) k_erpt_chain_init(PTParams P, ErptArgs A, int nq) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= nq) return;
  const long long q = A.q0 + slot;
  long long lo = 0, hi = A.n_init - 1;
  while (lo < hi) {
    const long long mid = (lo + hi) >> 1;
    if (A.incl[mid] > q) hi = mid;
    else lo = mid + 1;
  }
  const unsigned long long g = (unsigned long long)lo;
  const unsigned long long key = stream_key(P.seed, tag(kInit, g));
  for (int d = 0; d < A.nd; ++d) A.y[size_t(d) * A.B + slot] = erpt_init_dim(P, A, g, key, d);
  A.yV[slot] = A.c0[g];
  A.dep[slot] = A.dep0[g];
}

// A small step of every chain (src/energyredistributionrenderer.cpp:99-100); the proposal's path in slot.
__global__ void __launch_bounds__(256) k_erpt_propose(PTParams P, PTState st, ErptArgs A) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  reset_queues(P, st, slot);
  if (slot >= P.nb) return;
  const unsigned long long id = (unsigned long long)(A.q0 + slot) * unsigned(A.M) + *A.m;
  const unsigned long long key = stream_key(P.seed, tag(kFlow, id));
  for (int d = 0; d < A.nd; ++d) {
    const size_t o = size_t(d) * A.B + slot;
    const float v = A.y[o];
    A.z[o] = moves(d, P.D) ? mutate_coord(v, stream_u(key, 3u + 2u * d), stream_u(key, 4u + 2u * d)) : v;
  }
  start_from(P, st, slot, PssSrc(P, slot));
}

// src/energyredistributionrenderer.cpp:101-115: q = min(1, |z| / |y|), the move when q > u, then a deposit
// of |depVal| y / |y| / (xs ys) at the (new) current sample's pixel, y being
// the radiance before the move.
__global__ void __launch_bounds__(256) k_erpt_accept(PTParams P, PTState st, ErptArgs A) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.nb) return;
  const unsigned long long id = (unsigned long long)(A.q0 + slot) * unsigned(A.M) + *A.m;
  const unsigned long long key = stream_key(P.seed, tag(kFlow, id));
  const float4 zv = finite_or_zero(st.L[slot], &st.tally[2]);
  const float4 yv = A.yV[slot];
  const double ny = cv_norm(yv);
  const float yl = __double2float_rn(ny), zl = __double2float_rn(cv_norm(zv));
  const float ratio = __fdiv_rn(zl, yl);
  const float q = ratio < 1.f ? ratio : 1.f;
  const bool acc = q > stream_u(key, 1);
  count_warp(acc, A.accepted);
  if (acc) {
    for (int d = 0; d < A.nd; ++d) A.y[size_t(d) * A.B + slot] = A.z[size_t(d) * A.B + slot];
    A.yV[slot] = zv;
  }
  const double dn = A.dep[slot];
  const double in = __ddiv_rn(1.0, ny);
  const float isp = __fdiv_rn(1.f, float(A.xs * A.ys));
  float4 t = make_float4(__double2float_rn(__dmul_rn(dn, double(yv.x))), __double2float_rn(__dmul_rn(dn, double(yv.y))),
                         __double2float_rn(__dmul_rn(dn, double(yv.z))), 0.f);
  t = make_float4(__double2float_rn(__dmul_rn(double(t.x), in)), __double2float_rn(__dmul_rn(double(t.y), in)),
                  __double2float_rn(__dmul_rn(double(t.z), in)), 0.f);
  deposit(A.sum, P.cam.W, P.cam.H, A.y[slot], A.y[size_t(A.B) + slot], isp, t);
}

// Advances an iteration counter (the last node of an iteration's graph).
__global__ void k_tick(unsigned long long* counter) { ++*counter; }

// Inclusive prefix sums of n ints into long longs: per-block scans, a scan of
// the block totals by one block, then the block offsets added.
constexpr int kScanBlock = 1024;
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(const int* in, long long* out, long long* totals,
                                                           long long n) {
  __shared__ long long warp_sum[kScanBlock / 32];
  const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  long long v = i < n ? in[i] : 0;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const long long x = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= o) v += x;
  }
  if (lane == 31) warp_sum[w] = v;
  __syncthreads();
  if (w == 0) {
    long long s = warp_sum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long x = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += x;
    }
    warp_sum[lane] = s;
  }
  __syncthreads();
  if (w > 0) v += warp_sum[w - 1];
  if (i < n) out[i] = v;
  if (threadIdx.x == kScanBlock - 1) totals[blockIdx.x] = v;
}
__global__ void __launch_bounds__(kScanBlock) k_scan_totals(long long* totals, int nblocks) {
  // one block: each thread scans a contiguous run, then the runs are offset
  __shared__ long long run_sum[kScanBlock];
  const int per = (nblocks + kScanBlock - 1) / kScanBlock;
  const int b0 = threadIdx.x * per, b1 = min(nblocks, b0 + per);
  long long s = 0;
  for (int b = b0; b < b1; ++b) s += totals[b];
  run_sum[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int k = 0; k < kScanBlock; ++k) {
      const long long x = run_sum[k];
      run_sum[k] = acc;
      acc += x;
    }
  }
  __syncthreads();
  long long acc = run_sum[threadIdx.x];
  for (int b = b0; b < b1; ++b) {
    acc += totals[b];
    totals[b] = acc;  // inclusive
  }
}
__global__ void __launch_bounds__(kScanBlock) k_scan_add(long long* out, const long long* totals, long long n) {
  const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n && blockIdx.x > 0) out[i] += totals[blockIdx.x - 1];
}

}  // namespace chain

// ---------------------------------------------------------------- host ----
// The wavefront shared by every phase: extend / shade / shadow D times.
struct Wave {
  TraceKernels tk;
  void (*shade)(DeviceScene, PTParams, PTState, int);
  int traceGrid, shadowGrid, shadeGrid;
};

static Wave make_wave(gbrt_scene* s, bool pss) {
  Wave w;
  w.tk = pick_kernels(s, false);
  const bool ext = ext_scene(s);
  if (pss) w.shade = ext ? k_shade<true, PssSrc> : k_shade<false, PssSrc>;
  else w.shade = ext ? k_shade<true, StreamSrc> : k_shade<false, StreamSrc>;
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, w.tk.ext, kTraceBlock, 0);
  w.traceGrid = std::max(1, per) * s->ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, w.tk.sh, kTraceBlock, 0);
  w.shadowGrid = std::max(1, per) * s->ctx->num_sms;
  w.shadeGrid = s->ctx->num_sms * 8;
  return w;
}

static unsigned long long run_wave(gbrt_scene* s, const Wave& w, const PTParams& P, const PTState& st,
                                   cudaStream_t stream) {
  for (int it = 0; it < P.D; ++it) {
    const int cur = it & 1;
    w.tk.ext<<<cap_grid(w.traceGrid, P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st, cur);
    w.shade<<<cap_grid(w.shadeGrid, P.nb, 256), 256, 0, stream>>>(s->view, P, st, cur);
    w.tk.sh<<<cap_grid(w.shadowGrid, 2ll * P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st);
  }
  return 3ull * unsigned(P.D);
}

// Runs `iterations` times the launches that `enqueue` issues on stream: they
// are captured once into a CUDA graph and the graph is replayed, so an
// iteration of many small launches (few chains) costs one graph launch of
// host time. The launches read their iteration number from a device counter
// that the captured sequence advances.
template <class F>
static cudaError_t replay(cudaStream_t stream, long long iterations, F enqueue) {
  if (iterations <= 0) return cudaSuccess;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  enqueue();
  e = cudaStreamEndCapture(stream, &graph);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  for (long long k = 0; k < iterations && e == cudaSuccess; ++k) e = cudaGraphLaunch(exec, stream);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  return e;
}

static cudaError_t alloc_state(gbrt_scene* s, Buffers& buf, PTState& st, long long B) {
  std::memset(&st, 0, sizeof st);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(buf.alloc(&st.alpha, B)); A(buf.alloc(&st.L, B)); A(buf.alloc(&st.ctl, B));
  A(buf.alloc(&st.pv_p, B)); A(buf.alloc(&st.pv_n, B)); A(buf.alloc(&st.pv_d, B)); A(buf.alloc(&st.pv_a, B));
  A(buf.alloc(&st.ext[0], 2 * B)); A(buf.alloc(&st.ext[1], 2 * B));
  A(buf.alloc(&st.ext_slot[0], B)); A(buf.alloc(&st.ext_slot[1], B));
  A(buf.alloc(&st.hits, B));
  if (s->view.inst) A(buf.alloc(&st.hit_inst, B));
  A(buf.alloc(&st.sh_ray, 4 * B)); A(buf.alloc(&st.sh_c, 2 * B)); A(buf.alloc(&st.sh_slot, 2 * B));
  A(buf.alloc(&st.counts, 4)); A(buf.alloc(&st.work, 4)); A(buf.alloc(&st.tally, 8)); A(buf.alloc(&st.err, 1));
  st.ext_cap = int(B);
  st.sh_cap = int(2 * B);
  if (e != cudaSuccess) return e;
  A(cudaMemsetAsync(st.tally, 0, 8 * sizeof(unsigned long long), buf.stream));
  A(cudaMemsetAsync(st.err, 0, sizeof(int), buf.stream));
  return e;
}

static gbrt_status check_chain_params(gbrt_ctx* ctx, const gbrt_camera* cam, const gbrt_render_params* prm,
                                      const char* who) {
  if (!cam || !prm) return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": NULL argument");
  if (cam->width <= 0 || cam->height <= 0 || prm->max_depth <= 0 || prm->max_depth > 64)
    return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": bad camera or max depth");
  if (prm->semantics != GBRT_SEM_REFERENCE)
    return fail(ctx, GBRT_ERR_INVALID_ARG, std::string(who) + ": the renderer's estimator only (GBRT_SEM_REFERENCE)");
  return GBRT_OK;
}

// Common tail: tallies, error word, film copy-out, statistics.
static gbrt_status chain_finish(gbrt_scene* s, const char* who, const PTState& st, double* d_sum, float* d_film,
                                size_t n3, float* film, cudaEvent_t ev0, cudaEvent_t ev1, cudaStream_t stream,
                                gbrt_chain_stats* stats, cudaError_t e) {
  gbrt_ctx* ctx = s->ctx;
  unsigned long long tally[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int err = 0;
  if (e == cudaSuccess) {
    k_finalize<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_sum, d_film, n3, 1.0);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(ev1, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(tally, st.tally, sizeof tally, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&err, st.err, sizeof err, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(film, d_film, n3 * sizeof(float), cudaMemcpyDeviceToHost, stream);
  cudaError_t r = cudaStreamSynchronize(stream);
  if (e == cudaSuccess) e = r;
  float ms = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  if (e != cudaSuccess) return cuda_fail(ctx, e, who);
  if (stats) {
    stats->extension_rays = tally[0];
    stats->shadow_rays = tally[1];
    stats->nonfinite = tally[2];
    stats->render_ms = ms;
  }
  if (err) return fail(ctx, GBRT_ERR_NUMERIC, err_text(who, err));
  return GBRT_OK;
}

static gbrt_status mlt_impl(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                            const gbrt_mlt_params* mp, float* film, gbrt_chain_stats* stats) {
  gbrt_ctx* ctx = s->ctx;
  gbrt_status vs = check_chain_params(ctx, cam, prm, "gbrt_render_mlt");
  if (vs != GBRT_OK) return vs;
  if (!mp || !film || mp->mutations <= 0 || mp->bootstrap <= 0 || mp->chains < 0 ||
      !(mp->large_step_prob >= 0.f && mp->large_step_prob <= 1.f) ||
      !(mp->termination_prob >= 0.f && mp->termination_prob <= 1.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_mlt: bad Metropolis parameters");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  cudaStream_t stream = ctx->stream;
  const int W = cam->width, H = cam->height, D = prm->max_depth, nd = chain::dims(D);
  const long long total = (long long)mp->mutations * W * H;
  // Default: at least 16 mutations per chain, at most 2^20 chains (a
  // wavefront that fills the GPU), at least 4096.
  long long N = mp->chains > 0 ? mp->chains : std::min<long long>(1ll << 20, std::max<long long>(total / 16, 4096));
  N = std::max<long long>(1, std::min(N, total));
  if (N > (1ll << 26)) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_mlt: more than 2^26 chains");
  const long long M = std::max<long long>(1, total / N);
  const int nb = mp->bootstrap;
  const long long Bb = std::min<long long>(nb, 1ll << 20);  // bootstrap wavefront
  const long long B = std::max(N, Bb);
  const size_t n3 = size_t(W) * H * 3;

  Buffers buf(ctx, stream);
  PTState st;
  cudaError_t e = alloc_state(s, buf, st, B);
  float *cur = nullptr, *prop = nullptr, *d_film = nullptr;
  float4 *curV = nullptr, *bootL = nullptr;
  double* d_sum = nullptr;
  int* d_pick = nullptr;
  unsigned long long* d_acc = nullptr;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(buf.alloc(&cur, size_t(nd) * N)); A(buf.alloc(&prop, size_t(nd) * N)); A(buf.alloc(&curV, N));
  A(buf.alloc(&bootL, nb)); A(buf.alloc(&d_sum, n3)); A(buf.alloc(&d_film, n3)); A(buf.alloc(&d_pick, N));
  A(buf.alloc(&d_acc, 1));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_mlt buffers");
  A(cudaMemsetAsync(d_sum, 0, n3 * sizeof(double), stream));
  A(cudaMemsetAsync(d_acc, 0, sizeof(unsigned long long), stream));
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, stream);
  unsigned long long launches = 0;

  PTParams P{};
  init_params(P, s->ctx, *cam, *prm, 1);
  P.seed = prm->seed;
  P.xs = P.ys = P.spp = 1;
  // Bootstrap (src/metropolisrenderer.cpp:77-100): large steps at full length (MetropolisSample
  // starts with pathLength MAX_DEPTH and terminationProb 1).
  P.term_p = 0.f;
  P.rr_pdf = 1.f;
  P.inv_log1mp = 0.f;
  const Wave wS = make_wave(s, false), wP = make_wave(s, true);
  for (long long i0 = 0; i0 < nb && e == cudaSuccess; i0 += Bb) {
    P.g0 = chain::tag(chain::kBoot, (unsigned long long)i0);
    P.nb = int(std::min<long long>(Bb, nb - i0));
    chain::k_chain_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
    launches += 1 + run_wave(s, wS, P, st, stream);
    chain::k_collect<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st, bootL + i0);
    launches += 1;
    A(cudaGetLastError());
  }
  // Initial samples (src/metropolisrenderer.cpp:102-113) on the host: the running sum of the
  // bootstrap luminances in float, as the renderer keeps it, and chain c's
  // start where it first exceeds (u + c) / N of the total.
  std::vector<float4> hb(static_cast<size_t>(nb));
  if (e == cudaSuccess) A(cudaMemcpyAsync(hb.data(), bootL, sizeof(float4) * nb, cudaMemcpyDeviceToHost, stream));
  if (e == cudaSuccess) A(cudaStreamSynchronize(stream));
  if (e != cudaSuccess) {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    return cuda_fail(ctx, e, "gbrt_render_mlt bootstrap");
  }
  std::vector<float> cum(static_cast<size_t>(nb));
  float sumI = 0.f;
  for (int i = 0; i < nb; ++i) {
    sumI += chain::lum_bgr(hb[i]);
    cum[i] = sumI;
  }
  const float b = sumI / float(nb);
  const double u0 = stream_u(stream_key(prm->seed, chain::tag(chain::kPick, 0)), 0);
  std::vector<int> pick(static_cast<size_t>(N));
  for (long long c = 0; c < N; ++c) {
    const float off = float((u0 + double(c)) / double(N) * double(sumI));
    long long bi = std::upper_bound(cum.begin(), cum.end(), off) - cum.begin();
    pick[c] = int(std::min<long long>(bi, nb - 1));
  }
  A(cudaMemcpyAsync(d_pick, pick.data(), sizeof(int) * N, cudaMemcpyHostToDevice, stream));
  unsigned long long* d_iter = nullptr;
  A(buf.alloc(&d_iter, 1));
  A(cudaMemsetAsync(d_iter, 0, sizeof(unsigned long long), stream));
  chain::MltArgs MA;
  MA.cur = cur; MA.prop = prop; MA.curV = curV; MA.sum = d_sum; MA.accepted = d_acc;
  MA.N = int(N); MA.nd = nd; MA.large_p = mp->large_step_prob; MA.b = b; MA.mutations = float(mp->mutations);
  MA.t = d_iter;
  P.g0 = 0;
  P.nb = int(N);
  const int grid = int((N + 255) / 256);
  chain::k_mlt_init<<<grid, 256, 0, stream>>>(P, MA, d_pick, bootL);
  ++launches;
  // The chains (src/metropolisrenderer.cpp:131-190), one mutation of every chain per wavefront.
  P.term_p = mp->termination_prob;
  P.rr_pdf = mp->termination_prob > 0.f ? mp->termination_prob : 1.f;
  P.inv_log1mp = (mp->termination_prob > 0.f && mp->termination_prob < 1.f)
                     ? float(1.0 / std::log(1.0 - double(mp->termination_prob)))
                     : 0.f;
  P.pss = prop;
  P.pss_stride = int(N);
  if (e == cudaSuccess) {
    unsigned long long per = 0;
    A(replay(stream, M, [&] {
      chain::k_mlt_propose<<<grid, 256, 0, stream>>>(P, st, MA);
      per = 3 + run_wave(s, wP, P, st, stream);
      chain::k_mlt_accept<<<grid, 256, 0, stream>>>(P, st, MA);
      chain::k_tick<<<1, 1, 0, stream>>>(d_iter);
    }));
    launches += per * (unsigned long long)M;
  }
  unsigned long long acc = 0;
  if (e == cudaSuccess) A(cudaMemcpyAsync(&acc, d_acc, sizeof acc, cudaMemcpyDeviceToHost, stream));
  gbrt_status r = chain_finish(s, "gbrt_render_mlt", st, d_sum, d_film, n3, film, ev0, ev1, stream, stats, e);
  if (stats && r == GBRT_OK) {
    stats->paths = (unsigned long long)nb + (unsigned long long)(N * M);
    stats->chains = (unsigned long long)N;
    stats->mutations = (unsigned long long)(N * M);
    stats->accepted = acc;
    stats->normaliser = b;
    stats->kernel_launches = launches + 1;
  }
  return r;
}

static gbrt_status erpt_impl(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                             const gbrt_erpt_params* ep, float* film, gbrt_chain_stats* stats) {
  gbrt_ctx* ctx = s->ctx;
  gbrt_status vs = check_chain_params(ctx, cam, prm, "gbrt_render_erpt");
  if (vs != GBRT_OK) return vs;
  if (!ep || !film || ep->mutations <= 0 || ep->x_samples <= 0 || ep->y_samples <= 0 || ep->batch_chains < 0)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_erpt: bad energy-redistribution parameters");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  cudaStream_t stream = ctx->stream;
  const int W = cam->width, H = cam->height, D = prm->max_depth, nd = chain::dims(D);
  const int xs = ep->x_samples, ys = ep->y_samples, spp = xs * ys, M = ep->mutations;
  const long long npix = (long long)W * H, n_init = npix * spp;
  const long long B = std::max<long long>(1, ep->batch_chains > 0 ? std::min<long long>(ep->batch_chains, 1ll << 26)
                                                                  : (1ll << 22));
  const size_t n3 = size_t(npix) * 3;

  Buffers buf(ctx, stream);
  PTState st;
  cudaError_t e = alloc_state(s, buf, st, B);
  chain::ErptArgs EA;
  std::memset(&EA, 0, sizeof EA);
  float* d_film = nullptr;
  double *d_sum = nullptr, *d_ed = nullptr;
  long long* totals = nullptr;
  const long long nblk = (n_init + chain::kScanBlock - 1) / chain::kScanBlock;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(buf.alloc(&EA.y, size_t(nd) * B)); A(buf.alloc(&EA.z, size_t(nd) * B)); A(buf.alloc(&EA.yV, B));
  A(buf.alloc(&EA.dep, B)); A(buf.alloc(&EA.count, n_init)); A(buf.alloc(&EA.c0, n_init));
  A(buf.alloc(&EA.dep0, n_init));
  long long* incl = nullptr;
  A(buf.alloc(&incl, n_init)); A(buf.alloc(&totals, nblk)); A(buf.alloc(&EA.accepted, 1));
  A(buf.alloc(&d_sum, n3)); A(buf.alloc(&d_film, n3)); A(buf.alloc(&d_ed, 3));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_erpt buffers");
  if (nblk > (long long)chain::kScanBlock * 4096) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_erpt: too many samples");
  unsigned long long* d_iter = nullptr;
  A(buf.alloc(&d_iter, 1));
  EA.m = d_iter;
  EA.incl = incl;
  EA.sum = d_sum;
  EA.nd = nd; EA.xs = xs; EA.ys = ys; EA.M = M; EA.B = int(B); EA.n_init = n_init;
  A(cudaMemsetAsync(d_sum, 0, n3 * sizeof(double), stream));
  A(cudaMemsetAsync(d_ed, 0, 3 * sizeof(double), stream));
  A(cudaMemsetAsync(EA.accepted, 0, sizeof(unsigned long long), stream));
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventRecord(ev0, stream);
  unsigned long long launches = 0, paths = 0;
  const Wave wS = make_wave(s, false), wP = make_wave(s, true);

  PTParams P{};
  init_params(P, s->ctx, *cam, *prm, 1);
  P.xs = P.ys = P.spp = 1;
  // computeEd: pixel corners, termination probability 0.1 (its roulette
  // compensation included).
  P.term_p = 0.1f;
  P.rr_pdf = 0.1f;
  P.inv_log1mp = float(1.0 / std::log(1.0 - double(0.1f)));
  for (long long p0 = 0; p0 < npix && e == cudaSuccess; p0 += B) {
    P.g0 = chain::tag(chain::kEd, (unsigned long long)p0);
    P.nb = int(std::min<long long>(B, npix - p0));
    chain::k_erpt_corner_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
    launches += 2 + run_wave(s, wS, P, st, stream);
    chain::k_sum_radiance<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st, d_ed);
    A(cudaGetLastError());
  }
  paths += (unsigned long long)npix;
  double hed[3] = {0, 0, 0};
  if (e == cudaSuccess) A(cudaMemcpyAsync(hed, d_ed, sizeof hed, cudaMemcpyDeviceToHost, stream));
  if (e == cudaSuccess) A(cudaStreamSynchronize(stream));
  if (e != cudaSuccess) {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    return cuda_fail(ctx, e, "gbrt_render_erpt ed");
  }
  {
    const double fb = float(hed[0]), fg = float(hed[1]), fr = float(hed[2]);
    double sq = fb * fb;
    sq += fg * fg;
    sq += fr * fr;
    EA.ed = float(std::sqrt(sq) / double(npix * M));
  }
  // Initial samples: their radiance, chain counts and deposit norms.
  P.term_p = 0.f;
  P.rr_pdf = 1.f;
  P.inv_log1mp = 0.f;
  P.pss = EA.z;
  P.pss_stride = int(B);
  for (long long g0 = 0; g0 < n_init && e == cudaSuccess; g0 += B) {
    P.g0 = (unsigned long long)g0;
    P.nb = int(std::min<long long>(B, n_init - g0));
    chain::k_erpt_init_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st, EA);
    launches += 2 + run_wave(s, wP, P, st, stream);
    chain::k_erpt_count<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st, EA);
    A(cudaGetLastError());
  }
  paths += (unsigned long long)n_init;
  chain::k_scan_blocks<<<unsigned(nblk), chain::kScanBlock, 0, stream>>>(EA.count, incl, totals, n_init);
  chain::k_scan_totals<<<1, chain::kScanBlock, 0, stream>>>(totals, int(nblk));
  chain::k_scan_add<<<unsigned(nblk), chain::kScanBlock, 0, stream>>>(incl, totals, n_init);
  launches += 3;
  long long T = 0;
  if (e == cudaSuccess) A(cudaMemcpyAsync(&T, incl + (n_init - 1), sizeof T, cudaMemcpyDeviceToHost, stream));
  if (e == cudaSuccess) A(cudaStreamSynchronize(stream));
  if (e != cudaSuccess) {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    return cuda_fail(ctx, e, "gbrt_render_erpt chains");
  }
  // The chains, in batches of B, one mutation of every chain per wavefront.
  P.pss = EA.z;
  for (long long q0 = 0; q0 < T && e == cudaSuccess; q0 += B) {
    const int nq = int(std::min<long long>(B, T - q0));
    EA.q0 = q0;
    P.g0 = 0;
    P.nb = nq;
    const int grid = (nq + 255) / 256;
    chain::k_erpt_chain_init<<<grid, 256, 0, stream>>>(P, EA, nq);
    A(cudaMemsetAsync(d_iter, 0, sizeof(unsigned long long), stream));
    ++launches;
    unsigned long long per = 0;
    A(replay(stream, M, [&] {
      chain::k_erpt_propose<<<grid, 256, 0, stream>>>(P, st, EA);
      per = 3 + run_wave(s, wP, P, st, stream);
      chain::k_erpt_accept<<<grid, 256, 0, stream>>>(P, st, EA);
      chain::k_tick<<<1, 1, 0, stream>>>(d_iter);
    }));
    launches += per * (unsigned long long)M;
  }
  paths += (unsigned long long)T * unsigned(M);
  unsigned long long acc = 0;
  if (e == cudaSuccess) A(cudaMemcpyAsync(&acc, EA.accepted, sizeof acc, cudaMemcpyDeviceToHost, stream));
  gbrt_status r = chain_finish(s, "gbrt_render_erpt", st, d_sum, d_film, n3, film, ev0, ev1, stream, stats, e);
  if (stats && r == GBRT_OK) {
    stats->paths = paths;
    stats->chains = (unsigned long long)T;
    stats->mutations = (unsigned long long)T * unsigned(M);
    stats->accepted = acc;
    stats->normaliser = EA.ed;
    stats->kernel_launches = launches + 1;
  }
  return r;
}

}  // namespace gbrt

extern "C" {

gbrt_status gbrt_render_mlt(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                            const gbrt_mlt_params* mp, float* film, gbrt_chain_stats* stats) {
  if (!s) return gbrt::fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_mlt: NULL scene");
  gbrt::clear_error(s->ctx);
  if (stats) std::memset(stats, 0, sizeof *stats);
  return gbrt::mlt_impl(s, cam, prm, mp, film, stats);
}

gbrt_status gbrt_render_erpt(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                             const gbrt_erpt_params* ep, float* film, gbrt_chain_stats* stats) {
  if (!s) return gbrt::fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_erpt: NULL scene");
  gbrt::clear_error(s->ctx);
  if (stats) std::memset(stats, 0, sizeof *stats);
  return gbrt::erpt_impl(s, cam, prm, ep, film, stats);
}

}  // extern "C"
