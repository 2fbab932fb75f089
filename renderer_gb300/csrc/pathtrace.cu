// pathtrace.cu — wavefront unidirectional path tracer (gbrt_render*).
//
// GPU restatement of PerPixelRenderer::render (src/perpixelrenderer.cpp:43-101)
// driving UniDiPathTracingIntegrator (src/unidipathtracingintegrator.cpp:34-107)
// over Renderer::createPath (src/renderer.cpp:47-106), in the renderer's own
// estimator ("reference semantics", quirks included).
//
// The renderer first builds a whole path (a list of stored, non-specular
// vertices with their throughputs) and then walks it, adding for every stored
// vertex k either the emission of vertex k+1, when that vertex is an emitter,
// or next-event estimation with light lightIndex[k]. Here the same estimator
// is evaluated in streaming form: the last stored vertex is kept "pending" in
// the path state; when the next stored vertex turns out to be an emitter its
// emission is used for the pending vertex (no shadow ray), otherwise the
// pending vertex gets its shadow ray. At most two shadow rays per path leave
// one shade step (the pending vertex and a new vertex that ends the path).
//
// Per wavefront batch of B paths (path index g = pixel * spp + sample, so a
// warp's camera rays are coherent):
//   raygen      camera rays, path state, extension queue 0
//   D times:    extend  (closest hit, persistent, shared-memory stacks)
//               shade   (materials, emission, NEE; warp-aggregated pushes
//                        into the next extension queue and the shadow queue)
//               shadow  (any hit; unoccluded contributions added to the path)
//   accumulate  per-pixel FP64 sum and sum of squares
// Queue sizes live in device memory, so launch grids never depend on them.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "gbrt_internal.h"
#include "guide_internal.h"
#include "shading.cuh"
#include "traverse.cuh"

namespace gbrt {

namespace cg = cooperative_groups;

struct CamDev {
  float eye[3];
  float u[3], v[3], w[3];
  float l, r, t, b;
  int W, H;
};

struct PTParams {
  CamDev cam;
  unsigned long long seed;
  unsigned long long g0;   // first path index of the batch
  int nb;                  // paths in the batch
  int idx32;               // every path index of the frame fits in 32 bits
  int xs, ys, spp;
  int D;                   // maximum path length
  float rr_pdf;            // Russian-roulette compensation pdf
  float term_p;            // termination probability
  float inv_log1mp;        // 1 / log(1 - term_p), for the geometric draw
  int physical;            // GBRT_SEM_PHYSICAL
  int guided;              // sample non-specular vertices from the guide's mixtures too
  float guide_frac;        // probability of sampling the guide (one-sample MIS)
  int record;              // write training records for the guide
  int guide_depth;         // guide vertices i < guide_depth only (0: all)
  int train_relative;      // training weights relative to the sample's pixel
  int train_product;       // training target BSDF x incident radiance x cos (else radiance x cos)
  const double* film_sum;  // sums of the earlier passes (pixel estimates for the training weights)
  const double* pass_sum;  // sums of the current pass
  double inv_samples;      // 1 / samples per pixel in film_sum + pass_sum
  const float* pss;        // primary samples of the Markov-chain renderers: dim d of slot s at pss[d * pss_stride + s]
  int pss_stride;
  unsigned long long nan_every;  // injected fault: radiance of path indices divisible by this is NaN (0: off)
};

// Where a path's random numbers come from. StreamSrc: the counter-based
// stream of the path's sample index (the per-pixel renderers). PssSrc: a
// stored primary-sample vector per slot (the Markov-chain renderers, whose
// mutations move these numbers). Both use the dimension layout of dim_path /
// dim_light.
struct StreamSrc {
  unsigned long long key;
  __device__ __forceinline__ StreamSrc(const PTParams& P, int slot)
      : key(stream_key(P.seed, P.g0 + (unsigned long long)slot)) {}
  __device__ __forceinline__ float u(unsigned d) const { return stream_u(key, d); }
  __device__ __forceinline__ int index(unsigned d, int n) const { return stream_index(key, d, n); }
};
struct PssSrc {
  const float* p;
  unsigned stride;
  __device__ __forceinline__ PssSrc(const PTParams& P, int slot) : p(P.pss + slot), stride(unsigned(P.pss_stride)) {}
  __device__ __forceinline__ float u(unsigned d) const { return __ldg(p + size_t(d) * stride); }
  // floor(u * n) with the product in float, as the oracle computes it
  __device__ __forceinline__ int index(unsigned d, int n) const { return int(__fmul_rn(u(d), float(n))); }
};

// Path state, structure of arrays indexed by slot (path index - g0).
struct PTState {
  float4* alpha;   // current throughput
  float4* L;       // accumulated radiance
  int4* ctl;       // (i, pathLength, nStored, pending)
  float4* pv_p;    // pending vertex: point, material (int bits)
  float4* pv_n;    // pending vertex: normal, stored index k (int bits)
  float4* pv_d;    // pending vertex: incoming ray direction
  float4* pv_a;    // pending vertex: throughput
  float4* ext[2];  // extension queues: (o, tmin), (d, tmax) per entry
  int* ext_slot[2];
  RawHit* hits;
  int* hit_inst;   // instance of each hit, two-level scenes only (else null)
  float4* sh_ray;  // shadow queue: (o, tmin), (d, tmax)
  float4* sh_c;    // contribution, ignore prim in w (int bits)
  int* sh_slot;
  int* counts;     // [0], [1] extension counts, [2] shadow count
  int ext_cap, sh_cap;  // entries of each extension queue and of the shadow queue (0: not checked)
  unsigned long long* work;   // work counters of the persistent kernels
  unsigned long long* tally;  // [0] extension rays, [1] shadow rays, [2] non-finite samples
  int* err;
  // Path guiding (null when unused).
  float4* gin;     // per extension-queue entry: (point, guided), (normal facing wo, -), (wo, -)
  float4* mix;     // per extension-queue entry: the vertex's mixture (guide::kMixStride float4)
  float4* rec;     // training records, kRecords x kRecComp float4 per slot, record-major
  float4* tsamp;   // training samples, four float4 each
  int* tcount;     // training samples written
  int tcap;        // capacity of tsamp
  int nslots;      // slots allocated (stride of rec)
};

// Training records of the guide: the first kRecords guided vertices of a
// path. Record component c of record r of a slot is rec[(6 r + c) nslots +
// slot]: (point, pdf), (normal, wi.x), (wo, wi.y), (throughput after the
// vertex, wi.z), (radiance of the path when the next vertex was reached),
// (mean throughput before the vertex, -, -, -).
// ctl.z of a guided path: records written (low 4 bits), kRecOpen while the
// last record waits for its radiance snapshot.
constexpr int kRecords = 4;
constexpr int kRecComp = 6;
constexpr int kRecOpen = 0x100;

// Many images in one wavefront (gbrt_render_batch_fused). The jobs' paths
// are numbered one after the other (job j owns global path indices
// [start_j, start_j + total_j)); a wavefront holds global paths [G0, G0 + nb)
// of any number of jobs, and every slot records its job. A job's parameters
// carry g0 = G0 - start_j (mod 2^64), rewritten per wavefront, so that
// g0 + slot is the path's index within its own image, as in a single render.
struct BatchJob {
  PTParams P;
  unsigned long long start, total;  // the job's global path range
  unsigned long long pix0;          // its first pixel in the batch's film and sums
  unsigned long long wlane;         // accumulation lanes of the jobs before it in this wavefront (prefix)
  unsigned long long wnp;           // its pixels in this wavefront
  int group;                        // lanes per pixel in the accumulation: spp rounded up to 2^k, at most 32
};
struct BatchDev {
  const DeviceScene* scenes;        // per job
  BatchJob* jobs;
  const unsigned long long* starts; // per job, start (for the search by path index)
  unsigned short* job_of;           // per slot
  unsigned long long* cursor;       // [0] G0, [1] nb, [2] all paths, [3] accumulation lanes of the wavefront
  double* sum;                      // FP64 sums of all jobs' pixels
  float* film;                      // films of all jobs
  unsigned long long stride;        // global paths between this pipeline's wavefronts
  int n_jobs;
  int B;                            // wavefront capacity
  int shared_sum;                   // several pipelines add into the sums: atomics
};

// The job of global path index g: the last job starting at or before g.
__device__ __forceinline__ int batch_job_of(const BatchDev& bt, unsigned long long g) {
  int lo = 0, hi = bt.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(bt.starts + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------- raygen ----
// Path length: min(3 + Geometric(p), D) (src/renderer.cpp:52-61), from the
// uniform ul; D when p is 0.
__device__ __forceinline__ int ref_path_length(const PTParams& P, float ul) {
  if (!(P.term_p > 0.f)) return P.D;
  int k = 0;
  if (P.term_p < 1.f) {
    // Geometric draw by inversion, floor(log(1 - u) / log(1 - p)). 1 - u is
    // exact in float (u has 24 bits), so the float quotient differs from the
    // double one the CPU oracle uses by a few ulp; only when it falls that
    // close to an integer is it recomputed in double.
    float x = logf(1.f - ul) * P.inv_log1mp;
    float fx = floorf(x);
    if (x - fx < 1e-5f * fmaxf(1.f, x) || fx + 1.f - x < 1e-5f * fmaxf(1.f, x))
      fx = float(floor(log(1.0 - double(ul)) / log(1.0 - double(P.term_p))));
    k = max(int(fx), 0);
  }
  return min(3 + k, P.D);
}

// A new path in slot: unit throughput, no radiance, the camera ray in the
// first extension queue.
__device__ __forceinline__ void start_path(const PTParams& P, const PTState& st, int slot, int plen, float dx,
                                           float dy, float dz) {
  st.alpha[slot] = make_float4(1.f, 1.f, 1.f, 0.f);
  st.L[slot] = make_float4(0.f, 0.f, 0.f, 0.f);
  // ctl.w: reference semantics, "a stored vertex is pending"; physical
  // semantics, "the previous vertex was specular (or the camera)".
  st.ctl[slot] = make_int4(0, plen, 0, P.physical ? 1 : 0);
  st.ext[0][2 * slot] = make_float4(P.cam.eye[0], P.cam.eye[1], P.cam.eye[2], kEps);
  st.ext[0][2 * slot + 1] = make_float4(dx, dy, dz, CUDART_INF_F);
  st.ext_slot[0][slot] = slot;
}

// Camera::getRay (src/camera.cpp:50-58) for the image point (sxp, syp) in
// pixel units: image plane at z = -1 in camera space.
__device__ __forceinline__ void camera_dir(const PTParams& P, float sxp, float syp, float& dx, float& dy, float& dz) {
  float x = P.cam.l + (P.cam.r - P.cam.l) * (sxp + 0.5f) / float(P.cam.W);
  float y = P.cam.t + (P.cam.b - P.cam.t) * (syp + 0.5f) / float(P.cam.H);
  dx = x * P.cam.u[0] + y * P.cam.v[0] - P.cam.w[0];
  dy = x * P.cam.u[1] + y * P.cam.v[1] - P.cam.w[1];
  dz = x * P.cam.u[2] + y * P.cam.v[2] - P.cam.w[2];
}

// The camera ray of the path in slot (path index P.g0 + slot of its image).
__device__ __forceinline__ void raygen_slot(const PTParams& P, const PTState& st, int slot) {
  unsigned long long g = P.g0 + (unsigned long long)slot;
  int pixel, s;
  if (P.idx32) {
    unsigned g32 = unsigned(g);
    pixel = int(g32 / unsigned(P.spp));
    s = int(g32 - unsigned(pixel) * unsigned(P.spp));
  } else {
    pixel = int(g / unsigned(P.spp));
    s = int(g % unsigned(P.spp));
  }
  int px = pixel % P.cam.W, py = pixel / P.cam.W;
  int a = s / P.ys, b = s % P.ys;  // JitteredSampler strata: x outer, y inner
  unsigned long long key = stream_key(P.seed, g);
  float sxp = float(px) + (stream_u(key, 0) + float(a)) / float(P.xs);
  float syp = float(py) + (stream_u(key, 1) + float(b)) / float(P.ys);
  float dx, dy, dz;
  camera_dir(P, sxp, syp, dx, dy, dz);
  // The physical estimator plays Russian roulette per vertex instead.
  const int plen = P.physical ? P.D : ref_path_length(P, stream_u(key, 2));
  start_path(P, st, slot, plen, dx, dy, dz);
}

__global__ void __launch_bounds__(256) k_raygen(PTParams P, PTState st) {
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot == 0) {
    st.counts[0] = P.nb;
    st.work[0] = 0;  // work counter of the first extend
  }
  if (slot >= P.nb) return;
  raygen_slot(P, st, slot);
}

// Adds a warp's traversal counters to two global totals (all lanes call it).
__device__ __forceinline__ void warp_add_counters(TraceCounters c, unsigned long long* nodes,
                                                  unsigned long long* prims) {
  for (int o = 16; o > 0; o >>= 1) {
    c.nodes += __shfl_xor_sync(0xffffffffu, c.nodes, o);
    c.prims += __shfl_xor_sync(0xffffffffu, c.prims, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(nodes, c.nodes);
    atomicAdd(prims, c.prims);
  }
}

// ----------------------------------------------------- extend / shadow ----
// Persistent traversal kernels: each warp takes 32 rays at a time from its
// queue with one atomic and traces them to completion.
//
// Queue protocol (no host-side resets inside a batch): k_raygen sets
// counts[0] and zeroes work[0]; k_extend on queue cur zeroes, before shade and
// shadow run, counts[cur^1] (next extension queue), counts[2] (shadow queue),
// work[cur^1] (next extend) and work[2] (this iteration's shadow pass).
// MS: the scene of each ray is its job's (gbrt_render_batch_fused).
template <bool COUNT, bool WT, int STACK, bool GEN, bool MS>
__device__ __forceinline__ void extend_body(const DeviceScene& S, const PTState& st, int cur, const BatchDev& bt) {
  const int n = st.counts[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    st.tally[0] += (unsigned long long)n;
    st.counts[cur ^ 1] = 0;
    st.counts[2] = 0;
    st.work[cur ^ 1] = 0;
    st.work[2] = 0;
  }
  const float4* rays = st.ext[cur];
  unsigned long long* work = st.work + cur;
  const int lane = threadIdx.x & 31;
  TraceCounters cnt{0, 0};
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned long long)n) break;
    int i = int(base) + lane;
    if (i >= n) continue;
    TRay r = make_tray(rays[2 * i], rays[2 * i + 1]);
    RawHit h;
    int32_t inst = -1;
    if (MS) {
      const DeviceScene& Sj = bt.scenes[bt.job_of[st.ext_slot[cur][i]]];
      h.rec = trace_ray<false, COUNT, WT, STACK, GEN>(Sj, r, -1, h.t, h.u, h.v, st.err, &cnt, &inst);
      st.hits[i] = h;
      if (GEN && st.hit_inst) st.hit_inst[i] = inst;
    } else {
      h.rec = trace_ray<false, COUNT, WT, STACK, GEN>(S, r, -1, h.t, h.u, h.v, st.err, &cnt, &inst);
      st.hits[i] = h;
      if (GEN && S.inst) st.hit_inst[i] = inst;
    }
  }
  if (COUNT) warp_add_counters(cnt, &st.tally[3], &st.tally[4]);
}

template <bool COUNT, bool WT, int STACK, bool GEN>
__global__ void __launch_bounds__(kTraceBlock) k_extend(DeviceScene S, PTState st, int cur) {
  extend_body<COUNT, WT, STACK, GEN, false>(S, st, cur, BatchDev{});
}

template <bool WT, int STACK, bool GEN>
__global__ void __launch_bounds__(kTraceBlock) k_extend_ms(PTState st, int cur, BatchDev bt) {
  extend_body<false, WT, STACK, GEN, true>(bt.scenes[0], st, cur, bt);
}

template <bool COUNT, bool WT, int STACK, bool GEN, bool MS>
__device__ __forceinline__ void shadow_body(const DeviceScene& S, const PTState& st, const BatchDev& bt) {
  const int n = st.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) st.tally[1] += (unsigned long long)n;
  unsigned long long* work = st.work + 2;
  const int lane = threadIdx.x & 31;
  TraceCounters cnt{0, 0};
  for (;;) {
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(work, 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= (unsigned long long)n) break;
    int i = int(base) + lane;
    if (i >= n) continue;
    float4 c = st.sh_c[i];
    TRay r = make_tray(st.sh_ray[2 * i], st.sh_ray[2 * i + 1]);
    float t, u, v;
    const int slot = st.sh_slot[i];
    int32_t rec;
    if (MS) {
      const DeviceScene& Sj = bt.scenes[bt.job_of[slot]];
      rec = trace_ray<true, COUNT, WT, STACK, GEN>(Sj, r, __float_as_int(c.w), t, u, v, st.err, &cnt);
    } else {
      rec = trace_ray<true, COUNT, WT, STACK, GEN>(S, r, __float_as_int(c.w), t, u, v, st.err, &cnt);
    }
    if (rec == -1) {
      float4* L = st.L + slot;
      atomicAdd(&L->x, c.x);
      atomicAdd(&L->y, c.y);
      atomicAdd(&L->z, c.z);
    }
  }
  if (COUNT) warp_add_counters(cnt, &st.tally[5], &st.tally[6]);
}

template <bool COUNT, bool WT, int STACK, bool GEN>
__global__ void __launch_bounds__(kTraceBlock) k_shadow(DeviceScene S, PTState st) {
  shadow_body<COUNT, WT, STACK, GEN, false>(S, st, BatchDev{});
}

template <bool WT, int STACK, bool GEN>
__global__ void __launch_bounds__(kTraceBlock) k_shadow_ms(PTState st, BatchDev bt) {
  shadow_body<false, WT, STACK, GEN, true>(bt.scenes[0], st, bt);
}

// What the error word of a render says (bits kErrStack, kErrIndex).
static std::string err_text(const char* who, int err) {
  std::string m = who;
  if (err & kErrStack) m += ": traversal stack overflow";
  if (err & kErrIndex) m += ": index out of range (checked build)";
  return m;
}

// A persistent grid no larger than a wavefront of `items` needs (each warp
// fetches 32 items at a time; a shade thread takes one): small wavefronts
// then launch a few blocks instead of a full grid that exits at once.
static inline int cap_grid(int full, long long items, int per_block) {
  const long long need = (items + per_block - 1) / per_block;
  return int(std::max<long long>(1, std::min<long long>(full, need)));
}

// -------------------------------------------------------------- shade ----
// Queue push aggregated over the threads of a warp that reach it together
// (one atomic per converged group), so a push can sit inside divergent code
// and its payload need not stay live until a common exit point.
__device__ __forceinline__ int agg_push(int* counter) {
  cg::coalesced_group g = cg::coalesced_threads();
  int base = 0;
  if (g.thread_rank() == 0) base = atomicAdd(counter, int(g.size()));
  return g.shfl(base, 0) + int(g.thread_rank());
}

__device__ __forceinline__ void push_ext(const PTState& st, int nxt, int slot, V3f p, V3f d) {
  int e = agg_push(&st.counts[nxt]);
  if (!in_range(st.ext_cap == 0 || e < st.ext_cap, st.err)) return;
  st.ext[nxt][2 * e] = make_float4(p.x, p.y, p.z, kEps);
  st.ext[nxt][2 * e + 1] = make_float4(d.x, d.y, d.z, CUDART_INF_F);
  st.ext_slot[nxt][e] = slot;
}

__device__ __forceinline__ void load_pending(const PTState& st, int slot, Vertex& pv, V3f& pa, int& k) {
  float4 pp = st.pv_p[slot], pn = st.pv_n[slot], pd = st.pv_d[slot], a = st.pv_a[slot];
  pv.p = v3(pp.x, pp.y, pp.z);
  pv.n = v3(pn.x, pn.y, pn.z);
  pv.d = v3(pd.x, pd.y, pd.z);
  pv.mat = __float_as_int(pp.w);
  pv.tu = pd.w;
  pv.tv = a.w;
  pa = v3(a.x, a.y, a.z);
  k = __float_as_int(pn.w);
}

// Next-event estimation at a stored vertex: UniDiPathTracingIntegrator lines
// 83-99 with Light::getIntensity for light lightIndex[k]. A non-zero
// contribution goes to the shadow queue with its shadow ray.
template <bool EXT, class R>
__device__ __forceinline__ void nee(const DeviceScene& S, const PTParams& P, const PTState& st, int slot,
                                    const R& rs, const Vertex& vx, V3f alpha, int k) {
  if (S.n_lights <= 0 || vx.mat < 0) return;
  unsigned dl = dim_light(P.D, k);
  float lx = rs.u(dl), ly = rs.u(dl + 1);
  int li = min(rs.index(dl + 2, S.n_lights), S.n_lights - 1);  // floor(u * n)
  const DevLight& Lt = S.lights[li];
  V3f dir, Le, sd;
  float stmax;
  int ignore = -1;
  if (Lt.type == GBRT_LIGHT_AREA) {
    V3f lp = ld3(Lt.origin) + lx * ld3(Lt.u) + ly * ld3(Lt.v);
    dir = vx.p - lp;
    Le = area_intensity(Lt, dir);
    sd = -normalize(dir);
    stmax = len(dir) - kEps;
    ignore = Lt.prim;
  } else if (Lt.type == GBRT_LIGHT_POINT || Lt.type == GBRT_LIGHT_CONE) {
    dir = vx.p - ld3(Lt.origin);
    float inv = 1.f / len2(dir);
    Le = v3(Lt.intensity[0] * inv, Lt.intensity[1] * inv, Lt.intensity[2] * inv);
    // ConeLight::getIntensity (src/conelight.cpp:31-45): only inside the cone.
    if (Lt.type == GBRT_LIGHT_CONE && !(acosf(dot(normalize(dir), ld3(Lt.nhat))) <= Lt.v[0])) return;
    sd = -normalize(dir);
    stmax = len(dir) - kEps;
  } else if (Lt.type == GBRT_LIGHT_ENV && S.env_light >= 0) {
    float pdf;
    V3f s = cosine_power_dir(vx.n, lx, ly, 1.f, pdf);
    dir = -s;
    V3f e = env_get(S, dir);
    float ip = 1.f / pdf;
    Le = v3(e.x * ip, e.y * ip, e.z * ip);
    // Ray(at, -s, -inf, -EPSILON) of the renderer == Ray(at, s, EPSILON, inf).
    sd = s;
    stmax = CUDART_INF_F;
  } else {
    return;  // BlackLight
  }
  if (is_zero(Le)) return;
  V3f f = brdf_eval<EXT>(S, vx, dir);
  float inCos = dot(-normalize(dir), vx.n);
  float outCos = dot(-normalize(vx.d), vx.n);
  if (signum(inCos) != signum(outCos)) return;
  float ac = fabsf(inCos);
  V3f c = v3(alpha.x * f.x * Le.x * ac, alpha.y * f.y * Le.y * ac, alpha.z * f.z * Le.z * ac);
  if (is_zero(c)) return;
  int e = agg_push(&st.counts[2]);
  if (!in_range(st.sh_cap == 0 || e < st.sh_cap, st.err)) return;
  st.sh_ray[2 * e] = make_float4(vx.p.x, vx.p.y, vx.p.z, kEps);
  st.sh_ray[2 * e + 1] = make_float4(sd.x, sd.y, sd.z, stmax);
  st.sh_c[e] = make_float4(c.x, c.y, c.z, __int_as_float(ignore));
  st.sh_slot[e] = slot;
}

// Shading of the hit at the head of one path: the body of the loop of
// Renderer::createPath (src/renderer.cpp:73-104) for one iteration, with the
// stored-vertex bookkeeping of UniDiPathTracingIntegrator::integrate(path)
// done in streaming form (see the file comment).
template <bool EXT, class R, bool MS>
__device__ __forceinline__ void shade_body(const DeviceScene& S0, const PTParams& P0, const PTState& st, int cur,
                                           const BatchDev& bt) {
  const int n = st.counts[cur];
  const int nxt = cur ^ 1;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int slot = st.ext_slot[cur][q];
    const int job = MS ? int(bt.job_of[slot]) : 0;
    const DeviceScene& S = MS ? bt.scenes[job] : S0;
    const PTParams& P = MS ? bt.jobs[job].P : P0;
    const RawHit h = st.hits[q];
    if (!in_range(h.rec < S.n_recs && h.rec >= -1 - S.n_planes, st.err)) continue;
    const float4 ro = st.ext[cur][2 * q], rd = st.ext[cur][2 * q + 1];
    int4 c = st.ctl[slot];
    int i = c.x, plen = c.y, nst = c.z;
    bool pend = c.w != 0;
    const R rs(P, slot);
    const V3f d = v3(rd.x, rd.y, rd.z);
    const bool envHit = h.rec == -1 && S.env_light >= 0 && isinf(rd.w) && rd.w > 0.f;
    if (h.rec == -1 && !envHit) {
      // The path leaves the scene: the last stored vertex gets NEE (line 85).
      if (pend) {
        Vertex pv; V3f pa; int k;
        load_pending(st, slot, pv, pa, k);
        nee<EXT>(S, P, st, slot, rs, pv, pa, k);
        st.ctl[slot] = make_int4(i, plen, nst, 0);
      }
      continue;
    }
    Vertex vx;
    vx.d = d;
    vx.mat = -1;
    vx.tu = 0.f;
    vx.tv = 0.f;
    int light = -1;
    if (envHit) {
      light = S.env_light;
      vx.p = normalize(d);  // point at infinity (w = 0)
      vx.n = -vx.p;
    } else {
      vx.p = v3(ro.x, ro.y, ro.z) + h.t * d;
      if (h.rec >= 0) {
        const int4 m = __ldg(&S.meta[h.rec]);
        const float4* rp = S.recs + 3 * int64_t(h.rec);
        const float4 a = __ldg(rp);
        const int kind = __float_as_int(a.w);
        vx.mat = m.y;
        light = m.w;
        if (!in_range(light < S.n_lights && vx.mat < S.n_materials, st.err)) continue;
        if (EXT && S.tri_uv) hit_texcoords(S, h.rec, h.u, h.v, vx.p, vx.tu, vx.tv);
        if (kind == kRecTriangle) {
          if (m.z >= 0) {
            const float* nn = S.tri_nrm + 12 * int64_t(m.z);
            float w0 = 1.f - h.u - h.v;
            vx.n = normalize(w0 * ld3(nn) + h.u * ld3(nn + 3) + h.v * ld3(nn + 6));
          } else {
            const float4 b = __ldg(rp + 1), cc = __ldg(rp + 2);
            V3f p1 = v3(a.x, a.y, a.z), p2 = v3(b.x, b.y, b.z), p3 = v3(cc.x, cc.y, cc.z);
            vx.n = normalize(cross(p1 - p2, p1 - p3));
          }
        } else if (kind == kRecSphere) {
          vx.n = normalize(vx.p - v3(a.x, a.y, a.z));
        } else if (EXT && kind == kRecCSG) {
          csg_surface(S, __float_as_int(h.u), v3(ro.x, ro.y, ro.z), d, vx.p, vx.n, vx.mat, vx.tu, vx.tv);
        } else {
          vx.n = ld3(S.lights[light].nhat);
        }
        if (EXT && S.inst) {
          const int in = st.hit_inst[q];
          if (in >= 0) vx.n = instance_normal(S, in, vx.n);
        }
      } else {
        const float4 pl = __ldg(&S.planes[-2 - h.rec]);
        vx.n = normalize(v3(pl.x, pl.y, pl.z));
        vx.mat = S.plane_meta[-2 - h.rec].y;
      }
    }
    if (light >= 0) {
      // Emitter. Its own next-event term is zero (Material::brdf of a light
      // is zero), so only its emission matters; the path ends here.
      V3f e = envHit ? env_get(S, vx.p) : area_intensity(S.lights[light], -d);
      float4 L4 = st.L[slot];
      if (nst == 0) {
        // The first stored vertex is an emitter: its emission is the sample.
        L4.x = e.x; L4.y = e.y; L4.z = e.z;
      } else if (pend) {
        // The pending vertex sees this emitter (lines 70-81).
        Vertex pv; V3f pa; int k;
        load_pending(st, slot, pv, pa, k);
        V3f dir = envHit ? -vx.p : pv.p - vx.p;
        V3f f = brdf_eval<EXT>(S, pv, dir);
        float inCos = dot(-normalize(dir), pv.n);
        float outCos = dot(-normalize(pv.d), pv.n);
        if (signum(inCos) == signum(outCos)) {
          float ac = fabsf(inCos);
          L4.x += pa.x * f.x * e.x * ac;
          L4.y += pa.y * f.y * e.y * ac;
          L4.z += pa.z * f.z * e.z * ac;
        }
      }
      st.L[slot] = L4;
      st.ctl[slot] = make_int4(i, plen, nst, 0);
      continue;
    }
    float pdf;
    V3f f;
    const V3f out = out_direction<EXT>(S, vx, rs.u(dim_path(i)), rs.u(dim_path(i) + 1), pdf, f);
    if (mat_specular(S.materials, vx.mat)) {
      // Specular vertices are not stored (lines 87-91).
      if (i == plen - 1 && plen < P.D) plen++;
      i++;
      if (i < plen) {
        push_ext(st, nxt, slot, vx.p, out);
      } else if (pend) {
        Vertex pv; V3f pa; int k;
        load_pending(st, slot, pv, pa, k);
        nee<EXT>(S, P, st, slot, rs, pv, pa, k);
        pend = false;
      }
      st.ctl[slot] = make_int4(i, plen, nst, pend ? 1 : 0);
      continue;
    }
    // Stored, non-specular vertex k = nst (lines 92-102): the previous pending
    // vertex is now known not to be followed by an emitter.
    if (pend) {
      Vertex pv; V3f pa; int k;
      load_pending(st, slot, pv, pa, k);
      nee<EXT>(S, P, st, slot, rs, pv, pa, k);
    }
    const float4 a4 = st.alpha[slot];
    const V3f alpha = v3(a4.x, a4.y, a4.z);
    const int k = nst++;
    bool ends = pdf == 0.f || is_zero(alpha);
    V3f na = alpha;
    if (!ends) {
      float sc = fabsf(dot(normalize(out), vx.n)) / pdf;
      na = v3(alpha.x * f.x * sc, alpha.y * f.y * sc, alpha.z * f.z * sc);
      if (i > 3) {
        float ir = 1.f / P.rr_pdf;
        na = v3(na.x * ir, na.y * ir, na.z * ir);
      }
      i++;
      ends = i >= plen;
    }
    if (ends) {
      // This vertex is the last stored one: next-event estimation now.
      nee<EXT>(S, P, st, slot, rs, vx, alpha, k);
      st.ctl[slot] = make_int4(i, plen, nst, 0);
    } else {
      st.pv_p[slot] = make_float4(vx.p.x, vx.p.y, vx.p.z, __int_as_float(vx.mat));
      st.pv_n[slot] = make_float4(vx.n.x, vx.n.y, vx.n.z, __int_as_float(k));
      st.pv_d[slot] = make_float4(d.x, d.y, d.z, vx.tu);
      st.pv_a[slot] = make_float4(alpha.x, alpha.y, alpha.z, vx.tv);
      st.alpha[slot] = make_float4(na.x, na.y, na.z, 0.f);
      st.ctl[slot] = make_int4(i, plen, nst, 1);
      push_ext(st, nxt, slot, vx.p, out);
    }
  }
}

template <bool EXT, class R>
__global__ void __launch_bounds__(256, 4) k_shade(DeviceScene S, PTParams P, PTState st, int cur) {
  shade_body<EXT, R, false>(S, P, st, cur, BatchDev{});
}

template <bool EXT>
__global__ void __launch_bounds__(256, 4) k_shade_ms(PTState st, int cur, BatchDev bt) {
  shade_body<EXT, StreamSrc, true>(bt.scenes[0], bt.jobs[0].P, st, cur, bt);
}

// ------------------------------------------------------ shade, physical ----
// GBRT_SEM_PHYSICAL: next-event estimation with one uniformly chosen light
// (weighted by the light count), emission on BSDF-sampled hits, both combined
// by the power heuristic; Russian roulette with survival 1 - p from the
// fourth vertex on. Path state: alpha.xyz throughput, alpha.w the pdf of the
// last sampled direction, ctl = (vertex index, -, guide records, last vertex
// specular).
//
// With guiding, a non-specular vertex samples its direction from the
// vertex's vMF mixture with probability guide_frac and from the BSDF
// otherwise (one-sample MIS: the pdf of either choice is the mixture
// guide_frac q + (1 - guide_frac) p_bsdf, used in the throughput and in both
// power heuristics).
__device__ __forceinline__ void nee_phys(const DeviceScene& S, const PTState& st, int slot, unsigned long long key,
                                         unsigned base, const PhysBsdf& b, V3f x, V3f n, V3f wo, V3f alpha,
                                         const float4* M, float frac) {
  const int nL = S.n_lights;
  const float pChoose = 1.f / float(nL);
  const int li = min(stream_index(key, base + 3, nL), nL - 1);
  const DevLight& Lt = S.lights[li];
  const float lx = stream_u(key, base + 4), ly = stream_u(key, base + 5);
  V3f wi, Le;
  float dist, pl;
  bool delta = false;
  int ignore = -1;
  if (Lt.type == GBRT_LIGHT_AREA) {
    V3f y = ld3(Lt.origin) + lx * ld3(Lt.u) + ly * ld3(Lt.v);
    V3f d = y - x;
    dist = len(d);
    wi = normalize(d);
    float cl = dot(-wi, ld3(Lt.nhat));
    if (!(cl > 0.f)) return;
    Le = ld3(Lt.intensity);
    pl = pChoose * dist * dist / (cl * Lt.normal_len);
    ignore = Lt.prim;
  } else if (Lt.type == GBRT_LIGHT_POINT || Lt.type == GBRT_LIGHT_CONE) {
    V3f d = ld3(Lt.origin) - x;
    dist = len(d);
    wi = normalize(d);
    if (Lt.type == GBRT_LIGHT_CONE && !(acosf(dot(-wi, ld3(Lt.nhat))) <= Lt.v[0])) return;
    float inv = 1.f / len2(d);
    Le = inv * ld3(Lt.intensity);
    pl = pChoose;
    delta = true;
  } else if (Lt.type == GBRT_LIGHT_ENV && S.env_light >= 0) {
    // In proportion to the map's luminance (or uniformly over the sphere
    // without the tables).
    float pe = 0.25f * kInvPi;
    if (S.env_marg) {
      if (!env_sample(S, lx, ly, wi, pe)) return;
    } else {
      wi = uniform_sphere(lx, ly);
    }
    dist = CUDART_INF_F;
    Le = env_get(S, wi);
    pl = pChoose * pe;
  } else {
    return;
  }
  if (is_zero(Le)) return;
  float pb;
  V3f f = phys_eval(b, n, wo, wi, pb);
  if (is_zero(f)) return;
  if (M) pb = frac * guide::mixture_pdf(M, wi.x, wi.y, wi.z) + (1.f - frac) * pb;
  float w = delta ? 1.f : power_heuristic(pl, pb);
  float sc = fabsf(dot(n, wi)) * w / pl;
  V3f c = v3(alpha.x * f.x * Le.x * sc, alpha.y * f.y * Le.y * sc, alpha.z * f.z * Le.z * sc);
  if (is_zero(c)) return;
  int e = agg_push(&st.counts[2]);
  if (!in_range(st.sh_cap == 0 || e < st.sh_cap, st.err)) return;
  st.sh_ray[2 * e] = make_float4(x.x, x.y, x.z, kEps);
  st.sh_ray[2 * e + 1] = make_float4(wi.x, wi.y, wi.z, isinf(dist) ? CUDART_INF_F : dist - kEps);
  st.sh_c[e] = make_float4(c.x, c.y, c.z, __int_as_float(ignore));
  st.sh_slot[e] = slot;
}

// Normal (unflipped), material and texture coordinates of a surface hit that
// is not an emitter; o, d: the ray.
template <bool EXT>
__device__ __forceinline__ void surface_normal(const DeviceScene& S, const RawHit& h, int inst, V3f o, V3f d, V3f x,
                                               V3f& nrm, int& mat, float& tu, float& tv) {
  tu = 0.f;
  tv = 0.f;
  if (h.rec >= 0) {
    const int4 m = __ldg(&S.meta[h.rec]);
    const float4* rp = S.recs + 3 * int64_t(h.rec);
    const float4 a = __ldg(rp);
    const int kind = __float_as_int(a.w);
    mat = m.y;
    if (kind == kRecTriangle) {
      if (m.z >= 0) {
        const float* nn = S.tri_nrm + 12 * int64_t(m.z);
        float w0 = 1.f - h.u - h.v;
        nrm = normalize(w0 * ld3(nn) + h.u * ld3(nn + 3) + h.v * ld3(nn + 6));
      } else {
        const float4 b = __ldg(rp + 1), cc = __ldg(rp + 2);
        V3f p1 = v3(a.x, a.y, a.z), p2 = v3(b.x, b.y, b.z), p3 = v3(cc.x, cc.y, cc.z);
        nrm = normalize(cross(p1 - p2, p1 - p3));
      }
    } else if (EXT && kind == kRecCSG) {
      csg_surface(S, __float_as_int(h.u), o, d, x, nrm, mat, tu, tv);
      return;
    } else {
      nrm = normalize(x - v3(a.x, a.y, a.z));  // sphere
    }
    if (EXT && inst >= 0) nrm = instance_normal(S, inst, nrm);
    if (EXT && S.tri_uv) hit_texcoords(S, h.rec, h.u, h.v, x, tu, tv);
  } else {
    const float4 pl = __ldg(&S.planes[-2 - h.rec]);
    nrm = normalize(v3(pl.x, pl.y, pl.z));
    mat = S.plane_meta[-2 - h.rec].y;
  }
}

template <bool GUIDED, bool EXT, bool MS>
__device__ __forceinline__ void shade_phys_body(const DeviceScene& S0, const PTParams& P0, const PTState& st,
                                                int cur, const BatchDev& bt) {
  const int n = st.counts[cur];
  const int nxt = cur ^ 1;
  const float pChoose0 = MS ? 0.f : (S0.n_lights > 0 ? 1.f / float(S0.n_lights) : 0.f);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int slot = st.ext_slot[cur][q];
    const int job = MS ? int(bt.job_of[slot]) : 0;
    const DeviceScene& S = MS ? bt.scenes[job] : S0;
    const PTParams& P = MS ? bt.jobs[job].P : P0;
    const float pChoose = MS ? (S.n_lights > 0 ? 1.f / float(S.n_lights) : 0.f) : pChoose0;
    const RawHit h = st.hits[q];
    if (!in_range(h.rec < S.n_recs && h.rec >= -1 - S.n_planes, st.err)) continue;
    const float4 ro = st.ext[cur][2 * q], rd = st.ext[cur][2 * q + 1];
    int4 c = st.ctl[slot];
    const int i = c.x;
    if (GUIDED && P.record && (c.z & kRecOpen)) {
      // The radiance the path had gathered before this vertex: the rest of
      // the path is what the last recorded direction brought in.
      st.rec[size_t(kRecComp * ((c.z & 15) - 1) + 4) * st.nslots + slot] = st.L[slot];
      c.z &= ~kRecOpen;
    }
    const bool prevSpec = c.w != 0;
    const float4 a4 = st.alpha[slot];
    const V3f alpha = v3(a4.x, a4.y, a4.z);
    const float prevPdf = a4.w;
    const V3f d = v3(rd.x, rd.y, rd.z);
    const bool envHit = h.rec == -1 && S.env_light >= 0 && isinf(rd.w) && rd.w > 0.f;
    if (h.rec == -1 && !envHit) continue;
    if (envHit) {
      V3f dn = normalize(d);
      V3f Le = env_get(S, dn);
      float w = prevSpec ? 1.f : power_heuristic(prevPdf, pChoose * (S.env_marg ? env_pdf(S, dn) : 0.25f * kInvPi));
      float4 L4 = st.L[slot];
      L4.x += alpha.x * Le.x * w; L4.y += alpha.y * Le.y * w; L4.z += alpha.z * Le.z * w;
      st.L[slot] = L4;
      continue;
    }
    const V3f x = v3(ro.x, ro.y, ro.z) + h.t * d;
    if (h.rec >= 0) {
      const int lt = __ldg(&S.meta[h.rec]).w;
      if (!in_range(lt < S.n_lights, st.err)) continue;
      if (lt >= 0) {
        // An area light: emission on its front side (AreaLight is one-sided).
        const DevLight& Lt = S.lights[lt];
        float dl = len(d);
        float cl = dot(-(1.f / dl) * d, ld3(Lt.nhat));
        if (cl > 0.f) {
          float w = 1.f;
          if (!prevSpec) {
            float dist = h.t * dl;
            w = power_heuristic(prevPdf, pChoose * dist * dist / (cl * Lt.normal_len));
          }
          float4 L4 = st.L[slot];
          L4.x += alpha.x * Lt.intensity[0] * w;
          L4.y += alpha.y * Lt.intensity[1] * w;
          L4.z += alpha.z * Lt.intensity[2] * w;
          st.L[slot] = L4;
        }
        continue;
      }
    }
    V3f nrm;
    int mat = -1;
    float tu, tv;
    surface_normal<EXT>(S, h, (EXT && S.inst) ? st.hit_inst[q] : -1, v3(ro.x, ro.y, ro.z), d, x, nrm, mat, tu, tv);
    const PhysBsdf b = phys_bsdf<EXT>(S, mat, tu, tv);
    if (b.kind <= 0) continue;
    const unsigned long long key = stream_key(P.seed, P.g0 + (unsigned long long)slot);
    const unsigned base = dim_phys(i);
    const V3f wo = -normalize(d);
    const bool flipped = dot(nrm, wo) < 0.f;
    if (flipped) nrm = -nrm;
    const bool depthOk = P.guide_depth == 0 || i < P.guide_depth;
    const bool guideHere = GUIDED && P.guided && depthOk && b.kind >= 1 && b.kind <= 3;
    const float4* M = guideHere ? st.mix + guide::kMixStride * size_t(q) : nullptr;
    if (b.kind <= 3 && S.n_lights > 0) nee_phys(S, st, slot, key, base, b, x, nrm, wo, alpha, M, P.guide_frac);
    V3f wi, wgt;
    float pdf;
    bool spec;
    const float u0 = stream_u(key, base), u1 = stream_u(key, base + 1), u2 = stream_u(key, base + 2);
    if (guideHere) {
      if (stream_u(key, base + 7) < P.guide_frac) {
        guide::mixture_sample(M, u0, u1, u2, wi.x, wi.y, wi.z);
      } else if (!phys_sample(b, nrm, wo, flipped, u0, u1, u2, wi, wgt, pdf, spec)) {
        continue;
      }
      float pb;
      V3f f = phys_eval(b, nrm, wo, wi, pb);
      pdf = P.guide_frac * guide::mixture_pdf(M, wi.x, wi.y, wi.z) + (1.f - P.guide_frac) * pb;
      if (is_zero(f) || !(pdf > 0.f)) continue;
      wgt = (dot(nrm, wi) / pdf) * f;
      spec = false;
    } else if (!phys_sample(b, nrm, wo, flipped, u0, u1, u2, wi, wgt, pdf, spec)) {
      continue;
    }
    V3f na = mulc(alpha, wgt);
    if (i + 1 >= 3 && P.term_p > 0.f) {
      if (stream_u(key, base + 6) < P.term_p) continue;
      na = (1.f / (1.f - P.term_p)) * na;
    }
    if (i + 1 >= P.D) continue;
    int z = 0;
    if (GUIDED) {
      z = c.z;
      if (P.record && depthOk && b.kind >= 1 && b.kind <= 3 && (z & 15) < kRecords) {
        const size_t r = size_t(kRecComp * (z & 15)) * st.nslots + slot;
        const size_t ns = size_t(st.nslots);
        st.rec[r] = make_float4(x.x, x.y, x.z, pdf);
        st.rec[r + ns] = make_float4(nrm.x, nrm.y, nrm.z, wi.x);
        st.rec[r + 2 * ns] = make_float4(wo.x, wo.y, wo.z, wi.y);
        st.rec[r + 3 * ns] = make_float4(na.x, na.y, na.z, wi.z);
        st.rec[r + 5 * ns] = make_float4((alpha.x + alpha.y + alpha.z) * (1.f / 3.f), alpha.x, alpha.y, alpha.z);
        z = ((z & 15) + 1) | kRecOpen;
      }
    }
    st.alpha[slot] = make_float4(na.x, na.y, na.z, pdf);
    st.ctl[slot] = make_int4(i + 1, c.y, z, spec ? 1 : 0);
    push_ext(st, nxt, slot, x, wi);
  }
}

template <bool GUIDED, bool EXT>
__global__ void __launch_bounds__(256, 4) k_shade_phys(DeviceScene S, PTParams P, PTState st, int cur) {
  shade_phys_body<GUIDED, EXT, false>(S, P, st, cur, BatchDev{});
}

template <bool EXT>
__global__ void __launch_bounds__(256, 4) k_shade_phys_ms(PTState st, int cur, BatchDev bt) {
  shade_phys_body<false, EXT, true>(bt.scenes[0], bt.jobs[0].P, st, cur, bt);
}

// ------------------------------------------------------------ guiding ----
// Network inputs of the current extension queue: a surface vertex with a
// non-specular BSDF gets (point, 1), (normal facing wo), (wo); everything
// else a neutral row that the guided shade ignores.
__global__ void __launch_bounds__(256) k_guide_prep(DeviceScene S, PTState st, int cur) {
  const int n = st.counts[cur];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&st.tally[7], (unsigned long long)n);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const RawHit h = st.hits[q];
    float4 r0 = make_float4(0.f, 0.f, 0.f, 0.f), r1 = make_float4(0.f, 0.f, 1.f, 0.f), r2 = r1;
    if (h.rec != -1 && !(h.rec >= 0 && __ldg(&S.meta[h.rec]).w >= 0)) {
      const float4 ro = st.ext[cur][2 * q], rd = st.ext[cur][2 * q + 1];
      const V3f d = v3(rd.x, rd.y, rd.z);
      const V3f x = v3(ro.x, ro.y, ro.z) + h.t * d;
      V3f nrm;
      int mat = -1;
      float tu, tv;
      surface_normal<true>(S, h, S.inst ? st.hit_inst[q] : -1, v3(ro.x, ro.y, ro.z), d, x, nrm, mat, tu, tv);
      const PhysBsdf b = phys_bsdf<true>(S, mat, tu, tv);
      if (b.kind >= 1 && b.kind <= 3) {
        const V3f wo = -normalize(d);
        if (dot(nrm, wo) < 0.f) nrm = -nrm;
        r0 = make_float4(x.x, x.y, x.z, 1.f);
        r1 = make_float4(nrm.x, nrm.y, nrm.z, 0.f);
        r2 = make_float4(wo.x, wo.y, wo.z, 0.f);
      }
    }
    st.gin[3 * size_t(q)] = r0;
    st.gin[3 * size_t(q) + 1] = r1;
    st.gin[3 * size_t(q) + 2] = r2;
  }
}

// Training samples from the records of a finished batch. The radiance that
// arrived along a recorded direction is what the path gathered after the
// record's snapshot, divided by the throughput up to that direction; the
// target is its mean over the channels times |cos| at the vertex, and the
// sample weight target / pdf (pdf: the density the direction was drawn
// from). With GBRT_GUIDE_PRODUCT the target is the BSDF times that radiance
// times |cos|: the path's gain after the vertex over its throughput before
// it (per channel) is already f Li |cos| / pdf, the sample weight.
// With GBRT_GUIDE_PIXEL_RELATIVE the weight is also scaled to the
// sample's share of its pixel: times the throughput from the camera to the
// vertex, over sqrt(p^2 + 0.01) with p the pixel's current estimate (the
// denominator of relMSE), so that dim regions weigh as much as bright ones.
__global__ void __launch_bounds__(256) k_guide_collect(PTParams P, PTState st) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if (slot >= P.nb) return;
  const int nrec = st.ctl[slot].z & 15;
  if (nrec == 0) return;
  const float4 L = st.L[slot];
  const size_t ns = size_t(st.nslots);
  const unsigned long long pix = (P.g0 + (unsigned long long)slot) / unsigned(P.spp);
  const double* ps = P.film_sum + 3 * pix;
  const double* pc = P.pass_sum + 3 * pix;
  const float pl = float((ps[0] + ps[1] + ps[2] + pc[0] + pc[1] + pc[2]) * (1.0 / 3.0) * P.inv_samples);
  const float inv_pix = rsqrtf(pl * pl + 0.01f);
  for (int r = 0; r < nrec; ++r) {
    const size_t b = size_t(kRecComp * r) * ns + slot;
    const float4 r0 = st.rec[b], r1 = st.rec[b + ns], r2 = st.rec[b + 2 * ns], r3 = st.rec[b + 3 * ns],
                 sn = st.rec[b + 4 * ns], r5 = st.rec[b + 5 * ns];
    float w;
    if (P.train_product) {
      // (gathered after the vertex) / (throughput up to it) = f Li cos / pdf
      float lr = 0.f;
      if (r5.y > 0.f) lr += (L.x - sn.x) / r5.y;
      if (r5.z > 0.f) lr += (L.y - sn.y) / r5.z;
      if (r5.w > 0.f) lr += (L.z - sn.z) / r5.w;
      w = lr * (1.f / 3.f);
    } else {
      float li = 0.f;
      if (r3.x > 0.f) li += (L.x - sn.x) / r3.x;
      if (r3.y > 0.f) li += (L.y - sn.y) / r3.y;
      if (r3.z > 0.f) li += (L.z - sn.z) / r3.z;
      const float cosi = fabsf(r1.x * r1.w + r1.y * r2.w + r1.z * r3.w);
      w = (li * (1.f / 3.f)) * cosi / r0.w;
    }
    if (P.train_relative) w *= r5.x * inv_pix;
    if (!(w > 0.f) || !isfinite(w)) continue;
    const int e = agg_push(st.tcount);
    if (e >= st.tcap) continue;
    st.tsamp[4 * size_t(e)] = make_float4(r0.x, r0.y, r0.z, w);
    st.tsamp[4 * size_t(e) + 1] = make_float4(r1.x, r1.y, r1.z, 0.f);
    st.tsamp[4 * size_t(e) + 2] = make_float4(r2.x, r2.y, r2.z, 0.f);
    st.tsamp[4 * size_t(e) + 3] = make_float4(r1.w, r2.w, r3.w, 0.f);
  }
}

// --------------------------------------------------------- accumulate ----
// Float-float running sum (Knuth's TwoSum: every addition's rounding error is
// carried in lo), so that a batch's samples of a pixel are summed to about
// 2^-48 relative, the accuracy of an FP64 sum, with FP32 operations only: the
// GB300's FP64 pipe runs at a small fraction of its FP32 rate, and one FP64
// conversion and addition per sample and channel was most of the
// accumulation's time. Each pixel's float-float sums are added into the FP64
// pixel sums once per batch. Squares enter as exact product pairs (fmaf).
struct FSum {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    const float s = hi + x;
    const float bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
  }
  __device__ __forceinline__ void add_square(float x) {
    const float p = x * x;
    add(p);
    lo += fmaf(x, x, -p);
  }
  __device__ __forceinline__ void merge(float h, float l) {
    add(h);
    lo += l;
  }
  __device__ __forceinline__ void shfl_merge(int offset, int width = 32) {
    const float h = __shfl_down_sync(0xffffffffu, hi, offset, width);
    const float l = __shfl_down_sync(0xffffffffu, lo, offset, width);
    merge(h, l);
  }
  __device__ __forceinline__ double value() const { return double(hi) + double(lo); }
};

// One thread per pixel touched by the batch; samples of a pixel are
// contiguous slots. Non-finite samples are counted and dropped.
__global__ void __launch_bounds__(256) k_accumulate(PTParams P, PTState st, double* sum, double* sumsq) {
  unsigned long long p0 = P.g0 / unsigned(P.spp);
  unsigned long long p1 = (P.g0 + unsigned(P.nb) - 1) / unsigned(P.spp);
  unsigned long long p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p > p1) return;
  unsigned long long gb = max(P.g0, p * unsigned(P.spp));
  unsigned long long ge = min(P.g0 + unsigned(P.nb), (p + 1) * unsigned(P.spp));
  FSum s0, s1, s2, q0, q1, q2;
  unsigned long long bad = 0;
  for (unsigned long long g = gb; g < ge; ++g) {
    float4 L = st.L[g - P.g0];
    if (P.nan_every && g % P.nan_every == 0) L.x = CUDART_NAN_F;
    if (!isfinite(L.x) || !isfinite(L.y) || !isfinite(L.z)) { ++bad; continue; }
    s0.add(L.x); s1.add(L.y); s2.add(L.z);
    if (sumsq) { q0.add_square(L.x); q1.add_square(L.y); q2.add_square(L.z); }
  }
  if (bad) atomicAdd(&st.tally[2], bad);
  size_t o = size_t(p) * 3;
  sum[o] += s0.value(); sum[o + 1] += s1.value(); sum[o + 2] += s2.value();
  if (sumsq) { sumsq[o] += q0.value(); sumsq[o + 1] += q1.value(); sumsq[o + 2] += q2.value(); }
}

// The same with one warp per pixel, for many samples per pixel.
__global__ void __launch_bounds__(256) k_accumulate_warp(PTParams P, PTState st, double* sum, double* sumsq) {
  const unsigned long long p0 = P.g0 / unsigned(P.spp);
  const unsigned long long p1 = (P.g0 + unsigned(P.nb) - 1) / unsigned(P.spp);
  const unsigned long long p = p0 + (blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (p > p1) return;  // whole warps leave together
  const unsigned long long gb = max(P.g0, p * unsigned(P.spp));
  const unsigned long long ge = min(P.g0 + unsigned(P.nb), (p + 1) * unsigned(P.spp));
  FSum s0, s1, s2, q0, q1, q2;
  unsigned long long bad = 0;
  for (unsigned long long g = gb + lane; g < ge; g += 32) {
    float4 L = st.L[g - P.g0];
    if (P.nan_every && g % P.nan_every == 0) L.x = CUDART_NAN_F;
    if (!isfinite(L.x) || !isfinite(L.y) || !isfinite(L.z)) { ++bad; continue; }
    s0.add(L.x); s1.add(L.y); s2.add(L.z);
    if (sumsq) { q0.add_square(L.x); q1.add_square(L.y); q2.add_square(L.z); }
  }
  for (int o = 16; o > 0; o >>= 1) {
    s0.shfl_merge(o); s1.shfl_merge(o); s2.shfl_merge(o);
    if (sumsq) { q0.shfl_merge(o); q1.shfl_merge(o); q2.shfl_merge(o); }
    bad += __shfl_down_sync(0xffffffffu, bad, o);
  }
  if (lane == 0) {
    if (bad) atomicAdd(&st.tally[2], bad);
    size_t o = size_t(p) * 3;
    sum[o] += s0.value(); sum[o + 1] += s1.value(); sum[o + 2] += s2.value();
    if (sumsq) { sumsq[o] += q0.value(); sumsq[o + 1] += q1.value(); sumsq[o + 2] += q2.value(); }
  }
}

// Accumulation of a batch: a thread per pixel for few samples per pixel, a
// warp per pixel for many.
static void launch_accumulate(const PTParams& P, const PTState& st, double* sum, double* sumsq, cudaStream_t stream) {
  const unsigned long long p0 = P.g0 / unsigned(P.spp), p1 = (P.g0 + unsigned(P.nb) - 1) / unsigned(P.spp);
  const unsigned long long np = p1 - p0 + 1;
  if (P.spp >= 256)
    k_accumulate_warp<<<unsigned((np * 32 + 255) / 256), 256, 0, stream>>>(P, st, sum, sumsq);
  else
    k_accumulate<<<unsigned((np + 255) / 256), 256, 0, stream>>>(P, st, sum, sumsq);
}

__global__ void k_finalize(const double* sum, float* film, size_t n3, double inv_spp) {
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n3) film[i] = float(sum[i] * inv_spp);
}

// ---------------------------------------------------- many-image batch ----
// Start of a wavefront of the fused batch (one block of 1024 threads): nb,
// every job's g0 for this wavefront, and the accumulation's thread map: job j
// gets its pixels in the wavefront x group_j lanes, rounded up to whole warps
// (so that a warp never mixes jobs), as an exclusive prefix.
__global__ void __launch_bounds__(1024) k_batch_begin(BatchDev bt, PTState st) {
  __shared__ unsigned long long part[1024];
  const unsigned long long G0 = bt.cursor[0], all = bt.cursor[2];
  const unsigned long long nb = G0 < all ? min((unsigned long long)bt.B, all - G0) : 0ull;
  const unsigned long long G1 = G0 + nb;
  const int J = bt.n_jobs, per = (J + 1023) / 1024;
  unsigned long long local = 0;
  for (int k = 0; k < per; ++k) {
    const int j = int(threadIdx.x) * per + k;
    if (j >= J) break;
    BatchJob& b = bt.jobs[j];
    b.P.g0 = G0 - b.start;
    b.P.nb = int(nb);
    const unsigned long long a = max(G0, b.start), e = min(G1, b.start + b.total);
    unsigned long long np = 0;
    if (a < e) {
      const unsigned long long spp = unsigned(b.P.spp);
      np = (e - 1 - b.start) / spp - (a - b.start) / spp + 1;
    }
    b.wnp = np;
    const unsigned long long lanes = (np * unsigned(b.group) + 31) & ~31ull;
    b.wlane = lanes;
    local += lanes;
  }
  part[threadIdx.x] = local;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {
    const unsigned long long v = int(threadIdx.x) >= off ? part[threadIdx.x - off] : 0ull;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  unsigned long long run = part[threadIdx.x] - local;
  for (int k = 0; k < per; ++k) {
    const int j = int(threadIdx.x) * per + k;
    if (j >= J) break;
    const unsigned long long lanes = bt.jobs[j].wlane;
    bt.jobs[j].wlane = run;
    run += lanes;
  }
  if (threadIdx.x == 1023) bt.cursor[3] = part[1023];
  if (threadIdx.x == 0) {
    bt.cursor[1] = nb;
    st.counts[0] = int(nb);
    st.work[0] = 0;  // work counter of the first extend
  }
}

// Camera rays of the wavefront: each slot finds its job and starts the path
// exactly as a single render of that job would.
__global__ void __launch_bounds__(256) k_raygen_ms(PTState st, BatchDev bt) {
  const int slot = blockIdx.x * blockDim.x + threadIdx.x;
  if ((unsigned long long)slot >= bt.cursor[1]) return;
  const int j = batch_job_of(bt, bt.cursor[0] + (unsigned long long)slot);
  bt.job_of[slot] = (unsigned short)j;
  raygen_slot(bt.jobs[j].P, st, slot);
}

// Per-pixel FP64 sums of the wavefront: a group of lanes per pixel (the
// job's group size, a power of two up to 32, all within one warp) takes
// every group-th sample of the pixel's samples in the wavefront, and the
// group adds its partial sums by shuffles.
__global__ void __launch_bounds__(256) k_accumulate_ms(PTState st, BatchDev bt) {
  const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bt.cursor[3]) return;  // whole warps: the lane count is a multiple of 32
  int lo = 0, hi = bt.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bt.jobs[mid].wlane <= t) lo = mid;
    else hi = mid - 1;
  }
  const BatchJob& b = bt.jobs[lo];
  const int G = b.group;  // uniform over the warp
  const unsigned long long l = t - b.wlane, px = l / unsigned(G);
  const int sub = int(l % unsigned(G));
  const bool live = px < b.wnp;
  const unsigned long long G0 = bt.cursor[0], G1 = G0 + bt.cursor[1];
  const unsigned long long spp = unsigned(b.P.spp);
  const unsigned long long a = max(G0, b.start) - b.start, e = min(G1, b.start + b.total) - b.start;
  const unsigned long long p = a / spp + px;
  FSum s0, s1, s2;
  unsigned long long bad = 0;
  if (live) {
    const unsigned long long gb = max(a, p * spp), ge = min(e, (p + 1) * spp);
    for (unsigned long long g = gb + unsigned(sub); g < ge; g += unsigned(G)) {
      float4 L = st.L[b.start + g - G0];
      if (b.P.nan_every && g % b.P.nan_every == 0) L.x = CUDART_NAN_F;
      if (!isfinite(L.x) || !isfinite(L.y) || !isfinite(L.z)) { ++bad; continue; }
      s0.add(L.x); s1.add(L.y); s2.add(L.z);
    }
  }
  for (int o = G >> 1; o > 0; o >>= 1) {
    s0.shfl_merge(o, G); s1.shfl_merge(o, G); s2.shfl_merge(o, G);
    bad += __shfl_down_sync(0xffffffffu, bad, o, G);
  }
  if (live && sub == 0) {
    if (bad) atomicAdd(&st.tally[2], bad);
    double* o = bt.sum + 3 * (b.pix0 + p);
    if (bt.shared_sum) {  // a pixel's samples can lie in two pipelines' wavefronts
      atomicAdd(o, s0.value()); atomicAdd(o + 1, s1.value()); atomicAdd(o + 2, s2.value());
    } else {
      o[0] += s0.value(); o[1] += s1.value(); o[2] += s2.value();
    }
  }
}

__global__ void k_batch_end(BatchDev bt) {
  if (threadIdx.x == 0 && blockIdx.x == 0) bt.cursor[0] += bt.stride;
}

// Films of all jobs from their sums (1 / spp of each job).
__global__ void k_finalize_ms(BatchDev bt, unsigned long long n3) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n3) return;
  const unsigned long long pix = i / 3;
  int lo = 0, hi = bt.n_jobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bt.jobs[mid].pix0 <= pix) lo = mid;
    else hi = mid - 1;
  }
  bt.film[i] = float(bt.sum[i] * (1.0 / double(bt.jobs[lo].P.spp)));
}

// ------------------------------------------------------------- driver ----
static CamDev make_camera(const gbrt_camera& c) {
  // Camera::init (src/camera.cpp:34-48) in float with double-length
  // normalisation like QVector3D.
  auto nrm = [](double x, double y, double z, float out[3]) {
    float fx = float(x), fy = float(y), fz = float(z);
    double l = double(fx) * fx + double(fy) * fy + double(fz) * fz;
    if (std::fabs(l - 1.0) <= 1e-12) { out[0] = fx; out[1] = fy; out[2] = fz; return; }
    double s = l > 1e-12 ? std::sqrt(l) : 0.0;
    out[0] = s > 0 ? float(fx / s) : 0.f;
    out[1] = s > 0 ? float(fy / s) : 0.f;
    out[2] = s > 0 ? float(fz / s) : 0.f;
  };
  CamDev d;
  for (int k = 0; k < 3; ++k) d.eye[k] = c.eye[k];
  float w[3], u[3], v[3];
  nrm(float(c.eye[0] - c.look_at[0]), float(c.eye[1] - c.look_at[1]), float(c.eye[2] - c.look_at[2]), w);
  float cu[3] = {c.up[1] * w[2] - c.up[2] * w[1], c.up[2] * w[0] - c.up[0] * w[2], c.up[0] * w[1] - c.up[1] * w[0]};
  nrm(cu[0], cu[1], cu[2], u);
  v[0] = w[1] * u[2] - w[2] * u[1];
  v[1] = w[2] * u[0] - w[0] * u[2];
  v[2] = w[0] * u[1] - w[1] * u[0];
  for (int k = 0; k < 3; ++k) { d.u[k] = u[k]; d.v[k] = v[k]; d.w[k] = w[k]; }
  float aspect = float(c.width) / float(c.height);
  d.t = float(std::tan(double(c.fov / 2)));
  d.b = -d.t;
  d.r = aspect * d.t;
  d.l = -d.r;
  d.W = c.width;
  d.H = c.height;
  return d;
}

// The extend / shadow kernels for a scene and flags: traversal counters,
// watertight triangles, short stack when the tree is shallow enough.
struct TraceKernels {
  void (*ext)(DeviceScene, PTState, int);
  void (*sh)(DeviceScene, PTState);
};
template <bool C, bool W, bool G>
static TraceKernels pick_stack(bool shortStack) {
  if (shortStack) return {k_extend<C, W, kShortStack, G>, k_shadow<C, W, kShortStack, G>};
  return {k_extend<C, W, kStackSize, G>, k_shadow<C, W, kStackSize, G>};
}
template <bool G>
static TraceKernels pick_flags(bool count, bool wt, bool shortStack) {
  if (count) return wt ? pick_stack<true, true, G>(shortStack) : pick_stack<true, false, G>(shortStack);
  return wt ? pick_stack<false, true, G>(shortStack) : pick_stack<false, false, G>(shortStack);
}
// Traversal counters, watertight triangles, short stack when the tree is
// shallow enough, the general leaves (CSG objects, instances) only for scenes
// that have them.
static TraceKernels pick_kernels(const gbrt_scene* s, bool count) {
  if (s->ctx->fault_small_stack) {
    // Injected fault: a stack too small for most trees, so that the overflow
    // check sets the error word (the call returns GBRT_ERR_NUMERIC).
    if (s->view.csg_prog || s->view.inst) return {k_extend<false, false, kFaultStack, true>, k_shadow<false, false, kFaultStack, true>};
    return {k_extend<false, false, kFaultStack, false>, k_shadow<false, false, kFaultStack, false>};
  }
  const bool shortStack = stack_need(s->max_depth4) <= kShortStack;
  if (s->view.csg_prog || s->view.inst) return pick_flags<true>(count, s->watertight, shortStack);
  return pick_flags<false>(count, s->watertight, shortStack);
}

// The shade kernel: estimator, guiding, and the texture / CSG / instance code
// only for scenes that have textures, CSG objects or instances.
static bool ext_scene(const gbrt_scene* s) {
  return s->view.tri_uv != nullptr || s->view.csg_prog != nullptr || s->view.inst != nullptr;
}
static void (*pick_shade(const gbrt_scene* s, bool physical, bool guided))(DeviceScene, PTParams, PTState, int) {
  const bool ext = ext_scene(s);
  if (!physical) return ext ? k_shade<true, StreamSrc> : k_shade<false, StreamSrc>;
  if (guided) return ext ? k_shade_phys<true, true> : k_shade_phys<true, false>;
  return ext ? k_shade_phys<false, true> : k_shade_phys<false, false>;
}

static void init_params(PTParams& P, const gbrt_ctx* ctx, const gbrt_camera& cam, const gbrt_render_params& prm,
                        unsigned long long total) {
  P.cam = make_camera(cam);
  P.nan_every = ctx->fault_nan_every;
  P.seed = prm.seed;
  P.xs = prm.x_samples;
  P.ys = prm.y_samples;
  P.spp = prm.x_samples * prm.y_samples;
  P.D = prm.max_depth;
  P.term_p = prm.termination_prob;
  P.rr_pdf = prm.termination_prob > 0.f ? prm.termination_prob : 1.f;
  P.inv_log1mp = (prm.termination_prob > 0.f && prm.termination_prob < 1.f)
                     ? float(1.0 / std::log(1.0 - double(prm.termination_prob)))
                     : 0.f;
  P.idx32 = total <= 0xffffffffull ? 1 : 0;
  P.physical = prm.semantics == GBRT_SEM_PHYSICAL ? 1 : 0;
}

struct Buffers {
  std::vector<void*> ptrs;
  const gbrt_ctx* ctx;
  cudaStream_t stream;
  Buffers(const gbrt_ctx* c, cudaStream_t s) : ctx(c), stream(s) {}
  ~Buffers() {
    for (void* p : ptrs) cudaFreeAsync(p, stream);
  }
  template <typename T>
  cudaError_t alloc(T** out, size_t count) {
    void* p = nullptr;
    cudaError_t e = ctx_alloc(ctx, &p, std::max<size_t>(count, 1) * sizeof(T), stream);
    if (e == cudaSuccess) ptrs.push_back(p);
    *out = static_cast<T*>(p);
    return e;
  }
};

// keep_sums: add to d_sum_in / d_sumsq instead of clearing them first (both
// must then be given); film_scale: the film is sum x film_scale (0: 1 / spp).
static gbrt_status render_impl(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm, float* d_film,
                               double* d_sum_in, double* d_sumsq, const volatile int32_t* stop, gbrt_stats* stats,
                               bool keep_sums = false, double film_scale = 0.0) {
  gbrt_ctx* ctx = s->ctx;
  if (!cam || !prm || !d_film) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render: NULL argument");
  if (cam->width <= 0 || cam->height <= 0 || prm->x_samples <= 0 || prm->y_samples <= 0 || prm->max_depth <= 0 ||
      prm->max_depth > 64)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render: bad camera or render parameters");
  if (prm->semantics != GBRT_SEM_REFERENCE && prm->semantics != GBRT_SEM_PHYSICAL)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render: unknown semantics");
  if (!(prm->termination_prob >= 0.f && prm->termination_prob <= 1.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render: termination probability outside [0, 1]");
  cudaStream_t stream = ctx->stream;
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const unsigned long long npix = (unsigned long long)cam->width * cam->height;
  const int spp = prm->x_samples * prm->y_samples;
  const unsigned long long total = npix * (unsigned long long)spp;
  // 2^26 paths (~20 GB of state) per wavefront by default: fewer, fuller
  // launches for the deep bounces (the 67M-path frame in one wavefront runs
  // 19 % faster than with 2^23, 1.6 % faster than with 2^25).
  long long B = prm->batch_paths > 0 ? prm->batch_paths : (1ll << 26);
  B = std::min<long long>(B, (long long)total);
  B = std::max<long long>(B, 1);

  PTParams P{};
  init_params(P, ctx, *cam, *prm, total);

  Buffers buf(ctx, stream);
  PTState st{};
  cudaError_t e = cudaSuccess;
  double* d_sum = d_sum_in;
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
  if (!d_sum) A(buf.alloc(&d_sum, npix * 3));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "render buffers");
  if (!keep_sums) {
    A(cudaMemsetAsync(d_sum, 0, npix * 3 * sizeof(double), stream));
    if (d_sumsq) A(cudaMemsetAsync(d_sumsq, 0, npix * 3 * sizeof(double), stream));
  }
  A(cudaMemsetAsync(st.tally, 0, 8 * sizeof(unsigned long long), stream));
  A(cudaMemsetAsync(st.err, 0, sizeof(int), stream));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "render set-up");

  const bool count = (prm->flags & GBRT_RENDER_COUNT_TRAVERSAL) != 0;
  const bool timeK = (prm->flags & GBRT_RENDER_TIME_KERNELS) != 0;
  const TraceKernels tk = pick_kernels(s, count);
  auto kExt = tk.ext;
  auto kSh = tk.sh;
  // Persistent grids: every SM filled with as many blocks as fit.
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kExt, kTraceBlock, 0);
  const int traceGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kSh, kTraceBlock, 0);
  const int shadowGrid = std::max(1, per) * ctx->num_sms;
  const int shadeGrid = ctx->num_sms * 8;
  auto kShade = pick_shade(s, P.physical != 0, false);
  cudaEvent_t ev0, ev1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  // Per-kernel timing: one event pair per launch of extend / shade / shadow.
  std::vector<cudaEvent_t> kev;
  auto mark = [&]() {
    cudaEvent_t e2;
    cudaEventCreate(&e2);
    cudaEventRecord(e2, stream);
    kev.push_back(e2);
  };
  cudaEventRecord(ev0, stream);
  unsigned long long launches = 0;
  gbrt_status status = GBRT_OK;
  for (unsigned long long g0 = 0; g0 < total; g0 += (unsigned long long)B) {
    if (stop && *stop) { status = fail(ctx, GBRT_ERR_CANCELLED, "gbrt_render: cancelled"); break; }
    P.g0 = g0;
    P.nb = int(std::min<unsigned long long>((unsigned long long)B, total - g0));
    k_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
    ++launches;
    for (int it = 0; it < P.D; ++it) {
      int cur = it & 1;
      if (timeK) mark();
      kExt<<<cap_grid(traceGrid, P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st, cur);
      if (timeK) mark();
      kShade<<<cap_grid(shadeGrid, P.nb, 256), 256, 0, stream>>>(s->view, P, st, cur);
      if (timeK) mark();
      kSh<<<cap_grid(shadowGrid, 2ll * P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st);
      if (timeK) mark();
      launches += 3;
    }
    launch_accumulate(P, st, d_sum, d_sumsq, stream);
    ++launches;
    A(cudaGetLastError());
    if (e != cudaSuccess) break;
  }
  size_t n3 = size_t(npix) * 3;
  k_finalize<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_sum, d_film, n3,
                                                             film_scale > 0.0 ? film_scale : 1.0 / spp);
  ++launches;
  cudaEventRecord(ev1, stream);
  A(cudaGetLastError());
  unsigned long long tally[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int err = 0;
  A(cudaMemcpyAsync(tally, st.tally, sizeof tally, cudaMemcpyDeviceToHost, stream));
  A(cudaMemcpyAsync(&err, st.err, sizeof err, cudaMemcpyDeviceToHost, stream));
  A(cudaStreamSynchronize(stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev0, ev1);
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  double kms[3] = {0, 0, 0};
  for (size_t k = 0; k + 3 < kev.size(); k += 4) {
    for (int j = 0; j < 3; ++j) {
      float t = 0.f;
      cudaEventElapsedTime(&t, kev[k + j], kev[k + j + 1]);
      kms[j] += t;
    }
  }
  for (cudaEvent_t x : kev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->paths = status == GBRT_OK ? total : 0;
    stats->extension_rays = tally[0];
    stats->shadow_rays = tally[1];
    stats->nonfinite = tally[2];
    stats->render_ms = ms;
    stats->kernel_launches = launches;
    stats->extend_ms = kms[0];
    stats->shade_ms = kms[1];
    stats->shadow_ms = kms[2];
    unsigned long long nl = kev.size() / 4;
    stats->extend_launches = stats->shade_launches = stats->shadow_launches = nl;
    stats->nodes_closest = tally[3];
    stats->prims_closest = tally[4];
    stats->nodes_any = tally[5];
    stats->prims_any = tally[6];
  }
  if (err) return fail(ctx, GBRT_ERR_NUMERIC, err_text("gbrt_render", err));
  return status;
}

// ------------------------------------------- render without allocation ----
// gbrt_render_device_noalloc keeps its wavefront state in one file-scope
// device array instead of allocating it. Its layout, per path of a batch of
// at most kNoAllocBatch paths, mirrors PTState; every sub-array starts on a
// 256-byte boundary.
constexpr long long kNoAllocBatch = GBRT_NOALLOC_MAX_BATCH;

struct NoAllocLayout {
  size_t off[20];
  size_t bytes;
};

constexpr size_t noalloc_align(size_t x) { return (x + 255) & ~size_t(255); }

static NoAllocLayout noalloc_layout() {
  const size_t B = size_t(kNoAllocBatch);
  const size_t sizes[20] = {
      B * sizeof(float4), B * sizeof(float4), B * sizeof(int4),                          // alpha, L, ctl
      B * sizeof(float4), B * sizeof(float4), B * sizeof(float4), B * sizeof(float4),    // pending vertex
      2 * B * sizeof(float4), 2 * B * sizeof(float4),                                    // ext[0], ext[1]
      B * sizeof(int), B * sizeof(int),                                                  // ext_slot[0], [1]
      B * sizeof(RawHit),                                                                // hits
      4 * B * sizeof(float4), 2 * B * sizeof(float4), 2 * B * sizeof(int),               // shadow queue
      4 * sizeof(int), 4 * sizeof(unsigned long long), 8 * sizeof(unsigned long long),   // counts, work, tally
      sizeof(int),                                                                       // err
      B * sizeof(int)};                                                                  // hit_inst
  NoAllocLayout L{};
  size_t o = 0;
  for (int i = 0; i < 20; ++i) {
    L.off[i] = o;
    o += noalloc_align(sizes[i]);
  }
  L.bytes = o;
  return L;
}

// 65,536 paths x 308 bytes + counters, rounded up: 20 MiB.
constexpr size_t kNoAllocScratchBytes = size_t(20) << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of g_noalloc_scratch, looked up once per context with the
// context's device current (the array's host-side name is not a device
// address). Kept in the context, not in a process-wide table: a context
// created after cudaDeviceReset belongs to a new CUDA context in which the
// module, and so the array, may sit at another address.
static gbrt_status noalloc_scratch(gbrt_ctx* ctx, unsigned char** out) {
  if (!ctx->noalloc_scratch) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    ctx->noalloc_scratch = static_cast<unsigned char*>(p);
  }
  *out = ctx->noalloc_scratch;
  return GBRT_OK;
}

static gbrt_status render_noalloc_impl(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                                       float* d_film, double* d_sum, double* d_sumsq, gbrt_stats* stats) {
  gbrt_ctx* ctx = s->ctx;
  if (!cam || !prm || !d_film || !d_sum)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_device_noalloc: NULL camera, params, film or sum");
  if (cam->width <= 0 || cam->height <= 0 || prm->x_samples <= 0 || prm->y_samples <= 0 || prm->max_depth <= 0 ||
      prm->max_depth > 64)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_device_noalloc: bad camera or render parameters");
  if (prm->batch_paths < 0 || prm->batch_paths > kNoAllocBatch)
    return fail(ctx, GBRT_ERR_INVALID_ARG,
                "gbrt_render_device_noalloc: batch_paths exceeds the 65536-path (GBRT_NOALLOC_MAX_BATCH) "
                "scratch of the no-allocation entry point");
  if (prm->semantics != GBRT_SEM_REFERENCE && prm->semantics != GBRT_SEM_PHYSICAL)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_device_noalloc: unknown semantics");
  if (!(prm->termination_prob >= 0.f && prm->termination_prob <= 1.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_device_noalloc: termination probability outside [0, 1]");
  const NoAllocLayout Lay = noalloc_layout();
  if (Lay.bytes > kNoAllocScratchBytes)
    return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_render_device_noalloc: scratch layout exceeds the array");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  unsigned char* base = nullptr;
  gbrt_status gs = noalloc_scratch(ctx, &base);
  if (gs != GBRT_OK) return gs;
  cudaStream_t stream = ctx->stream;
  auto at = [&](int i) { return static_cast<void*>(base + Lay.off[i]); };
  PTState st{};
  st.alpha = static_cast<float4*>(at(0));
  st.L = static_cast<float4*>(at(1));
  st.ctl = static_cast<int4*>(at(2));
  st.pv_p = static_cast<float4*>(at(3));
  st.pv_n = static_cast<float4*>(at(4));
  st.pv_d = static_cast<float4*>(at(5));
  st.pv_a = static_cast<float4*>(at(6));
  st.ext[0] = static_cast<float4*>(at(7));
  st.ext[1] = static_cast<float4*>(at(8));
  st.ext_slot[0] = static_cast<int*>(at(9));
  st.ext_slot[1] = static_cast<int*>(at(10));
  st.hits = static_cast<RawHit*>(at(11));
  st.sh_ray = static_cast<float4*>(at(12));
  st.sh_c = static_cast<float4*>(at(13));
  st.sh_slot = static_cast<int*>(at(14));
  st.counts = static_cast<int*>(at(15));
  st.work = static_cast<unsigned long long*>(at(16));
  st.tally = static_cast<unsigned long long*>(at(17));
  st.err = static_cast<int*>(at(18));
  st.hit_inst = s->view.inst ? static_cast<int*>(at(19)) : nullptr;
  st.ext_cap = int(kNoAllocBatch);
  st.sh_cap = int(2 * kNoAllocBatch);

  const unsigned long long npix = (unsigned long long)cam->width * cam->height;
  const int spp = prm->x_samples * prm->y_samples;
  const unsigned long long total = npix * (unsigned long long)spp;
  long long B = prm->batch_paths > 0 ? prm->batch_paths : kNoAllocBatch;
  B = std::max<long long>(1, std::min<long long>(B, (long long)total));
  PTParams P{};
  init_params(P, ctx, *cam, *prm, total);

  // The array keeps the previous call's contents: clear what starts at zero.
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(cudaMemsetAsync(st.tally, 0, 8 * sizeof(unsigned long long), stream));
  A(cudaMemsetAsync(st.err, 0, sizeof(int), stream));
  A(cudaMemsetAsync(d_sum, 0, npix * 3 * sizeof(double), stream));
  if (d_sumsq) A(cudaMemsetAsync(d_sumsq, 0, npix * 3 * sizeof(double), stream));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_device_noalloc set-up");

  const TraceKernels tk = pick_kernels(s, (prm->flags & GBRT_RENDER_COUNT_TRAVERSAL) != 0);
  auto kExt = tk.ext;
  auto kSh = tk.sh;
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kExt, kTraceBlock, 0);
  const int traceGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kSh, kTraceBlock, 0);
  const int shadowGrid = std::max(1, per) * ctx->num_sms;
  const int shadeGrid = ctx->num_sms * 8;
  auto kShade = pick_shade(s, P.physical != 0, false);
  auto t0 = std::chrono::steady_clock::now();
  unsigned long long launches = 0;
  for (unsigned long long g0 = 0; g0 < total; g0 += (unsigned long long)B) {
    P.g0 = g0;
    P.nb = int(std::min<unsigned long long>((unsigned long long)B, total - g0));
    k_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
    ++launches;
    for (int it = 0; it < P.D; ++it) {
      int cur = it & 1;
      kExt<<<cap_grid(traceGrid, P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st, cur);
      kShade<<<cap_grid(shadeGrid, P.nb, 256), 256, 0, stream>>>(s->view, P, st, cur);
      kSh<<<cap_grid(shadowGrid, 2ll * P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st);
      launches += 3;
    }
    launch_accumulate(P, st, d_sum, d_sumsq, stream);
    ++launches;
    A(cudaGetLastError());
    if (e != cudaSuccess) break;
  }
  size_t n3 = size_t(npix) * 3;
  k_finalize<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_sum, d_film, n3, 1.0 / spp);
  ++launches;
  A(cudaGetLastError());
  unsigned long long tally[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int err = 0;
  A(cudaMemcpyAsync(tally, st.tally, sizeof tally, cudaMemcpyDeviceToHost, stream));
  A(cudaMemcpyAsync(&err, st.err, sizeof err, cudaMemcpyDeviceToHost, stream));
  A(cudaStreamSynchronize(stream));
  double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_device_noalloc");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->paths = total;
    stats->extension_rays = tally[0];
    stats->shadow_rays = tally[1];
    stats->nonfinite = tally[2];
    stats->render_ms = ms;
    stats->kernel_launches = launches;
    stats->nodes_closest = tally[3];
    stats->prims_closest = tally[4];
    stats->nodes_any = tally[5];
    stats->prims_any = tally[6];
  }
  if (err) return fail(ctx, GBRT_ERR_NUMERIC, err_text("gbrt_render_device_noalloc", err));
  return GBRT_OK;
}

// ------------------------------------------------------ guided render ----
// gbrt_render_guided: passes of the physical estimator; with a guide, the
// first train_passes passes record training samples and each is followed by
// steps_per_pass Adam steps; vertices sample the guide once it has been
// trained (or given weights). The film is the mean over all passes.
// Relative squared deviation of a pass from the mean of the earlier passes,
// summed over pixels and channels: sum ((x - m)^2 / (m^2 + 0.01)), x the
// pass's mean (its sums times inv_pass), m the earlier passes' mean (their
// sums times inv_prev).
__global__ void __launch_bounds__(256) k_pass_deviation(const double* __restrict__ pass_sum,
                                                        const double* __restrict__ prev_sum, size_t n3,
                                                        double inv_pass, double inv_prev, double* out) {
  double acc = 0.0;
  for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n3; i += size_t(gridDim.x) * blockDim.x) {
    double x = pass_sum[i] * inv_pass, m = prev_sum[i] * inv_prev;
    double d = x - m;
    if (isfinite(d)) acc += d * d / (m * m + 0.01);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double part[8];
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double b = 0.0;
    for (int k = 0; k < int(blockDim.x >> 5); ++k) b += part[k];
    atomicAdd(out, b);
  }
}

// prev_sum += pass_sum; with a deviation (dev != null), weighted += w *
// pass_sum * inv_pass (the pass's mean) and wtotal += w for w = n3 / *dev.
// Thread 0 also adds the pass's training samples (min(*tcount, tcap)) to
// *tsamples.
__global__ void k_pass_combine(const double* __restrict__ pass_sum, double* __restrict__ prev_sum,
                               double* __restrict__ weighted, size_t n3, double inv_pass, const double* dev,
                               double* wtotal, const int* tcount, int tcap, unsigned long long* tsamples) {
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const double w = (dev && *dev > 0.0) ? double(n3) / *dev : 0.0;
  if (i == 0) {
    if (dev) *wtotal += w;
    if (tcount) *tsamples += (unsigned long long)min(*tcount, tcap);
  }
  if (i >= n3) return;
  double x = pass_sum[i];
  prev_sum[i] += x;
  if (w > 0.0) weighted[i] += w * x * inv_pass;
}

// film = (sum over passes of w * pass mean) / (sum of w).
__global__ void k_finalize_weighted(const double* __restrict__ weighted, float* __restrict__ film, size_t n3,
                                    const double* wtotal) {
  size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i < n3) film[i] = float(weighted[i] / *wtotal);
}

static unsigned long long pass_seed(unsigned long long seed, int pass) {
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * (unsigned long long)(pass + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static gbrt_status render_guided_impl(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                                      gbrt_guide* g, const gbrt_guide_params* gp, float* film,
                                      gbrt_guide_stats* stats) {
  gbrt_ctx* ctx = s->ctx;
  if (!cam || !prm || !gp || !film) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: NULL argument");
  if (cam->width <= 0 || cam->height <= 0 || prm->x_samples <= 0 || prm->y_samples <= 0 || prm->max_depth <= 0 ||
      prm->max_depth > 64)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: bad camera or render parameters");
  if (prm->semantics != GBRT_SEM_PHYSICAL)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: needs the physical estimator (GBRT_SEM_PHYSICAL)");
  if (!(prm->termination_prob >= 0.f && prm->termination_prob < 1.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: termination probability outside [0, 1)");
  if (!(gp->guide_fraction >= 0.f && gp->guide_fraction <= 1.f) || gp->passes < 0 || gp->train_passes < 0 ||
      gp->steps_per_pass < 0 || gp->guide_depth < 0 || gp->late_pass_samples < 0 ||
      (gp->passes == 0 && !(gp->time_budget_ms > 0.f)))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: bad guide parameters");
  const bool useGuide = g && gp->guide_fraction > 0.f;
  const bool training = useGuide && gp->train_passes > 0 && gp->steps_per_pass > 0;
  if (training && (gp->batch_samples <= 0 || !(gp->learning_rate > 0.f)))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: training needs batch_samples and learning_rate");
  if (g && g->device != s->device)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: guide and scene live on different devices");
  cudaStream_t stream = ctx->stream;
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const unsigned long long npix = (unsigned long long)cam->width * cam->height;
  const int spp = prm->x_samples * prm->y_samples;
  // Passes after the last training pass may take more samples per pixel
  // (late_pass_samples x 1 strata), so that they fill the GPU.
  gbrt_render_params lateParams = *prm;
  if (gp->late_pass_samples > 0) {
    lateParams.x_samples = gp->late_pass_samples;
    lateParams.y_samples = 1;
  }
  const int lateSpp = lateParams.x_samples * lateParams.y_samples;
  const unsigned long long total = npix * (unsigned long long)spp;
  const unsigned long long lateTotal = npix * (unsigned long long)lateSpp;
  long long B = prm->batch_paths > 0 ? prm->batch_paths : (1ll << 23);
  B = std::max<long long>(1, std::min<long long>(B, (long long)std::max(total, lateTotal)));

  Buffers buf(ctx, stream);
  PTState st;
  std::memset(&st, 0, sizeof st);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  A(buf.alloc(&st.alpha, B)); A(buf.alloc(&st.L, B)); A(buf.alloc(&st.ctl, B));
  A(buf.alloc(&st.pv_p, 1)); A(buf.alloc(&st.pv_n, 1)); A(buf.alloc(&st.pv_d, 1)); A(buf.alloc(&st.pv_a, 1));
  A(buf.alloc(&st.ext[0], 2 * B)); A(buf.alloc(&st.ext[1], 2 * B));
  A(buf.alloc(&st.ext_slot[0], B)); A(buf.alloc(&st.ext_slot[1], B));
  A(buf.alloc(&st.hits, B));
  if (s->view.inst) A(buf.alloc(&st.hit_inst, B));
  A(buf.alloc(&st.sh_ray, 4 * B)); A(buf.alloc(&st.sh_c, 2 * B)); A(buf.alloc(&st.sh_slot, 2 * B));
  A(buf.alloc(&st.counts, 4)); A(buf.alloc(&st.work, 4)); A(buf.alloc(&st.tally, 8)); A(buf.alloc(&st.err, 1));
  st.ext_cap = int(B);
  st.sh_cap = int(2 * B);
  long long tcap = 0;
  // Asynchronous training: the Adam steps of pass p's samples run on a second
  // stream while pass p + 1 renders. Pass p infers with the snapshot wq[p & 1]
  // of the weights left by the steps of pass p - 2 and collects its samples
  // into tsamp[p & 1]; the render stream waits for those steps (event
  // trained[p & 1]) before the pass starts.
  const bool async = training && (gp->flags & GBRT_GUIDE_ASYNC_TRAINING) != 0;
  float4* tsampBuf[2] = {nullptr, nullptr};
  int* tcountBuf[2] = {nullptr, nullptr};
  __nv_bfloat16* wq[2] = {nullptr, nullptr};
  __nv_bfloat16* wt = nullptr;
  if (useGuide) {
    A(buf.alloc(&st.gin, 3 * B));
    A(buf.alloc(&st.mix, guide::kMixStride * B));
    if (training) {
      A(buf.alloc(&st.rec, (long long)kRecComp * kRecords * B));
      tcap = std::min<long long>((long long)gp->steps_per_pass * gp->batch_samples, 1ll << 25);
      for (int b = 0; b < (async ? 2 : 1); ++b) {
        A(buf.alloc(&tsampBuf[b], 4 * tcap));
        A(buf.alloc(&tcountBuf[b], 1));
      }
      st.tsamp = tsampBuf[0];
      st.tcount = tcountBuf[0];
      if (async) {
        A(buf.alloc(&wt, guide::kParams));
        A(buf.alloc(&wq[0], guide::kParams));
        A(buf.alloc(&wq[1], guide::kParams));
      }
    }
  }
  st.tcap = int(tcap);
  st.nslots = int(B);
  // Films: the current pass, the sum of all passes, the inverse-variance
  // weighted sum, and the deviation accumulator.
  const size_t n3 = size_t(npix) * 3;
  double *d_pass = nullptr, *d_sum = nullptr, *d_wsum = nullptr, *d_dev = nullptr, *d_wtot = nullptr;
  float* d_film = nullptr;
  A(buf.alloc(&d_pass, n3));
  A(buf.alloc(&d_sum, n3));
  A(buf.alloc(&d_wsum, n3));
  A(buf.alloc(&d_dev, 1));
  A(buf.alloc(&d_wtot, 1));
  A(buf.alloc(&d_film, n3));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "guided render buffers");
  A(cudaMemsetAsync(d_sum, 0, n3 * sizeof(double), stream));
  A(cudaMemsetAsync(d_wsum, 0, n3 * sizeof(double), stream));
  A(cudaMemsetAsync(d_wtot, 0, sizeof(double), stream));
  // Inverse-variance weighting of the passes when a guide is used: a pass
  // sampled by a network still in training is noisier than later ones.
  const bool weighted = training && !(gp->flags & GBRT_GUIDE_EQUAL_WEIGHTS);

  A(cudaMemsetAsync(st.tally, 0, 8 * sizeof(unsigned long long), stream));
  A(cudaMemsetAsync(st.err, 0, sizeof(int), stream));
  cudaStream_t ts = stream;  // the training stream
  cudaEvent_t trained[2] = {nullptr, nullptr}, sampled = nullptr;
  __nv_bfloat16* const wMain = g ? g->d_w : nullptr;
  if (async && e == cudaSuccess) {
    if (ctx->batch_streams.empty()) {
      cudaStream_t q;
      A(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
      if (e == cudaSuccess) ctx->batch_streams.push_back(q);
    }
    if (e == cudaSuccess) ts = ctx->batch_streams[0];
    for (__nv_bfloat16* w : {wt, wq[0], wq[1]})
      A(cudaMemcpyAsync(w, wMain, guide::kParams * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, stream));
    A(cudaEventCreateWithFlags(&trained[0], cudaEventDisableTiming));
    A(cudaEventCreateWithFlags(&trained[1], cudaEventDisableTiming));
    A(cudaEventCreateWithFlags(&sampled, cudaEventDisableTiming));
    // the training stream starts after the copies
    A(cudaEventRecord(sampled, stream));
    A(cudaStreamWaitEvent(ts, sampled, 0));
    if (e == cudaSuccess) g->d_wt = wt;
  }
  auto end_async = [&]() {
    if (!async || !g || !g->d_wt) return;
    // The render stream waits for every step, and the guide keeps the
    // weights of the last one.
    cudaEvent_t done = nullptr;
    if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess) {
      cudaEventRecord(done, ts);
      cudaStreamWaitEvent(stream, done, 0);
      cudaEventDestroy(done);
    }
    cudaMemcpyAsync(wMain, wt, guide::kParams * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, stream);
    g->d_w = wMain;
    g->d_wt = nullptr;
  };
  if (e != cudaSuccess) {
    end_async();
    for (cudaEvent_t x : {trained[0], trained[1], sampled})
      if (x) cudaEventDestroy(x);
    return cuda_fail(ctx, e, "guided render set-up");
  }

  const TraceKernels tk = pick_kernels(s, false);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tk.ext, kTraceBlock, 0);
  const int traceGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tk.sh, kTraceBlock, 0);
  const int shadowGrid = std::max(1, per) * ctx->num_sms;
  const int shadeGrid = ctx->num_sms * 8;
  cudaEvent_t ev0, ev1, t0, t1;
  cudaEventCreate(&ev0);
  cudaEventCreate(&ev1);
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  cudaEventRecord(ev0, stream);
  int passes = 0, steps = 0;
  unsigned long long infer_launches = 0;
  double train_ms = 0.0, elapsed = 0.0, infer_ms = 0.0;
  const bool timeK = (prm->flags & GBRT_RENDER_TIME_KERNELS) != 0;
  std::vector<cudaEvent_t> iev;
  gbrt_status status = GBRT_OK;
  unsigned long long samples = 0, pathsDone = 0;  // per-pixel samples and paths of the passes so far
  // Asynchronous training: steps issued up to each slot's last training,
  // whether a slot has a training in flight, and the slot of the last one.
  int stepsAt[2] = {0, 0}, lastSlot = -1;
  bool issued[2] = {false, false};
  const bool readyAtStart = g && g->ready;
  for (int pass = 0;; ++pass) {
    if (gp->passes > 0 && pass >= gp->passes) break;
    const bool record = training && pass < gp->train_passes;
    const bool late = !record;
    // Steps whose weights this pass infers with.
    int visible = steps;
    if (async) {
      const int b = record ? (pass & 1) : lastSlot;
      if (b >= 0 && issued[b]) {
        A(cudaStreamWaitEvent(stream, trained[b], 0));
        if (!record) {  // after training: both slots' steps are done, the last is newest
          A(cudaStreamWaitEvent(stream, trained[b ^ 1], 0));
        }
        g->d_w = wq[b];
        visible = stepsAt[b];
      } else {
        g->d_w = wq[0];  // the weights the call started with
        visible = 0;
      }
      if (record) {
        st.tsamp = tsampBuf[pass & 1];
        st.tcount = tcountBuf[pass & 1];
      }
    }
    const int sppPass = late ? lateSpp : spp;
    const unsigned long long passTotal = late ? lateTotal : total;
    PTParams P{};
    init_params(P, ctx, *cam, late ? lateParams : *prm, passTotal);
    P.seed = pass_seed(prm->seed, pass);
    // While training, sample the guide once it has had warmup_steps steps.
    const bool readyNow = async ? (readyAtStart || visible > 0) : (g && g->ready);
    P.guided = (useGuide && readyNow && (!training || visible >= gp->warmup_steps)) ? 1 : 0;
    P.guide_frac = gp->guide_fraction;
    P.record = record ? 1 : 0;
    P.guide_depth = gp->guide_depth;
    P.train_relative = (gp->flags & GBRT_GUIDE_PIXEL_RELATIVE) ? 1 : 0;
    P.train_product = (gp->flags & GBRT_GUIDE_PRODUCT) ? 1 : 0;
    P.film_sum = d_sum;
    P.pass_sum = d_pass;
    P.inv_samples = 1.0 / double(samples + (unsigned long long)sppPass);
    A(cudaMemsetAsync(d_pass, 0, n3 * sizeof(double), stream));
    if (record) A(cudaMemsetAsync(st.tcount, 0, sizeof(int), stream));
    auto kShade = pick_shade(s, true, P.guided || P.record);
    for (unsigned long long g0 = 0; g0 < passTotal && e == cudaSuccess; g0 += (unsigned long long)B) {
      P.g0 = g0;
      P.nb = int(std::min<unsigned long long>((unsigned long long)B, passTotal - g0));
      k_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
      for (int it = 0; it < P.D; ++it) {
        int cur = it & 1;
        tk.ext<<<cap_grid(traceGrid, P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st, cur);
        if (P.guided && (P.guide_depth == 0 || it < P.guide_depth)) {
          cudaEvent_t ea = nullptr, eb = nullptr;
          if (timeK) {
            cudaEventCreate(&ea);
            cudaEventCreate(&eb);
            cudaEventRecord(ea, stream);
          }
          k_guide_prep<<<shadeGrid, 256, 0, stream>>>(s->view, st, cur);
          A(guide::launch_infer(g, st.gin, st.counts + cur, 0, st.mix, stream));
          if (timeK) {
            cudaEventRecord(eb, stream);
            iev.push_back(ea);
            iev.push_back(eb);
          }
          ++infer_launches;
        }
        kShade<<<cap_grid(shadeGrid, P.nb, 256), 256, 0, stream>>>(s->view, P, st, cur);
        tk.sh<<<cap_grid(shadowGrid, 2ll * P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st);
      }
      launch_accumulate(P, st, d_pass, nullptr, stream);
      if (record) k_guide_collect<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
      A(cudaGetLastError());
    }
    if (e != cudaSuccess) break;
    // Fold the pass into the films. The first pass of a weighted render only
    // serves as the first mean (it was sampled without the guide).
    const bool wpass = weighted && pass > 0;
    if (wpass) {
      A(cudaMemsetAsync(d_dev, 0, sizeof(double), stream));
      k_pass_deviation<<<ctx->num_sms * 4, 256, 0, stream>>>(d_pass, d_sum, n3, 1.0 / sppPass,
                                                             1.0 / double(samples), d_dev);
    }
    k_pass_combine<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_pass, d_sum, d_wsum, n3, 1.0 / sppPass,
                                                                   wpass ? d_dev : nullptr, d_wtot,
                                                                   record ? st.tcount : nullptr, int(tcap),
                                                                   st.tally + 3);
    A(cudaGetLastError());
    ++passes;
    samples += (unsigned long long)sppPass;
    pathsDone += passTotal;
    if (record) {
      // Steps over the pass's samples; their count stays on the device.
      // Asynchronously: on the training stream once the pass's samples are
      // in, then a snapshot of the weights for pass + 2.
      if (async) {
        A(cudaEventRecord(sampled, stream));
        A(cudaStreamWaitEvent(ts, sampled, 0));
      }
      if (timeK) cudaEventRecord(t0, ts);
      for (int k = 0; k < gp->steps_per_pass && e == cudaSuccess; ++k) {
        A(guide::train_window(g, st.tsamp, st.tcount, int(tcap), k, gp->batch_samples, gp->learning_rate, true,
                              ts));
        if (!async) g->ready = true;
        ++steps;
      }
      if (timeK) cudaEventRecord(t1, ts);
      if (async) {
        const int b = pass & 1;
        A(cudaMemcpyAsync(wq[b], wt, guide::kParams * sizeof(__nv_bfloat16), cudaMemcpyDeviceToDevice, ts));
        A(cudaEventRecord(trained[b], ts));
        issued[b] = true;
        stepsAt[b] = steps;
        lastSlot = b;
      }
      if (timeK) {
        A(cudaEventSynchronize(t1));
        float tms = 0.f;
        cudaEventElapsedTime(&tms, t0, t1);
        train_ms += tms;
      }
    }
    if (e != cudaSuccess) break;
    if (gp->passes == 0) {
      // Equal-time rendering: the device clock decides after every pass.
      cudaEventRecord(ev1, stream);
      A(cudaEventSynchronize(ev1));
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev0, ev1);
      elapsed = ms;
      if (elapsed >= gp->time_budget_ms) break;
    }
  }
  end_async();
  if (async && steps > 0) g->ready = true;
  const bool timedAtEnd = gp->passes > 0 || async;
  if (timedAtEnd) cudaEventRecord(ev1, stream);
  if (e == cudaSuccess && passes > 0) {
    if (weighted && passes > 1)
      k_finalize_weighted<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_wsum, d_film, n3, d_wtot);
    else
      k_finalize<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_sum, d_film, n3, 1.0 / double(samples));
    A(cudaGetLastError());
    A(cudaMemcpyAsync(film, d_film, n3 * sizeof(float), cudaMemcpyDeviceToHost, stream));
  }
  unsigned long long tally[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int err = 0, gerr = 0;
  float loss = 0.f;
  A(cudaMemcpyAsync(tally, st.tally, sizeof tally, cudaMemcpyDeviceToHost, stream));
  A(cudaMemcpyAsync(&err, st.err, sizeof err, cudaMemcpyDeviceToHost, stream));
  if (g) {
    A(cudaMemcpyAsync(&gerr, g->d_err, sizeof gerr, cudaMemcpyDeviceToHost, stream));
    A(cudaMemcpyAsync(&loss, g->d_loss, sizeof loss, cudaMemcpyDeviceToHost, stream));
  }
  A(cudaStreamSynchronize(stream));
  if (timedAtEnd && e == cudaSuccess) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    elapsed = ms;
  }
  cudaEventDestroy(ev0);
  cudaEventDestroy(ev1);
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  for (cudaEvent_t x : {trained[0], trained[1], sampled})
    if (x) cudaEventDestroy(x);
  for (size_t k = 0; k + 1 < iev.size(); k += 2) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, iev[k], iev[k + 1]);
    infer_ms += ms;
  }
  for (cudaEvent_t x : iev) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_guided");
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->passes = passes;
    stats->train_steps = steps;
    stats->paths = pathsDone;
    stats->train_samples = tally[3];
    stats->total_ms = elapsed;
    stats->train_ms = train_ms;
    stats->last_loss = steps > 0 ? loss : 0.f;
    stats->extension_rays = tally[0];
    stats->shadow_rays = tally[1];
    stats->nonfinite = tally[2];
    stats->infer_ms = infer_ms;
    stats->infer_launches = infer_launches;
    stats->infer_rows = tally[7];
  }
  if (gerr) {
    cudaMemsetAsync(g->d_err, 0, sizeof(int), stream);
    return fail(ctx, GBRT_ERR_TIMEOUT, "gbrt_render_guided: a tensor-core wait timed out");
  }
  if (err) return fail(ctx, GBRT_ERR_NUMERIC, err_text("gbrt_render_guided", err));
  return status;
}

// -------------------------------------------------------------- batches ----
// gbrt_render_batch: every job is the wavefront of gbrt_render, enqueued on
// one of several streams without any host wait (stream-ordered buffers, the
// counters copied to pinned memory); jobs on different streams overlap.
struct JobOut {
  unsigned long long tally[8];
  int err;
  int pad;
};

static cudaError_t enqueue_job(gbrt_scene* s, const gbrt_camera& cam, const gbrt_render_params& prm, float* d_film,
                               long long cap, cudaStream_t stream, JobOut* h_out, unsigned long long* launches) {
  gbrt_ctx* ctx = s->ctx;
  const unsigned long long npix = (unsigned long long)cam.width * cam.height;
  const int spp = prm.x_samples * prm.y_samples;
  const unsigned long long total = npix * (unsigned long long)spp;
  long long B = prm.batch_paths > 0 ? prm.batch_paths : cap;
  B = std::max<long long>(1, std::min<long long>(B, (long long)total));
  PTParams P{};
  init_params(P, s->ctx, cam, prm, total);
  Buffers buf(ctx, stream);
  PTState st;
  std::memset(&st, 0, sizeof st);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  double* d_sum = nullptr;
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
  A(buf.alloc(&d_sum, npix * 3));
  if (e != cudaSuccess) return e;
  A(cudaMemsetAsync(d_sum, 0, npix * 3 * sizeof(double), stream));
  A(cudaMemsetAsync(st.tally, 0, 8 * sizeof(unsigned long long), stream));
  A(cudaMemsetAsync(st.err, 0, sizeof(int), stream));
  const TraceKernels tk = pick_kernels(s, false);
  auto kShade = pick_shade(s, P.physical != 0, false);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tk.ext, kTraceBlock, 0);
  const int traceGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, tk.sh, kTraceBlock, 0);
  const int shadowGrid = std::max(1, per) * ctx->num_sms;
  const int shadeGrid = ctx->num_sms * 8;
  for (unsigned long long g0 = 0; g0 < total && e == cudaSuccess; g0 += (unsigned long long)B) {
    P.g0 = g0;
    P.nb = int(std::min<unsigned long long>((unsigned long long)B, total - g0));
    k_raygen<<<(P.nb + 255) / 256, 256, 0, stream>>>(P, st);
    for (int it = 0; it < P.D; ++it) {
      int cur = it & 1;
      tk.ext<<<cap_grid(traceGrid, P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st, cur);
      kShade<<<cap_grid(shadeGrid, P.nb, 256), 256, 0, stream>>>(s->view, P, st, cur);
      tk.sh<<<cap_grid(shadowGrid, 2ll * P.nb, kTraceBlock), kTraceBlock, 0, stream>>>(s->view, st);
    }
    launch_accumulate(P, st, d_sum, nullptr, stream);
    *launches += 2 + 3ull * unsigned(P.D);
    A(cudaGetLastError());
  }
  const size_t n3 = size_t(npix) * 3;
  k_finalize<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(d_sum, d_film, n3, 1.0 / spp);
  *launches += 1;
  A(cudaGetLastError());
  A(cudaMemcpyAsync(h_out->tally, st.tally, sizeof h_out->tally, cudaMemcpyDeviceToHost, stream));
  A(cudaMemcpyAsync(&h_out->err, st.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
  return e;  // buf frees its arrays in stream order
}

static gbrt_status check_job(gbrt_ctx* ctx, const gbrt_batch_job& j) {
  if (!j.scene || j.scene->ctx != ctx) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch: job scene");
  const gbrt_camera& c = j.camera;
  const gbrt_render_params& p = j.params;
  if (c.width <= 0 || c.height <= 0 || p.x_samples <= 0 || p.y_samples <= 0 || p.max_depth <= 0 || p.max_depth > 64 ||
      (p.semantics != GBRT_SEM_REFERENCE && p.semantics != GBRT_SEM_PHYSICAL) ||
      !(p.termination_prob >= 0.f && p.termination_prob <= 1.f))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch: bad camera or render parameters");
  return GBRT_OK;
}

// Runs the jobs; films to device buffers, copied to the jobs' host films
// when copy_out is set. Returns per-job device milliseconds in job_ms.
static gbrt_status batch_impl(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int n, int S, long long cap, bool copy_out,
                              double* job_ms, gbrt_batch_stats* stats) {
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  while (int(ctx->batch_streams.size()) < S) {
    cudaStream_t q;
    GBRT_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    ctx->batch_streams.push_back(q);
  }
  const auto t0 = std::chrono::steady_clock::now();
  JobOut* h_out = nullptr;
  GBRT_CUDA_TRY(ctx, cudaMallocHost(&h_out, sizeof(JobOut) * size_t(n)));
  std::vector<float*> films(size_t(n), nullptr);
  std::vector<cudaEvent_t> ev(2 * size_t(n), nullptr);
  // Longest job first, each onto the stream with the least work so far
  // (paths x depth as the cost), so that the streams finish together.
  std::vector<int> order(static_cast<size_t>(n));
  std::vector<double> cost(static_cast<size_t>(n));
  for (int j = 0; j < n; ++j) {
    order[j] = j;
    const gbrt_render_params& p = jobs[j].params;
    cost[j] = double(jobs[j].camera.width) * jobs[j].camera.height * p.x_samples * p.y_samples * p.max_depth;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<double> load(static_cast<size_t>(S), 0.0);
  // Every stream starts after `begin` and records its own end, so that the
  // batch's device span is max over streams of (end - begin).
  cudaEvent_t begin = nullptr;
  std::vector<cudaEvent_t> ends(size_t(S), nullptr);
  unsigned long long launches = 0;
  cudaError_t e = cudaEventCreate(&begin);
  if (e == cudaSuccess) e = cudaEventRecord(begin, ctx->batch_streams[0]);
  for (int k = 1; k < S && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(ctx->batch_streams[k], begin, 0);
  for (int k = 0; k < n && e == cudaSuccess; ++k) {
    const int j = order[k];
    const int qi = int(std::min_element(load.begin(), load.end()) - load.begin());
    load[qi] += cost[j];
    cudaStream_t q = ctx->batch_streams[qi];
    const gbrt_camera& c = jobs[j].camera;
    std::memset(&h_out[j], 0, sizeof(JobOut));
    cudaEventCreate(&ev[2 * j]);
    cudaEventCreate(&ev[2 * j + 1]);
    e = ctx_alloc(ctx, &films[j], size_t(c.width) * c.height * 3 * sizeof(float), q);
    if (e != cudaSuccess) break;
    cudaEventRecord(ev[2 * j], q);
    e = enqueue_job(jobs[j].scene, c, jobs[j].params, films[j], cap, q, &h_out[j], &launches);
    cudaEventRecord(ev[2 * j + 1], q);
  }
  for (int k = 0; k < S; ++k) {
    if (cudaEventCreate(&ends[k]) == cudaSuccess) cudaEventRecord(ends[k], ctx->batch_streams[k]);
  }
  for (int k = 0; k < S; ++k) {
    cudaError_t r = cudaStreamSynchronize(ctx->batch_streams[k]);
    if (e == cudaSuccess) e = r;
  }
  double device_ms = 0.0;
  for (int k = 0; k < S; ++k) {
    float ms = 0.f;
    if (begin && ends[k] && cudaEventElapsedTime(&ms, begin, ends[k]) == cudaSuccess)
      device_ms = std::max(device_ms, double(ms));
    if (ends[k]) cudaEventDestroy(ends[k]);
  }
  if (begin) cudaEventDestroy(begin);
  gbrt_status status = e == cudaSuccess ? GBRT_OK : cuda_fail(ctx, e, "gbrt_render_batch");
  if (stats) std::memset(stats, 0, sizeof *stats);
  for (int j = 0; j < n; ++j) {
    if (status == GBRT_OK && copy_out && jobs[j].film) {
      const gbrt_camera& c = jobs[j].camera;
      cudaError_t r = cudaMemcpy(jobs[j].film, films[j], size_t(c.width) * c.height * 3 * sizeof(float),
                                 cudaMemcpyDeviceToHost);
      if (r != cudaSuccess) status = cuda_fail(ctx, r, "gbrt_render_batch copy-out");
    }
    if (films[j]) cudaFree(films[j]);
    float ms = 0.f;
    if (ev[2 * j] && ev[2 * j + 1]) cudaEventElapsedTime(&ms, ev[2 * j], ev[2 * j + 1]);
    if (job_ms) job_ms[j] = ms;
    if (ev[2 * j]) cudaEventDestroy(ev[2 * j]);
    if (ev[2 * j + 1]) cudaEventDestroy(ev[2 * j + 1]);
    if (status == GBRT_OK && h_out[j].err)
      status = fail(ctx, GBRT_ERR_NUMERIC, err_text("gbrt_render_batch", h_out[j].err));
    if (stats) {
      const gbrt_camera& c = jobs[j].camera;
      stats->paths += (unsigned long long)c.width * c.height * jobs[j].params.x_samples * jobs[j].params.y_samples;
      stats->extension_rays += h_out[j].tally[0];
      stats->shadow_rays += h_out[j].tally[1];
      stats->nonfinite += h_out[j].tally[2];
    }
  }
  cudaFreeHost(h_out);
  if (stats) {
    stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    stats->streams = S;
    stats->batch_paths = cap;
    stats->device_ms = device_ms;
    stats->kernel_launches = launches;
  }
  return status;
}

// The fused batch's kernels for the jobs' scenes: the general leaves if any
// scene needs them, the short stack only if every tree is shallow enough.
struct FusedKernels {
  void (*ext)(PTState, int, BatchDev);
  void (*sh)(PTState, BatchDev);
  void (*shade)(PTState, int, BatchDev);
};
template <bool W, int K, bool G>
static FusedKernels fused_trace(bool physical, bool ext) {
  FusedKernels f{k_extend_ms<W, K, G>, k_shadow_ms<W, K, G>, nullptr};
  if (physical) f.shade = ext ? k_shade_phys_ms<true> : k_shade_phys_ms<false>;
  else f.shade = ext ? k_shade_ms<true> : k_shade_ms<false>;
  return f;
}
template <bool W>
static FusedKernels fused_pick(bool shortStack, bool gen, bool physical, bool ext) {
  if (gen) return shortStack ? fused_trace<W, kShortStack, true>(physical, ext) : fused_trace<W, kStackSize, true>(physical, ext);
  return shortStack ? fused_trace<W, kShortStack, false>(physical, ext) : fused_trace<W, kStackSize, false>(physical, ext);
}

// gbrt_render_batch_fused: all jobs' paths in one numbering, wavefronts of B
// paths across jobs. P pipelines (each its own path state, job table copy,
// stream and graph) take wavefronts k, k + P, k + 2P, ...: while one
// pipeline's wavefront runs its last, nearly empty bounces, another's runs
// its full first ones.
struct FusedPipe {
  PTState st{};
  BatchDev bt{};
  BatchJob* jobs = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

static gbrt_status batch_fused_impl(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int n, const gbrt_batch_schedule& sc,
                                    bool copy_out, double* job_ms, gbrt_batch_stats* stats) {
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const auto t0 = std::chrono::steady_clock::now();
  const int traceBlock = sc.trace_block, shadeBlock = sc.shade_block, P = sc.pipelines;
  long long B = sc.wavefront_paths;
  if (n > 65535) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: more than 65,535 jobs");
  if (traceBlock != 64 && traceBlock != 128) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: trace block");
  if (shadeBlock != 128 && shadeBlock != 256) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: shade block");
  if (P < 1 || P > 8) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: pipelines outside 1..8");
  if (B < 1) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: wavefront size");
  const bool physical = jobs[0].params.semantics == GBRT_SEM_PHYSICAL;
  const bool wt = jobs[0].scene->watertight;
  bool gen = false, ext = false, shortStack = true, anyInst = false;
  int D = 0;
  unsigned long long total = 0, pixels = 0;
  // The jobs are numbered smallest first (paths x depth), so that small
  // images finish in the first wavefronts; pos[j] is job j's place.
  std::vector<int> ord(static_cast<size_t>(n)), pos(static_cast<size_t>(n));
  std::vector<double> cost(static_cast<size_t>(n));
  for (int j = 0; j < n; ++j) {
    ord[j] = j;
    const gbrt_render_params& pj = jobs[j].params;
    cost[j] = double(jobs[j].camera.width) * jobs[j].camera.height * pj.x_samples * pj.y_samples * pj.max_depth;
  }
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return cost[a] < cost[b]; });
  for (int k = 0; k < n; ++k) pos[ord[k]] = k;
  std::vector<BatchJob> hj(static_cast<size_t>(n));
  std::vector<DeviceScene> hs(static_cast<size_t>(n));
  std::vector<unsigned long long> starts(static_cast<size_t>(n));
  for (int k = 0; k < n; ++k) {
    const int j = ord[k];
    const gbrt_batch_job& jb = jobs[j];
    const gbrt_scene* scn = jb.scene;
    if ((jb.params.semantics == GBRT_SEM_PHYSICAL) != physical || scn->watertight != wt)
      return fail(ctx, GBRT_ERR_INVALID_ARG,
                  "gbrt_render_batch_fused: every job needs the same estimator and the same triangle test");
    gen = gen || scn->view.csg_prog || scn->view.inst;
    anyInst = anyInst || scn->view.inst;
    ext = ext || ext_scene(scn);
    shortStack = shortStack && stack_need(scn->max_depth4) <= kShortStack;
    D = std::max(D, jb.params.max_depth);
    const unsigned long long np = (unsigned long long)jb.camera.width * jb.camera.height;
    const unsigned long long tj = np * (unsigned long long)(jb.params.x_samples * jb.params.y_samples);
    BatchJob& b = hj[k];
    std::memset(&b, 0, sizeof b);
    init_params(b.P, ctx, jb.camera, jb.params, tj);
    b.start = total;
    b.total = tj;
    b.pix0 = pixels;
    b.group = 1;
    while (b.group < 32 && b.group < b.P.spp) b.group <<= 1;
    starts[k] = total;
    hs[k] = scn->view;
    total += tj;
    pixels += np;
  }
  B = std::min<long long>(B, (long long)total);
  if (B > (1ll << 30)) B = 1ll << 30;
  const unsigned long long waves = (total + (unsigned long long)B - 1) / (unsigned long long)B;
  const int nP = int(std::min<unsigned long long>((unsigned long long)P, waves));
  while (int(ctx->batch_streams.size()) < nP) {
    cudaStream_t q;
    GBRT_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
    ctx->batch_streams.push_back(q);
  }
  cudaStream_t stream = ctx->stream;
  Buffers buf(ctx, stream);
  cudaError_t e = cudaSuccess;
  auto A = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  DeviceScene* d_scenes = nullptr;
  unsigned long long* d_starts = nullptr;
  double* d_sum = nullptr;
  float* d_film = nullptr;
  A(buf.alloc(&d_scenes, size_t(n))); A(buf.alloc(&d_starts, size_t(n)));
  A(buf.alloc(&d_sum, size_t(pixels) * 3)); A(buf.alloc(&d_film, size_t(pixels) * 3));
  std::vector<FusedPipe> pipes(static_cast<size_t>(nP));
  for (int k = 0; k < nP && e == cudaSuccess; ++k) {
    PTState& st = pipes[k].st;
    A(buf.alloc(&st.alpha, B)); A(buf.alloc(&st.L, B)); A(buf.alloc(&st.ctl, B));
    A(buf.alloc(&st.pv_p, B)); A(buf.alloc(&st.pv_n, B)); A(buf.alloc(&st.pv_d, B)); A(buf.alloc(&st.pv_a, B));
    A(buf.alloc(&st.ext[0], 2 * B)); A(buf.alloc(&st.ext[1], 2 * B));
    A(buf.alloc(&st.ext_slot[0], B)); A(buf.alloc(&st.ext_slot[1], B));
    A(buf.alloc(&st.hits, B));
    if (anyInst) A(buf.alloc(&st.hit_inst, B));
    A(buf.alloc(&st.sh_ray, 4 * B)); A(buf.alloc(&st.sh_c, 2 * B)); A(buf.alloc(&st.sh_slot, 2 * B));
    A(buf.alloc(&st.counts, 4)); A(buf.alloc(&st.work, 4)); A(buf.alloc(&st.tally, 8)); A(buf.alloc(&st.err, 1));
    st.ext_cap = int(B);
    st.sh_cap = int(2 * B);
    BatchDev& bt = pipes[k].bt;
    A(buf.alloc(&pipes[k].jobs, size_t(n)));
    A(buf.alloc(&bt.job_of, size_t(B))); A(buf.alloc(&bt.cursor, 4));
    bt.scenes = d_scenes;
    bt.jobs = pipes[k].jobs;
    bt.starts = d_starts;
    bt.sum = d_sum;
    bt.film = d_film;
    bt.stride = (unsigned long long)nP * (unsigned long long)B;
    bt.n_jobs = n;
    bt.B = int(B);
    bt.shared_sum = nP > 1 ? 1 : 0;
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_batch_fused buffers");
  std::vector<unsigned long long> cur0(4 * size_t(nP));
  for (int k = 0; k < nP; ++k) {
    cur0[4 * k] = (unsigned long long)k * (unsigned long long)B;
    cur0[4 * k + 1] = 0;
    cur0[4 * k + 2] = total;
    cur0[4 * k + 3] = 0;
  }
  A(cudaMemcpyAsync(d_scenes, hs.data(), hs.size() * sizeof(DeviceScene), cudaMemcpyHostToDevice, stream));
  A(cudaMemcpyAsync(d_starts, starts.data(), starts.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                    stream));
  A(cudaMemsetAsync(d_sum, 0, size_t(pixels) * 3 * sizeof(double), stream));
  for (int k = 0; k < nP; ++k) {
    A(cudaMemcpyAsync(pipes[k].jobs, hj.data(), hj.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, stream));
    A(cudaMemcpyAsync(pipes[k].bt.cursor, &cur0[4 * k], 4 * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                      stream));
    A(cudaMemsetAsync(pipes[k].st.tally, 0, 8 * sizeof(unsigned long long), stream));
    A(cudaMemsetAsync(pipes[k].st.err, 0, sizeof(int), stream));
  }
  // The host arrays must outlive the copies; the pipelines start after them.
  A(cudaStreamSynchronize(stream));
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_batch_fused set-up");

  const FusedKernels fk = wt ? fused_pick<true>(shortStack, gen, physical, ext)
                             : fused_pick<false>(shortStack, gen, physical, ext);
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fk.ext, traceBlock, 0);
  const int traceGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fk.sh, traceBlock, 0);
  const int shadowGrid = std::max(1, per) * ctx->num_sms;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fk.shade, shadeBlock, 0);
  const int shadeGrid = std::max(1, per) * ctx->num_sms;
  // lanes of a job in a wavefront: (its paths / spp + 2 partial pixels) x
  // group, group < 2 spp and <= 32, rounded up to a warp: at most 2 paths + 155
  const unsigned long long lanes = 2ull * (unsigned long long)B + 160ull * (unsigned long long)n;
  // One wavefront of one pipeline as a graph: grids sized for a full
  // wavefront; the kernels read the wavefront's actual size from the device.
  for (int k = 0; k < nP && e == cudaSuccess; ++k) {
    cudaStream_t q = ctx->batch_streams[k];
    const PTState& st = pipes[k].st;
    const BatchDev& bt = pipes[k].bt;
    A(cudaStreamBeginCapture(q, cudaStreamCaptureModeThreadLocal));
    if (e != cudaSuccess) break;
    k_batch_begin<<<1, 1024, 0, q>>>(bt, st);
    k_raygen_ms<<<unsigned((B + 255) / 256), 256, 0, q>>>(st, bt);
    for (int it = 0; it < D; ++it) {
      const int cur = it & 1;
      fk.ext<<<cap_grid(traceGrid, B, traceBlock), traceBlock, 0, q>>>(st, cur, bt);
      fk.shade<<<cap_grid(shadeGrid, B, shadeBlock), shadeBlock, 0, q>>>(st, cur, bt);
      fk.sh<<<cap_grid(shadowGrid, 2 * B, traceBlock), traceBlock, 0, q>>>(st, bt);
    }
    k_accumulate_ms<<<unsigned((lanes + 255) / 256), 256, 0, q>>>(st, bt);
    k_batch_end<<<1, 32, 0, q>>>(bt);
    cudaError_t ce = cudaStreamEndCapture(q, &pipes[k].graph);
    A(cudaGetLastError());
    A(ce);
    if (e == cudaSuccess) A(cudaGraphInstantiate(&pipes[k].exec, pipes[k].graph, 0));
  }
  auto destroy_graphs = [&]() {
    for (FusedPipe& fp : pipes) {
      if (fp.exec) cudaGraphExecDestroy(fp.exec);
      if (fp.graph) cudaGraphDestroy(fp.graph);
    }
  };
  if (e != cudaSuccess) {
    destroy_graphs();
    return cuda_fail(ctx, e, "gbrt_render_batch_fused graph");
  }
  // Pipeline k runs wavefronts k, k + nP, ...; ev[w] is recorded on its
  // stream after wavefront w.
  std::vector<cudaEvent_t> ev(size_t(waves), nullptr);
  for (auto& x : ev) cudaEventCreate(&x);
  cudaEvent_t begin = nullptr, done = nullptr;
  cudaEventCreate(&begin);
  cudaEventCreate(&done);
  cudaEventRecord(begin, stream);
  for (int k = 0; k < nP; ++k) A(cudaStreamWaitEvent(ctx->batch_streams[k], begin, 0));
  for (unsigned long long w = 0; w < waves && e == cudaSuccess; ++w) {
    const int k = int(w % (unsigned long long)nP);
    A(cudaGraphLaunch(pipes[k].exec, ctx->batch_streams[k]));
    cudaEventRecord(ev[w], ctx->batch_streams[k]);
  }
  for (int k = 0; k < nP; ++k) A(cudaStreamWaitEvent(stream, ev[waves - 1 - (waves - 1 - k) % nP], 0));
  cudaEventRecord(done, stream);
  const unsigned long long n3 = pixels * 3;
  k_finalize_ms<<<unsigned((n3 + 255) / 256), 256, 0, stream>>>(pipes[0].bt, n3);
  A(cudaGetLastError());
  std::vector<unsigned long long> tally(8 * size_t(nP), 0ull);
  std::vector<int> err(size_t(nP), 0);
  for (int k = 0; k < nP; ++k) {
    A(cudaMemcpyAsync(&tally[8 * k], pipes[k].st.tally, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                      stream));
    A(cudaMemcpyAsync(&err[k], pipes[k].st.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
  }
  if (copy_out) {
    for (int j = 0; j < n && e == cudaSuccess; ++j) {
      if (!jobs[j].film) continue;
      const size_t np = size_t(jobs[j].camera.width) * jobs[j].camera.height;
      A(cudaMemcpyAsync(jobs[j].film, d_film + 3 * hj[pos[j]].pix0, np * 3 * sizeof(float), cudaMemcpyDeviceToHost,
                        stream));
    }
  }
  A(cudaStreamSynchronize(stream));
  double device_ms = 0.0;
  if (e == cudaSuccess) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, begin, done);
    device_ms = ms;
    for (int j = 0; j < n && job_ms; ++j) {
      // the wavefront that holds the job's last path
      const BatchJob& b = hj[pos[j]];
      const unsigned long long w = (b.start + b.total - 1) / (unsigned long long)B;
      float t = 0.f;
      cudaEventElapsedTime(&t, begin, ev[w]);
      job_ms[j] = t;
    }
  }
  for (auto& x : ev) cudaEventDestroy(x);
  cudaEventDestroy(begin);
  cudaEventDestroy(done);
  destroy_graphs();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gbrt_render_batch_fused");
  int anyErr = 0;
  for (int k = 0; k < nP; ++k) anyErr |= err[k];
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->paths = total;
    for (int k = 0; k < nP; ++k) {
      stats->extension_rays += tally[8 * k];
      stats->shadow_rays += tally[8 * k + 1];
      stats->nonfinite += tally[8 * k + 2];
    }
    stats->wall_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    stats->streams = nP;
    stats->batch_paths = B;
    stats->device_ms = device_ms;
    stats->kernel_launches = waves * (4ull + 3ull * unsigned(D)) + 1ull;
  }
  if (anyErr) return fail(ctx, GBRT_ERR_NUMERIC, err_text("gbrt_render_batch_fused", anyErr));
  return GBRT_OK;
}

}  // namespace gbrt

using namespace gbrt;

extern "C" {

gbrt_status gbrt_render_device(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm, float* d_film,
                               double* d_sum, double* d_sumsq, gbrt_stats* stats) {
  if (!s) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_device: NULL scene");
  clear_error(s->ctx);
  return render_impl(s, cam, prm, d_film, d_sum, d_sumsq, nullptr, stats);
}

gbrt_status gbrt_render(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm, float* film,
                        double* sum, double* sumsq, const volatile int32_t* stop, gbrt_stats* stats) {
  if (!s || !cam || !film) return fail(s ? s->ctx : nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render: NULL argument");
  gbrt_ctx* ctx = s->ctx;
  clear_error(ctx);
  if (cam->width <= 0 || cam->height <= 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render: bad resolution");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  size_t n3 = size_t(cam->width) * cam->height * 3;
  float* d_film = nullptr;
  double* d_sum = nullptr;
  double* d_sq = nullptr;
  cudaError_t e = ctx_alloc(ctx, &d_film, n3 * sizeof(float), ctx->stream);
  if (e == cudaSuccess && sum) e = ctx_alloc(ctx, &d_sum, n3 * sizeof(double), ctx->stream);
  if (e == cudaSuccess && sumsq) e = ctx_alloc(ctx, &d_sq, n3 * sizeof(double), ctx->stream);
  gbrt_status st = e == cudaSuccess ? GBRT_OK : cuda_fail(ctx, e, "gbrt_render buffers");
  if (st == GBRT_OK) st = render_impl(s, cam, prm, d_film, d_sum, d_sq, stop, stats);
  if (st == GBRT_OK || st == GBRT_ERR_CANCELLED) {
    cudaMemcpyAsync(film, d_film, n3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    if (sum) cudaMemcpyAsync(sum, d_sum, n3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    if (sumsq) cudaMemcpyAsync(sumsq, d_sq, n3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  }
  if (d_film) cudaFreeAsync(d_film, ctx->stream);
  if (d_sum) cudaFreeAsync(d_sum, ctx->stream);
  if (d_sq) cudaFreeAsync(d_sq, ctx->stream);
  e = cudaStreamSynchronize(ctx->stream);
  if (st == GBRT_OK && e != cudaSuccess) st = cuda_fail(ctx, e, "gbrt_render copy-out");
  return st;
}

gbrt_status gbrt_render_passes(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                               int32_t first_pass, int32_t n_passes, float* d_film, double* d_sum, double* d_sumsq,
                               gbrt_stats* stats) {
  if (!s) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_passes: NULL scene");
  gbrt_ctx* ctx = s->ctx;
  clear_error(ctx);
  if (!cam || !prm || !d_film || !d_sum || first_pass < 0 || n_passes <= 0 ||
      int64_t(first_pass) + n_passes > (int64_t(1) << 30))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_passes: bad argument");
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  const size_t n3 = size_t(std::max(cam->width, 0)) * size_t(std::max(cam->height, 0)) * 3;
  if (first_pass == 0) {
    GBRT_CUDA_TRY(ctx, cudaMemsetAsync(d_sum, 0, n3 * sizeof(double), ctx->stream));
    if (d_sumsq) GBRT_CUDA_TRY(ctx, cudaMemsetAsync(d_sumsq, 0, n3 * sizeof(double), ctx->stream));
  }
  const double spp = double(prm->x_samples) * double(prm->y_samples);
  gbrt_stats total;
  std::memset(&total, 0, sizeof total);
  for (int32_t k = 0; k < n_passes; ++k) {
    const int32_t pass = first_pass + k;
    gbrt_render_params p = *prm;
    p.seed = pass_seed(prm->seed, pass);
    gbrt_stats st;
    // the film of the last pass: all passes so far
    const double scale = 1.0 / (double(pass + 1) * spp);
    gbrt_status r = render_impl(s, cam, &p, d_film, d_sum, d_sumsq, nullptr, &st, true, scale);
    if (r != GBRT_OK) return r;
    total.paths += st.paths;
    total.extension_rays += st.extension_rays;
    total.shadow_rays += st.shadow_rays;
    total.nonfinite += st.nonfinite;
    total.render_ms += st.render_ms;
    total.kernel_launches += st.kernel_launches;
  }
  if (stats) *stats = total;
  return GBRT_OK;
}

gbrt_status gbrt_render_device_noalloc(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                                       float* d_film, double* d_sum, double* d_sumsq, gbrt_stats* stats) {
  if (!s) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_device_noalloc: NULL scene");
  clear_error(s->ctx);
  return render_noalloc_impl(s, cam, prm, d_film, d_sum, d_sumsq, stats);
}

gbrt_status gbrt_render_guided(gbrt_scene* s, const gbrt_camera* cam, const gbrt_render_params* prm,
                               gbrt_guide* guide, const gbrt_guide_params* gp, float* film,
                               gbrt_guide_stats* stats) {
  if (!s) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_render_guided: NULL scene");
  clear_error(s->ctx);
  return render_guided_impl(s, cam, prm, guide, gp, film, stats);
}

}  // extern "C"

extern "C" {

gbrt_status gbrt_render_batch(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int32_t n, int32_t streams,
                              int64_t batch_paths, double* job_ms, gbrt_batch_stats* stats) {
  if (!ctx || (n > 0 && !jobs) || n < 0 || streams < 0 || streams > 64 || batch_paths < 0)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch: bad argument");
  clear_error(ctx);
  for (int j = 0; j < n; ++j) {
    gbrt_status st = check_job(ctx, jobs[j]);
    if (st != GBRT_OK) return st;
    if (!jobs[j].film) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch: job without a film");
  }
  const int S = streams > 0 ? streams : ctx->batch_streams_tuned;
  const long long cap = batch_paths > 0 ? batch_paths : ctx->batch_paths_tuned;
  if (n == 0) {
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      stats->streams = S;
      stats->batch_paths = cap;
    }
    return GBRT_OK;
  }
  return batch_impl(ctx, jobs, n, S, cap, true, job_ms, stats);
}

gbrt_status gbrt_batch_autotune(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int32_t n, int32_t* streams,
                                int64_t* batch_paths) {
  if (!ctx || !jobs || n <= 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_batch_autotune: bad argument");
  clear_error(ctx);
  // A sample of the jobs at one sample per pixel. Wavefronts of 2^22 and
  // 2^24 paths only: at one sample per pixel an image of up to 2^20 pixels
  // fits a 2^20-path wavefront whole, so that size wins on the sample by
  // noise, while on the full jobs it means four times the launches (the
  // 64-scene batch: 539M paths/s against 734-746M with 2^22).
  std::vector<gbrt_batch_job> sample(jobs, jobs + std::min<int32_t>(n, 8));
  for (auto& j : sample) {
    gbrt_status st = check_job(ctx, j);
    if (st != GBRT_OK) return st;
    j.params.x_samples = 1;
    j.params.y_samples = 1;
    j.params.batch_paths = 0;
  }
  double best = 0.0;
  int bestS = ctx->batch_streams_tuned;
  long long bestB = ctx->batch_paths_tuned;
  for (long long B : {1ll << 22, 1ll << 24}) {
    for (int S : {1, 2, 4, 8}) {
      gbrt_batch_stats st;
      gbrt_status r = batch_impl(ctx, sample.data(), int(sample.size()), S, B, false, nullptr, &st);  // warm-up
      if (r == GBRT_OK) r = batch_impl(ctx, sample.data(), int(sample.size()), S, B, false, nullptr, &st);
      if (r != GBRT_OK) return r;
      double rate = double(st.paths) / std::max(st.wall_ms, 1e-6);
      if (rate > best) {
        best = rate;
        bestS = S;
        bestB = B;
      }
    }
  }
  ctx->batch_streams_tuned = bestS;
  ctx->batch_paths_tuned = bestB;
  if (streams) *streams = bestS;
  if (batch_paths) *batch_paths = bestB;
  return GBRT_OK;
}

gbrt_status gbrt_render_batch_fused(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int32_t n,
                                    const gbrt_batch_schedule* schedule, double* job_ms, gbrt_batch_stats* stats) {
  if (!ctx || (n > 0 && !jobs) || n < 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: bad argument");
  clear_error(ctx);
  for (int j = 0; j < n; ++j) {
    gbrt_status st = check_job(ctx, jobs[j]);
    if (st != GBRT_OK) return st;
    if (!jobs[j].film) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: job without a film");
  }
  gbrt_batch_schedule sc = ctx->fused_tuned;
  if (schedule) {
    if (schedule->wavefront_paths < 0 || schedule->pipelines < 0 || schedule->trace_block < 0 ||
        schedule->shade_block < 0)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_render_batch_fused: negative schedule value");
    if (schedule->wavefront_paths > 0) sc.wavefront_paths = schedule->wavefront_paths;
    if (schedule->pipelines > 0) sc.pipelines = schedule->pipelines;
    if (schedule->trace_block > 0) sc.trace_block = schedule->trace_block;
    if (schedule->shade_block > 0) sc.shade_block = schedule->shade_block;
  }
  if (n == 0) {
    if (stats) {
      std::memset(stats, 0, sizeof *stats);
      stats->batch_paths = sc.wavefront_paths;
      stats->streams = sc.pipelines;
    }
    return GBRT_OK;
  }
  return batch_fused_impl(ctx, jobs, n, sc, true, job_ms, stats);
}

gbrt_status gbrt_batch_autotune_fused(gbrt_ctx* ctx, const gbrt_batch_job* jobs, int32_t n,
                                      gbrt_batch_schedule* out) {
  if (!ctx || !jobs || n <= 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_batch_autotune_fused: bad argument");
  clear_error(ctx);
  // Every job at up to 2 x 2 samples per pixel: the mix of images a
  // wavefront holds is what the schedule is tuned for.
  std::vector<gbrt_batch_job> sample(jobs, jobs + n);
  for (auto& j : sample) {
    gbrt_status st = check_job(ctx, j);
    if (st != GBRT_OK) return st;
    j.params.x_samples = std::min(j.params.x_samples, 2);
    j.params.y_samples = std::min(j.params.y_samples, 2);
  }
  double best = 0.0;
  gbrt_batch_schedule bestS = ctx->fused_tuned;
  for (long long B : {1ll << 20, 1ll << 22, 1ll << 24}) {
    for (int P : {1, 2, 4}) {
      if ((long long)P * B > (1ll << 25)) continue;  // at most 2^25 paths of state in flight
      for (int tb : {64, 128}) {
        for (int sb : {128, 256}) {
          gbrt_batch_schedule sc{};
          sc.wavefront_paths = B;
          sc.pipelines = P;
          sc.trace_block = tb;
          sc.shade_block = sb;
          gbrt_batch_stats st;
          gbrt_status r = batch_fused_impl(ctx, sample.data(), n, sc, false, nullptr, &st);  // warm-up
          if (r == GBRT_OK) r = batch_fused_impl(ctx, sample.data(), n, sc, false, nullptr, &st);
          if (r != GBRT_OK) return r;
          const double rate = double(st.paths) / std::max(st.device_ms, 1e-6);
          if (rate > best) {
            best = rate;
            bestS = sc;
          }
        }
      }
    }
  }
  ctx->fused_tuned = bestS;
  if (out) *out = bestS;
  return GBRT_OK;
}

}  // extern "C"

// The Markov-chain renderers (Metropolis, energy redistribution) share this
// translation unit's wavefront kernels.
#include "chains.cuh"
