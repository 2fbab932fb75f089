// scene.cpp — context and scene objects of the C ABI: validation of the scene
// description, flattening into leaf-ordered primitive records, the SAH BVH
// build and the upload to HBM.
//
// Replaces scene_builder::getScene (src/sceneast.cpp:673-695), which wraps the
// lights and the scene in an IntersectableList and calls createBVH
// (src/intersectable.cpp:11-14, src/bvh.cpp:67-94). Primitive ids follow the
// type order documented in include/gbrt.h.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "bvh_build.h"
#include "bvh_gpu.h"
#include "gbrt_internal.h"

namespace gbrt {

static std::mutex g_err_mu;
static std::string g_last_error;

gbrt_status fail(gbrt_ctx* ctx, gbrt_status st, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_last_error = msg;
  return st;
}

gbrt_status cuda_fail(gbrt_ctx* ctx, cudaError_t e, const char* what) {
  std::string msg = std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " + what;
  return fail(ctx, e == cudaErrorMemoryAllocation ? GBRT_ERR_OOM : GBRT_ERR_CUDA, msg);
}

void clear_error(gbrt_ctx* ctx) {
  if (ctx) ctx->last_error.clear();
}

namespace {

// QVector3D-style helpers in float without contraction (the host code is built
// with -ffp-contract=off).
struct F3 {
  float x, y, z;
};
F3 f3(const float* p) { return {p[0], p[1], p[2]}; }
F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
bool isNull(F3 a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
// QVector3D::normalized (double length, unit vectors left unchanged).
F3 normalized(F3 a) {
  double l = double(a.x) * a.x + double(a.y) * a.y + double(a.z) * a.z;
  if (std::fabs(l - 1.0) <= 1e-12) return a;
  if (std::fabs(l) > 1e-12) {
    double s = std::sqrt(l);
    return {float(a.x / s), float(a.y / s), float(a.z / s)};
  }
  return {0.f, 0.f, 0.f};
}
float length(F3 a) { return float(std::sqrt(double(a.x) * a.x + double(a.y) * a.y + double(a.z) * a.z)); }
bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }
float lumBGR(const float* c) { return float(.299 * c[2] + .587 * c[1] + .114 * c[0]); }

struct Rec {
  float v[12];
  int32_t meta[4];
};

void setW(float& slot, int32_t bits) { std::memcpy(&slot, &bits, 4); }

template <typename T>
gbrt_status upload(gbrt_scene* s, const std::vector<T>& host, const T** dst) {
  *dst = nullptr;
  if (host.empty()) return GBRT_OK;
  void* p = nullptr;
  size_t bytes = host.size() * sizeof(T);
  GBRT_CUDA_TRY(s->ctx, fault_alloc(s->ctx));
  GBRT_CUDA_TRY(s->ctx, cudaMalloc(&p, bytes));
  s->allocations.push_back(p);
  GBRT_CUDA_TRY(s->ctx, cudaMemcpy(p, host.data(), bytes, cudaMemcpyHostToDevice));
  *dst = static_cast<const T*>(p);
  return GBRT_OK;
}

// Uploads records and meta in input order and gathers them into the leaf
// order of a GPU-built tree (order: leaf position -> input index).
gbrt_status gather_leaf_order(gbrt_scene* s, const std::vector<float4>& recv, const std::vector<int4>& meta,
                              const unsigned* order) {
  const float4* rin = nullptr;
  const int4* min_ = nullptr;
  std::vector<void*> keep;
  keep.swap(s->allocations);
  gbrt_status st = upload(s, recv, &rin);
  if (st == GBRT_OK) st = upload(s, meta, &min_);
  std::vector<void*> temps;
  temps.swap(s->allocations);
  s->allocations.swap(keep);
  void *rout = nullptr, *mout = nullptr;
  if (st == GBRT_OK) {
    cudaError_t e = cudaMalloc(&rout, recv.size() * sizeof(float4));
    if (e == cudaSuccess) s->allocations.push_back(rout);
    if (e == cudaSuccess) e = cudaMalloc(&mout, meta.size() * sizeof(int4));
    if (e == cudaSuccess) s->allocations.push_back(mout);
    if (e == cudaSuccess)
      e = gpu_gather_records(rin, min_, order, int64_t(meta.size()), static_cast<float4*>(rout),
                             static_cast<int4*>(mout), s->ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(s->ctx, e, "gbrt_scene_create: record gather");
  }
  for (void* p : temps) cudaFree(p);
  if (st == GBRT_OK) {
    s->view.recs = static_cast<const float4*>(rout);
    s->view.meta = static_cast<const int4*>(mout);
  }
  return st;
}

// Inverse of the affine map x -> A x + t given as a row-major 3 x 4 matrix
// [A | t], computed in double from the cofactors and rounded to float (the
// oracle computes it the same way). False when A is singular.
bool affine_inverse(const float in[12], float out[12]) {
  const double a00 = in[0], a01 = in[1], a02 = in[2], a10 = in[4], a11 = in[5], a12 = in[6];
  const double a20 = in[8], a21 = in[9], a22 = in[10];
  const double c00 = a11 * a22 - a12 * a21, c01 = a12 * a20 - a10 * a22, c02 = a10 * a21 - a11 * a20;
  const double det = a00 * c00 + a01 * c01 + a02 * c02;
  if (!(det != 0.0) || !std::isfinite(det)) return false;
  const double inv[3][3] = {{c00 / det, (a02 * a21 - a01 * a22) / det, (a01 * a12 - a02 * a11) / det},
                            {c01 / det, (a00 * a22 - a02 * a20) / det, (a02 * a10 - a00 * a12) / det},
                            {c02 / det, (a01 * a20 - a00 * a21) / det, (a00 * a11 - a01 * a10) / det}};
  const double t[3] = {in[3], in[7], in[11]};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) out[4 * r + c] = float(inv[r][c]);
    out[4 * r + 3] = float(-(inv[r][0] * t[0] + inv[r][1] * t[1] + inv[r][2] * t[2]));
  }
  return true;
}

// A point through a row-major 3 x 4 affine matrix, each row summed left to
// right in float (QMatrix4x4::map of an affine matrix).
F3 map_point(const float m[12], F3 p) {
  return {((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
          ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]};
}

// Relocates the child references of a mesh's nodes to the scene-wide node and
// record arrays.
void relocate_node4(Node4& n, int64_t node0, int64_t rec0) {
  for (int k = 0; k < 4; ++k) {
    const int32_t r = n.ref[k];
    if (r == kEmptyRef) continue;
    if (r >= 0) {
      n.ref[k] = int32_t(r + node0);
    } else {
      const uint32_t lv = ~uint32_t(r);
      const uint32_t first = (lv >> 4) + uint32_t(rec0);
      n.ref[k] = int32_t(~(first << 4 | (lv & 15u)));
    }
  }
}

void free_scene(gbrt_scene* s) {
  for (void* p : s->allocations) cudaFree(p);
  s->allocations.clear();
}

// Importance-sampling tables of an environment map (DeviceScene env_marg /
// env_cond / env_dens; the sampling itself is shading.cuh env_sample). Cell
// (r, c) of the mapping's parameter square is weighted by the luminance of
// the texel its centre looks up, the way EnvironmentMap::get maps directions
// (src/environmentmap.cpp:57-65 for the angular probe, whose lookup lands
// one texel before the cell: int(x - 1) truncated, then clamped, rows bounded
// by the width and columns by the height as in the renderer), times the solid
// angle per unit parameter area at the centre (lat-long 2 pi^2 sin(theta);
// angular 4 pi^2 sin(theta) / theta, nothing outside the disc). Sums in
// double, CDFs rounded to float, each cell's density the product of its float
// CDF steps (what the sampler draws) times W x H. False for a black map.
struct EnvTables {
  std::vector<float> marg, cond, dens;
};

bool build_env_tables(const float* tex, int W, int H, int mapping, const float coef[3], EnvTables& t) {
  const double pi = 3.14159265358979323846;
  std::vector<double> w(size_t(W) * H, 0.0), rowsum(size_t(H), 0.0);
  double total = 0.0;
  for (int r = 0; r < H; ++r) {
    for (int c = 0; c < W; ++c) {
      const double u = (c + 0.5) / W, v = (r + 0.5) / H;
      double jac;
      int tr = r, tc = c;
      if (mapping == GBRT_ENV_LATLONG) {
        jac = 2.0 * pi * pi * std::sin(pi * v);
      } else {
        const double cx = 2.0 * u - 1.0, cy = 2.0 * v - 1.0, rr = std::sqrt(cx * cx + cy * cy);
        if (!(rr < 1.0)) continue;
        jac = rr > 0.0 ? 4.0 * pi * pi * std::sin(pi * rr) / (pi * rr) : 4.0 * pi * pi;
        const int x = int(u * W - 1.0), y = int(v * H - 1.0);
        tr = std::min(std::max(std::min(y, W - 1), 0), H - 1);
        tc = std::min(std::max(std::min(x, H - 1), 0), W - 1);
      }
      const float* p = tex + (size_t(tr) * W + tc) * 3;  // BGR
      const float cb = p[0] * coef[0], cg = p[1] * coef[1], cr = p[2] * coef[2];
      const double lum = 0.299 * cr + 0.587 * cg + 0.114 * cb;
      const double x = lum > 0.0 && std::isfinite(lum) ? lum * jac : 0.0;
      w[size_t(r) * W + c] = x;
      rowsum[r] += x;
    }
    total += rowsum[r];
  }
  if (!(total > 0.0) || !std::isfinite(total)) return false;
  t.marg.assign(size_t(H) + 1, 0.f);
  t.cond.assign(size_t(H) * (W + 1), 0.f);
  t.dens.assign(size_t(H) * W, 0.f);
  double acc = 0.0;
  for (int r = 0; r < H; ++r) {
    t.marg[r] = float(acc / total);
    acc += rowsum[r];
    float* cr = &t.cond[size_t(r) * (W + 1)];
    double a = 0.0;
    for (int c = 0; c < W; ++c) {
      cr[c] = rowsum[r] > 0.0 ? float(a / rowsum[r]) : float(c) / float(W);
      a += w[size_t(r) * W + c];
    }
    cr[W] = 1.f;
  }
  t.marg[H] = 1.f;
  for (int r = 0; r < H; ++r) {
    const float dm = t.marg[r + 1] - t.marg[r];
    const float* cr = &t.cond[size_t(r) * (W + 1)];
    for (int c = 0; c < W; ++c) t.dens[size_t(r) * W + c] = dm * (cr[c + 1] - cr[c]) * float(W) * float(H);
  }
  return true;
}

}  // namespace
}  // namespace gbrt

using namespace gbrt;

extern "C" {

int32_t gbrt_abi_version(void) { return GBRT_ABI_VERSION; }

const char* gbrt_last_error(const gbrt_ctx* ctx) {
  if (ctx) return ctx->last_error.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_last_error.c_str();
}

gbrt_status gbrt_ctx_create(int32_t device, gbrt_ctx** out) {
  if (!out) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_ctx_create: out is NULL");
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    return fail(nullptr, GBRT_ERR_CUDA,
                std::string("gbrt_ctx_create: no CUDA device (") + cudaGetErrorString(e) + ")");
  }
  if (device < 0 || device >= n) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_ctx_create: bad device index");
  auto* c = new (std::nothrow) gbrt_ctx();
  if (!c) return fail(nullptr, GBRT_ERR_OOM, "gbrt_ctx_create: out of host memory");
  c->device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess) { delete c; return cuda_fail(nullptr, e, "cudaSetDevice"); }
  int major = 0, minor = 0;
  cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
  cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (major * 10 + minor != 103) {
    char buf[160];
    std::snprintf(buf, sizeof buf, "gbrt_ctx_create: device %d is sm_%d%d; this library is built for sm_103a (GB300) only",
                  device, major, minor);
    delete c;
    return fail(nullptr, GBRT_ERR_UNSUPPORTED, buf);
  }
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    delete c;
    return cuda_fail(nullptr, e, "cudaStreamCreate");
  }
  if ((e = cudaMalloc(&c->d_work, sizeof(unsigned long long))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_err, sizeof(int))) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(nullptr, e, "cudaMalloc(ctx scratch)");
  }
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  if ((e = cudaMemPoolCreate(&c->pool, &props)) != cudaSuccess) {
    cudaFree(c->d_work);
    cudaFree(c->d_err);
    cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(nullptr, e, "cudaMemPoolCreate");
  }
  uint64_t keep = ~0ull;  // freed memory stays in the pool for the next call
  cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  *out = c;
  return GBRT_OK;
}

gbrt_status gbrt_ctx_destroy(gbrt_ctx* ctx) {
  if (!ctx) return GBRT_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  cudaFree(ctx->d_work);
  cudaFree(ctx->d_err);
  for (cudaStream_t s : ctx->batch_streams) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  delete ctx;
  return GBRT_OK;
}

gbrt_status gbrt_ctx_trim(gbrt_ctx* ctx, uint64_t* reserved_bytes) {
  if (!ctx) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_ctx_trim: NULL context");
  clear_error(ctx);
  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  GBRT_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  for (cudaStream_t s : ctx->batch_streams) GBRT_CUDA_TRY(ctx, cudaStreamSynchronize(s));
  GBRT_CUDA_TRY(ctx, cudaMemPoolTrimTo(ctx->pool, 0));
  if (reserved_bytes) {
    uint64_t v = 0;
    GBRT_CUDA_TRY(ctx, cudaMemPoolGetAttribute(ctx->pool, cudaMemPoolAttrReservedMemCurrent, &v));
    *reserved_bytes = v;
  }
  return GBRT_OK;
}

gbrt_status gbrt_debug_fault(gbrt_ctx* ctx, int32_t kind, int64_t arg) {
  if (!ctx) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_debug_fault: NULL context");
  clear_error(ctx);
  switch (kind) {
    case GBRT_FAULT_NONE:
      ctx->fault_alloc_countdown = -1;
      ctx->fault_nan_every = 0;
      ctx->fault_small_stack = false;
      ctx->fault_guide_wait_ns = 0;
      return GBRT_OK;
    case GBRT_FAULT_ALLOC:
      if (arg < 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_debug_fault: negative allocation count");
      ctx->fault_alloc_countdown = arg;
      return GBRT_OK;
    case GBRT_FAULT_NAN:
      if (arg < 0) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_debug_fault: negative NaN period");
      ctx->fault_nan_every = uint64_t(arg);
      return GBRT_OK;
    case GBRT_FAULT_SMALL_STACK:
      ctx->fault_small_stack = arg != 0;
      return GBRT_OK;
    case GBRT_FAULT_GUIDE_WAIT:
      if (arg < 0 || arg > 1000000000) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_debug_fault: wait outside [0, 1 s]");
      ctx->fault_guide_wait_ns = uint64_t(arg);
      return GBRT_OK;
    default:
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_debug_fault: unknown fault kind");
  }
}

gbrt_status gbrt_scene_create(gbrt_ctx* ctx, const gbrt_scene_desc* d, gbrt_scene** out) {
  if (!ctx || !d || !out) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: NULL argument");
  *out = nullptr;
  clear_error(ctx);
  auto t0 = std::chrono::steady_clock::now();
  if (d->n_materials < 0 || d->n_tri < 0 || d->n_quads < 0 || d->n_spheres < 0 || d->n_planes < 0 ||
      d->n_lights < 0)
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: negative count");
  if ((d->n_materials && !d->materials) || (d->n_tri && !d->tri_pos) || (d->n_quads && !d->quads) ||
      (d->n_spheres && !d->spheres) || (d->n_planes && !d->planes) || (d->n_lights && !d->lights))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: NULL array with a non-zero count");
  if (d->n_textures < 0 || (d->n_textures && !d->textures))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: bad texture table");
  for (int i = 0; i < d->n_textures; ++i)
    if (d->textures[i].width <= 0 || d->textures[i].height <= 0 || !d->textures[i].texels)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: texture without an image");
  if (d->n_csg < 0 || d->n_csg_nodes < 0 || (d->n_csg && (!d->csg_roots || !d->csg_nodes)))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: bad CSG tables");
  bool anyTexture = false;
  for (int i = 0; i < d->n_materials; ++i)
    if (d->materials[i].type == GBRT_MAT_TEXTURE) {
      if (d->materials[i].texture < 0 || d->materials[i].texture >= d->n_textures)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: texture material without a texture");
      anyTexture = true;
    }
  int envLights = 0;
  for (int i = 0; i < d->n_lights; ++i) {
    int ty = d->lights[i].type;
    if (ty < GBRT_LIGHT_AREA || ty > GBRT_LIGHT_CONE)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: unknown light type");
    if (ty == GBRT_LIGHT_ENV) {
      ++envLights;
      if (!d->env || !d->env->texels || d->env->width <= 0 || d->env->height <= 0)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: environment light without an image");
      if (d->env->mapping != GBRT_ENV_ANGULAR && d->env->mapping != GBRT_ENV_LATLONG)
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: unknown environment mapping");
    }
  }
  if (envLights > 1)
    return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: at most one environment map per scene");
  const int64_t nPrims = int64_t(d->n_lights) + d->n_tri + d->n_quads + d->n_spheres + d->n_planes;
  if (nPrims >= (int64_t(1) << 31) - 2) return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: too many primitives");
  const int64_t nRecs = int64_t(d->n_tri) + 2 * int64_t(d->n_quads) + d->n_spheres;
  if (nRecs + d->n_lights >= (int64_t(1) << 27))
    return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: more than 2^27 bounded primitives");

  GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
  std::vector<Rec> recs;
  std::vector<Box> boxes;
  recs.reserve(size_t(nRecs + d->n_lights));
  boxes.reserve(size_t(nRecs + d->n_lights));
  std::vector<float> nrm;  // 12 floats per smooth triangle
  auto matIndex = [&](int32_t m) { return (m >= 0 && m < d->n_materials) ? m : -1; };
  auto boxOf = [](std::initializer_list<F3> pts) {
    Box b;
    for (int k = 0; k < 3; ++k) { b.lo[k] = INFINITY; b.hi[k] = -INFINITY; }
    for (F3 p : pts) {
      const float c[3] = {p.x, p.y, p.z};
      for (int k = 0; k < 3; ++k) { b.lo[k] = std::min(b.lo[k], c[k]); b.hi[k] = std::max(b.hi[k], c[k]); }
    }
    return b;
  };
  // quadHalf: 0 for a plain triangle, 1 / 2 for the first / second triangle
  // of a quad (the traversal keeps Quad::intersect's first-triangle rule).
  auto addTri = [&](F3 p1, F3 p2, F3 p3, int32_t prim, int32_t mat, int32_t nidx, int32_t quadHalf) {
    Rec r{};
    r.v[0] = p1.x; r.v[1] = p1.y; r.v[2] = p1.z; setW(r.v[3], kRecTriangle);
    r.v[4] = p2.x; r.v[5] = p2.y; r.v[6] = p2.z; setW(r.v[7], quadHalf);
    r.v[8] = p3.x; r.v[9] = p3.y; r.v[10] = p3.z; setW(r.v[11], prim);
    r.meta[0] = prim; r.meta[1] = mat; r.meta[2] = nidx; r.meta[3] = -1;
    recs.push_back(r);
    boxes.push_back(boxOf({p1, p2, p3}));
  };

  std::vector<DevLight> lights(size_t(d->n_lights));
  int32_t pid = 0;
  int32_t envLight = -1;
  for (int i = 0; i < d->n_lights; ++i, ++pid) {
    const gbrt_light& L = d->lights[i];
    DevLight& dl = lights[i];
    std::memset(&dl, 0, sizeof dl);
    dl.type = L.type;
    dl.prim = pid;
    for (int k = 0; k < 3; ++k) {
      dl.origin[k] = L.origin[k]; dl.u[k] = L.u[k]; dl.v[k] = L.v[k]; dl.intensity[k] = L.intensity[k];
    }
    if (L.type == GBRT_LIGHT_AREA) {
      if (!finite3(L.origin) || !finite3(L.u) || !finite3(L.v))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite area light");
      F3 o = f3(L.origin), u = f3(L.u), v = f3(L.v);
      F3 n = cross(u, v);
      F3 nh = normalized(n);
      dl.normal[0] = n.x; dl.normal[1] = n.y; dl.normal[2] = n.z;
      dl.normal_len = length(n);
      dl.nhat[0] = nh.x; dl.nhat[1] = nh.y; dl.nhat[2] = nh.z;
      Rec r{};
      r.v[0] = o.x; r.v[1] = o.y; r.v[2] = o.z; setW(r.v[3], kRecParallelogram);
      r.v[4] = u.x; r.v[5] = u.y; r.v[6] = u.z; setW(r.v[7], 0);
      r.v[8] = v.x; r.v[9] = v.y; r.v[10] = v.z; setW(r.v[11], pid);
      r.meta[0] = pid; r.meta[1] = -1; r.meta[2] = -1; r.meta[3] = i;
      recs.push_back(r);
      F3 ou = {o.x + u.x, o.y + u.y, o.z + u.z}, ov = {o.x + v.x, o.y + v.y, o.z + v.z};
      F3 ouv = {ou.x + v.x, ou.y + v.y, ou.z + v.z};
      boxes.push_back(boxOf({o, ou, ov, ouv}));
    } else if (L.type == GBRT_LIGHT_POINT) {
      if (!finite3(L.origin)) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite point light");
    } else if (L.type == GBRT_LIGHT_CONE) {
      if (!finite3(L.origin) || !finite3(L.u) || !std::isfinite(L.v[0]))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite cone light");
      F3 ax = normalized(f3(L.u));
      dl.nhat[0] = ax.x; dl.nhat[1] = ax.y; dl.nhat[2] = ax.z;  // unit axis
    } else if (L.type == GBRT_LIGHT_ENV) {
      envLight = i;
    }
  }
  for (int64_t i = 0; i < d->n_tri; ++i, ++pid) {
    const float* p = d->tri_pos + 9 * i;
    if (!finite3(p) || !finite3(p + 3) || !finite3(p + 6))
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite triangle vertex");
    int32_t nidx = -1;
    if (d->tri_nrm) {
      const float* n = d->tri_nrm + 9 * i;
      F3 n1 = f3(n), n2 = f3(n + 3), n3 = f3(n + 6);
      if (!isNull(n1) && !isNull(n2) && !isNull(n3)) {
        nidx = int32_t(nrm.size() / 12);
        if (nidx < 0) return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: too many smooth triangles");
        F3 m[3] = {normalized(n1), normalized(n2), normalized(n3)};
        for (int k = 0; k < 3; ++k) { nrm.push_back(m[k].x); nrm.push_back(m[k].y); nrm.push_back(m[k].z); }
        for (int k = 0; k < 3; ++k) nrm.push_back(0.f);
      }
    }
    addTri(f3(p), f3(p + 3), f3(p + 6), pid, matIndex(d->tri_mat ? d->tri_mat[i] : 0), nidx, 0);
  }
  for (int i = 0; i < d->n_quads; ++i, ++pid) {
    const gbrt_quad& q = d->quads[i];
    for (int k = 0; k < 4; ++k)
      if (!finite3(q.p[k])) return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite quad vertex");
    // Quad(p1,p2,p3,p4) = Triangle(p1,p2,p4) + Triangle(p4,p2,p3), src/quad.h:32.
    addTri(f3(q.p[0]), f3(q.p[1]), f3(q.p[3]), pid, matIndex(q.material), -1, 1);
    addTri(f3(q.p[3]), f3(q.p[1]), f3(q.p[2]), pid, matIndex(q.material), -1, 2);
  }
  for (int i = 0; i < d->n_spheres; ++i, ++pid) {
    const gbrt_sphere& s = d->spheres[i];
    if (!finite3(s.center) || !std::isfinite(s.radius))
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite sphere");
    Rec r{};
    r.v[0] = s.center[0]; r.v[1] = s.center[1]; r.v[2] = s.center[2]; setW(r.v[3], kRecSphere);
    r.v[4] = s.radius; setW(r.v[11], pid);
    r.meta[0] = pid; r.meta[1] = matIndex(s.material); r.meta[2] = -1; r.meta[3] = -1;
    recs.push_back(r);
    float ar = std::fabs(s.radius);
    Box b;
    for (int k = 0; k < 3; ++k) { b.lo[k] = s.center[k] - ar; b.hi[k] = s.center[k] + ar; }
    boxes.push_back(b);
  }
  std::vector<float4> planes(size_t(d->n_planes));
  std::vector<int2> planeMeta(size_t(d->n_planes));
  for (int i = 0; i < d->n_planes; ++i, ++pid) {
    const gbrt_plane& pl = d->planes[i];
    planes[i] = make_float4(pl.plane[0], pl.plane[1], pl.plane[2], pl.plane[3]);
    planeMeta[i] = make_int2(pid, matIndex(pl.material));
  }
  // CSG objects: each a postfix program over the node table and one record
  // whose box is the union of its leaves' boxes (CSGOperation::
  // createBoundingBox, src/csgoperation.cpp:66-76).
  std::vector<int32_t> csgProg;
  for (int i = 0; i < d->n_csg; ++i, ++pid) {
    const int32_t start = int32_t(csgProg.size());
    int leaves = 0, visited = 0;
    Box box{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    bool ok = true;
    // post-order walk with an explicit stack; (node, children pushed)
    std::vector<std::pair<int32_t, bool>> stk{{d->csg_roots[i], false}};
    while (!stk.empty() && ok) {
      auto [nidx, expanded] = stk.back();
      stk.pop_back();
      if (nidx < 0 || nidx >= d->n_csg_nodes || ++visited > 2 * GBRT_CSG_MAX_LEAVES) { ok = false; break; }
      const gbrt_csg_node& nd = d->csg_nodes[nidx];
      if (nd.op == GBRT_CSG_SPHERE || nd.op == GBRT_CSG_BOX) {
        if (!finite3(nd.a) || !finite3(nd.b) || ++leaves > GBRT_CSG_MAX_LEAVES) { ok = false; break; }
        for (int k = 0; k < 3; ++k) {
          float lo = nd.op == GBRT_CSG_BOX ? nd.a[k] : nd.a[k] - std::fabs(nd.b[0]);
          float hi = nd.op == GBRT_CSG_BOX ? nd.b[k] : nd.a[k] + std::fabs(nd.b[0]);
          box.lo[k] = std::min(box.lo[k], lo);
          box.hi[k] = std::max(box.hi[k], hi);
        }
        csgProg.push_back(nidx);
      } else if (nd.op >= GBRT_CSG_ISECT && nd.op <= GBRT_CSG_XOR) {
        if (expanded) {
          csgProg.push_back(nidx);
        } else {
          stk.push_back({nidx, true});
          stk.push_back({nd.right, false});
          stk.push_back({nd.left, false});
        }
      } else {
        ok = false;
      }
    }
    if (!ok)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: CSG object with a bad node or more than 8 leaves");
    Rec r{};
    r.v[0] = box.lo[0]; r.v[1] = box.lo[1]; r.v[2] = box.lo[2]; setW(r.v[3], kRecCSG);
    r.v[4] = box.hi[0]; r.v[5] = box.hi[1]; r.v[6] = box.hi[2]; setW(r.v[7], start);
    setW(r.v[8], int32_t(csgProg.size()) - start); setW(r.v[11], pid);
    r.meta[0] = pid; r.meta[1] = -1; r.meta[2] = -1; r.meta[3] = -1;
    recs.push_back(r);
    boxes.push_back(box);
  }

  // Instanced meshes: every mesh an instance uses gets its own tree over its
  // triangles (in its own space); each instance is one record of the top-level
  // tree, boxed by its mesh's box through its transform, and one entry of the
  // instance table (world-to-object rows, mesh root, prim id).
  if (d->n_meshes < 0 || d->n_instances < 0 || (d->n_instances && (!d->instances || !d->meshes)))
    return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: bad mesh or instance tables");
  struct MeshTree {
    Collapsed c4;
    std::vector<Rec> recs;  // leaf order
    std::vector<int32_t> tri_index;  // per leaf-order record, its triangle's index in the mesh
    Box box;
    int64_t node0 = 0, rec0 = 0;
    bool used = false;
  };
  std::vector<MeshTree> meshTrees(size_t(d->n_meshes));
  std::vector<float4> instTab(size_t(d->n_instances) * 4);
  for (int i = 0; i < d->n_instances; ++i) {
    const gbrt_instance& in = d->instances[i];
    if (in.mesh < 0 || in.mesh >= d->n_meshes)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: instance of a mesh that does not exist");
    for (int k = 0; k < 12; ++k)
      if (!std::isfinite(in.transform[k]))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite instance transform");
    meshTrees[in.mesh].used = true;
  }
  int meshDepth = 0;
  int64_t meshRecs = 0;
  for (int m = 0; m < d->n_meshes; ++m) {
    MeshTree& mt = meshTrees[m];
    if (!mt.used) continue;
    const gbrt_mesh& gm = d->meshes[m];
    if (gm.n_tri <= 0 || !gm.tri_pos)
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: instance of an empty mesh");
    meshRecs += gm.n_tri;
    if (nRecs + d->n_lights + d->n_csg + d->n_instances + meshRecs >= (int64_t(1) << 27))
      return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: more than 2^27 bounded primitives");
    std::vector<Rec> mrecs;
    std::vector<Box> mboxes;
    mrecs.reserve(size_t(gm.n_tri));
    mboxes.reserve(size_t(gm.n_tri));
    for (int64_t i = 0; i < gm.n_tri; ++i) {
      const float* p = gm.tri_pos + 9 * i;
      if (!finite3(p) || !finite3(p + 3) || !finite3(p + 6))
        return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: non-finite mesh vertex");
      int32_t nidx = -1;
      if (gm.tri_nrm) {
        const float* n = gm.tri_nrm + 9 * i;
        F3 n1 = f3(n), n2 = f3(n + 3), n3 = f3(n + 6);
        if (!isNull(n1) && !isNull(n2) && !isNull(n3)) {
          nidx = int32_t(nrm.size() / 12);
          if (nidx < 0) return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: too many smooth triangles");
          F3 q[3] = {normalized(n1), normalized(n2), normalized(n3)};
          for (int k = 0; k < 3; ++k) { nrm.push_back(q[k].x); nrm.push_back(q[k].y); nrm.push_back(q[k].z); }
          for (int k = 0; k < 3; ++k) nrm.push_back(0.f);
        }
      }
      F3 p1 = f3(p), p2 = f3(p + 3), p3 = f3(p + 6);
      Rec r{};
      r.v[0] = p1.x; r.v[1] = p1.y; r.v[2] = p1.z; setW(r.v[3], kRecTriangle);
      r.v[4] = p2.x; r.v[5] = p2.y; r.v[6] = p2.z; setW(r.v[7], 0);
      r.v[8] = p3.x; r.v[9] = p3.y; r.v[10] = p3.z; setW(r.v[11], kMeshTriangle);
      r.meta[0] = kMeshTriangle; r.meta[1] = matIndex(gm.tri_mat ? gm.tri_mat[i] : 0); r.meta[2] = nidx;
      r.meta[3] = -1;
      mrecs.push_back(r);
      mboxes.push_back(boxOf({p1, p2, p3}));
    }
    BuildResult mbr = build_bvh(mboxes, BuildOptions());
    if (mbr.max_depth > kMaxTreeDepth)
      return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: mesh BVH deeper than the traversal stack");
    mt.recs.resize(mrecs.size());
    mt.tri_index.resize(mrecs.size());
    for (size_t k = 0; k < mbr.order.size(); ++k) {
      mt.recs[k] = mrecs[mbr.order[k]];
      mt.tri_index[k] = int32_t(mbr.order[k]);
    }
    mt.c4 = collapse_bvh4(mbr);
    meshDepth = std::max(meshDepth, mt.c4.max_depth);
    mt.box = mboxes[0];
    for (const Box& b : mboxes)
      for (int k = 0; k < 3; ++k) { mt.box.lo[k] = std::min(mt.box.lo[k], b.lo[k]); mt.box.hi[k] = std::max(mt.box.hi[k], b.hi[k]); }
  }
  for (int i = 0; i < d->n_instances; ++i, ++pid) {
    const gbrt_instance& in = d->instances[i];
    float inv[12];
    if (!affine_inverse(in.transform, inv))
      return fail(ctx, GBRT_ERR_INVALID_ARG, "gbrt_scene_create: singular instance transform");
    for (int r = 0; r < 3; ++r) instTab[4 * i + r] = make_float4(inv[4 * r], inv[4 * r + 1], inv[4 * r + 2], inv[4 * r + 3]);
    float fpid, fmesh;
    std::memcpy(&fpid, &pid, 4);
    std::memcpy(&fmesh, &in.mesh, 4);
    instTab[4 * i + 3] = make_float4(0.f, fpid, fmesh, 0.f);  // x: mesh root, set below
    const Box& mb = meshTrees[in.mesh].box;
    Box wb{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    for (int c = 0; c < 8; ++c) {
      F3 corner = {(c & 1) ? mb.hi[0] : mb.lo[0], (c & 2) ? mb.hi[1] : mb.lo[1], (c & 4) ? mb.hi[2] : mb.lo[2]};
      F3 w = map_point(in.transform, corner);
      const float wc[3] = {w.x, w.y, w.z};
      for (int k = 0; k < 3; ++k) { wb.lo[k] = std::min(wb.lo[k], wc[k]); wb.hi[k] = std::max(wb.hi[k], wc[k]); }
    }
    // the box of the mapped corners, widened by a few ulp against the
    // rounding of the ray's own transform
    for (int k = 0; k < 3; ++k) {
      const float e = 4e-6f * std::max(std::fabs(wb.lo[k]), std::fabs(wb.hi[k])) + 1e-30f;
      wb.lo[k] -= e;
      wb.hi[k] += e;
    }
    Rec r{};
    r.v[0] = wb.lo[0]; r.v[1] = wb.lo[1]; r.v[2] = wb.lo[2]; setW(r.v[3], kRecInstance);
    setW(r.v[4], i); setW(r.v[11], pid);
    r.meta[0] = pid; r.meta[1] = -1; r.meta[2] = -1; r.meta[3] = -1;
    recs.push_back(r);
    boxes.push_back(wb);
  }

  float sb[6] = {0, 0, 0, 0, 0, 0};
  for (size_t i = 0; i < boxes.size(); ++i)
    for (int k = 0; k < 3; ++k) {
      sb[k] = i ? std::min(sb[k], boxes[i].lo[k]) : boxes[i].lo[k];
      sb[3 + k] = i ? std::max(sb[3 + k], boxes[i].hi[k]) : boxes[i].hi[k];
    }
  // The BVH: on the GPU when asked (falling back to the host when the tree
  // would be too deep for the traversal stack), else binned SAH on the host.
  GpuBuild gb{};
  bool gpuBuilt = false;
  if ((d->flags & GBRT_SCENE_GPU_BUILD) && !boxes.empty() && d->n_instances == 0) {
    GBRT_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    cudaError_t ce = gpu_build_bvh4(boxes, BuildOptions().max_leaf, ctx->stream, &gb);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce, "gbrt_scene_create: GPU BVH build");
    gpuBuilt = !gb.too_deep;
  }
  BuildResult br;
  Collapsed c4;
  std::vector<float4> recv(recs.size() * 3);
  std::vector<int4> meta(recs.size());
  std::vector<float4> nodes;
  if (gpuBuilt) {
    // records in input order; the device gathers them into leaf order
    for (size_t k = 0; k < recs.size(); ++k) {
      std::memcpy(&recv[3 * k], recs[k].v, sizeof recs[k].v);
      meta[k] = make_int4(recs[k].meta[0], recs[k].meta[1], recs[k].meta[2], recs[k].meta[3]);
    }
  } else {
    BuildOptions bo;
    br = build_bvh(boxes, bo);
    if (br.max_depth > kMaxTreeDepth)
      return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: BVH deeper than the traversal stack");
    for (size_t k = 0; k < br.order.size(); ++k) {
      const Rec& r = recs[br.order[k]];
      std::memcpy(&recv[3 * k], r.v, sizeof r.v);
      meta[k] = make_int4(r.meta[0], r.meta[1], r.meta[2], r.meta[3]);
    }
    c4 = collapse_bvh4(br);
    nodes.resize(c4.nodes.size() * 8);
    if (!c4.nodes.empty()) std::memcpy(nodes.data(), c4.nodes.data(), c4.nodes.size() * sizeof(Node4));
    // the meshes' nodes and records after the top-level ones
    int64_t node0 = int64_t(c4.nodes.size()), rec0 = int64_t(recs.size());
    for (MeshTree& mt : meshTrees) {
      if (!mt.used) continue;
      mt.node0 = node0;
      mt.rec0 = rec0;
      for (Node4 n4 : mt.c4.nodes) {
        relocate_node4(n4, node0, rec0);
        const float4* f = reinterpret_cast<const float4*>(&n4);
        nodes.insert(nodes.end(), f, f + 8);
      }
      for (const Rec& r : mt.recs) {
        float4 f[3];
        std::memcpy(f, r.v, sizeof r.v);
        recv.insert(recv.end(), f, f + 3);
        meta.push_back(make_int4(r.meta[0], r.meta[1], r.meta[2], r.meta[3]));
      }
      node0 += int64_t(mt.c4.nodes.size());
      rec0 += int64_t(mt.recs.size());
    }
    for (int i = 0; i < d->n_instances; ++i) {
      const int32_t root = int32_t(meshTrees[d->instances[i].mesh].node0);
      std::memcpy(&instTab[4 * i + 3].x, &root, 4);
    }
  }

  std::vector<DevMaterial> mats(size_t(d->n_materials));
  for (int i = 0; i < d->n_materials; ++i) {
    const gbrt_material& m = d->materials[i];
    DevMaterial& dm = mats[i];
    std::memset(&dm, 0, sizeof dm);
    dm.type = (m.type >= GBRT_MAT_DARK && m.type <= GBRT_MAT_TEXTURE) ? m.type : GBRT_MAT_DARK;
    dm.tex = m.type == GBRT_MAT_TEXTURE ? m.texture : -1;
    for (int k = 0; k < 3; ++k) { dm.kd[k] = m.kd[k]; dm.ks[k] = m.ks[k]; }
    dm.exponent = m.exponent;
    dm.ior = m.ior;
    dm.rho_d = lumBGR(m.kd);
    dm.rho_s = lumBGR(m.ks);
  }

  auto* s = new (std::nothrow) gbrt_scene();
  if (!s) {
    if (gpuBuilt) {
      cudaFree(gb.nodes);
      cudaFree(gb.order);
    }
    return fail(ctx, GBRT_ERR_OOM, "gbrt_scene_create: out of host memory");
  }
  if (gpuBuilt) {
    // The scene owns the GPU-built nodes; order is freed after the gather.
    s->allocations.push_back(gb.nodes);
  }
  s->ctx = ctx;
  s->device = ctx->device;
  s->watertight = (d->flags & GBRT_SCENE_WATERTIGHT) != 0;
  DeviceScene& v = s->view;
  gbrt_status st;
  std::vector<float> envTex;
  if (gpuBuilt) {
    st = gather_leaf_order(s, recv, meta, gb.order);
    cudaFree(gb.order);
    v.nodes = gb.nodes;
    if (st != GBRT_OK) {
      free_scene(s);
      delete s;
      return st;
    }
  }
  if ((!gpuBuilt && ((st = upload(s, nodes, &v.nodes)) != GBRT_OK || (st = upload(s, recv, &v.recs)) != GBRT_OK ||
                     (st = upload(s, meta, &v.meta)) != GBRT_OK)) ||
      (st = upload(s, nrm, &v.tri_nrm)) != GBRT_OK ||
      (st = upload(s, planes, &v.planes)) != GBRT_OK || (st = upload(s, planeMeta, &v.plane_meta)) != GBRT_OK ||
      (st = upload(s, mats, &v.materials)) != GBRT_OK || (st = upload(s, lights, &v.lights)) != GBRT_OK) {
    free_scene(s);
    delete s;
    return st;
  }
  v.n_nodes = gpuBuilt ? gb.n_nodes : int64_t(nodes.size() / 8);
  v.n_recs = int64_t(meta.size());
  if (d->flags & GBRT_SCENE_LIST_ORDER) {
    // Tie-breaking by list order: each primitive's rank, and each record's
    // triangle index within its mesh (0 outside meshes; meshes exist only
    // with the host build).
    std::vector<int32_t> rank(static_cast<size_t>(pid));
    for (int32_t i = 0; i < pid; ++i) rank[size_t(i)] = d->list_rank ? d->list_rank[i] : i;
    std::vector<int32_t> sub;
    if (d->n_instances > 0 && !gpuBuilt) {
      sub.assign(size_t(v.n_recs), 0);
      for (const MeshTree& mt : meshTrees)
        if (mt.used) std::copy(mt.tri_index.begin(), mt.tri_index.end(), sub.begin() + mt.rec0);
    }
    if ((pid > 0 && (st = upload(s, rank, &v.prim_rank)) != GBRT_OK) ||
        (!sub.empty() && (st = upload(s, sub, &v.rec_sub)) != GBRT_OK)) {
      free_scene(s);
      delete s;
      return st;
    }
  }
  if (d->n_instances > 0) {
    if ((st = upload(s, instTab, &v.inst)) != GBRT_OK) {
      free_scene(s);
      delete s;
      return st;
    }
    v.n_inst = d->n_instances;
  }
  v.n_planes = d->n_planes;
  v.n_materials = d->n_materials;
  v.n_lights = d->n_lights;
  v.env_light = -1;
  if (anyTexture) {
    // Texels of all textures back to back, their table, and the triangles'
    // texture coordinates (the Triangle constructor's default without any).
    std::vector<float> texels;
    std::vector<int4> info(size_t(d->n_textures));
    for (int i = 0; i < d->n_textures; ++i) {
      const gbrt_texture& t = d->textures[i];
      info[i] = make_int4(int(texels.size() / 3), t.width, t.height, 0);
      texels.insert(texels.end(), t.texels, t.texels + size_t(t.width) * t.height * 3);
    }
    std::vector<float> uv(size_t(d->n_tri) * 6);
    for (int64_t i = 0; i < d->n_tri; ++i) {
      static const float kDefault[6] = {0, 0, 0, 1, 1, 0};
      std::memcpy(&uv[6 * i], d->tri_uv ? d->tri_uv + 6 * i : kDefault, 6 * sizeof(float));
    }
    if ((st = upload(s, texels, &v.tex_texels)) != GBRT_OK || (st = upload(s, info, &v.tex_info)) != GBRT_OK ||
        (st = upload(s, uv, &v.tri_uv)) != GBRT_OK) {
      free_scene(s);
      delete s;
      return st;
    }
    v.n_textures = d->n_textures;
  }
  v.tri_pid0 = d->n_lights;
  if (d->n_csg > 0) {
    std::vector<float4> nodes4(size_t(d->n_csg_nodes) * 3);
    for (int i = 0; i < d->n_csg_nodes; ++i) {
      const gbrt_csg_node& nd = d->csg_nodes[i];
      int32_t op = nd.op, mat = nd.op <= GBRT_CSG_BOX ? matIndex(nd.material) : -1;
      float fo, fm, fl, fr;
      std::memcpy(&fo, &op, 4); std::memcpy(&fm, &mat, 4);
      std::memcpy(&fl, &nd.left, 4); std::memcpy(&fr, &nd.right, 4);
      nodes4[3 * i] = make_float4(nd.a[0], nd.a[1], nd.a[2], fo);
      nodes4[3 * i + 1] = make_float4(nd.b[0], nd.b[1], nd.b[2], fm);
      nodes4[3 * i + 2] = make_float4(fl, fr, 0.f, 0.f);
    }
    if ((st = upload(s, nodes4, &v.csg_nodes)) != GBRT_OK || (st = upload(s, csgProg, &v.csg_prog)) != GBRT_OK) {
      free_scene(s);
      delete s;
      return st;
    }
  }
  if (envLight >= 0) {
    const gbrt_env_map* e = d->env;
    envTex.assign(e->texels, e->texels + size_t(e->width) * e->height * 3);
    if ((st = upload(s, envTex, &v.env_texels)) != GBRT_OK) {
      free_scene(s);
      delete s;
      return st;
    }
    v.env_light = envLight;
    v.env_w = e->width;
    v.env_h = e->height;
    v.env_mapping = e->mapping;
    for (int k = 0; k < 3; ++k) v.env_coef[k] = d->lights[envLight].intensity[k];
    EnvTables et;
    if (!(d->flags & GBRT_SCENE_ENV_UNIFORM) &&
        build_env_tables(e->texels, e->width, e->height, e->mapping, v.env_coef, et)) {
      if ((st = upload(s, et.marg, &v.env_marg)) != GBRT_OK || (st = upload(s, et.cond, &v.env_cond)) != GBRT_OK ||
          (st = upload(s, et.dens, &v.env_dens)) != GBRT_OK) {
        free_scene(s);
        delete s;
        return st;
      }
    }
  }
  s->n_leaves = gpuBuilt ? gb.leaves : br.leaves;
  s->max_depth = gpuBuilt ? 0 : br.max_depth;
  // two levels: the top-level tree, the way into a mesh, the mesh's tree
  s->max_depth4 = gpuBuilt ? gb.depth4 : (d->n_instances > 0 ? c4.max_depth + 1 + meshDepth : c4.max_depth);
  if (3 * s->max_depth4 + 1 > 190) {  // the traversal kernels' longest stack
    free_scene(s);
    delete s;
    return fail(ctx, GBRT_ERR_UNSUPPORTED, "gbrt_scene_create: two-level tree deeper than the traversal stack");
  }
  s->sah_cost = gpuBuilt ? 0.0 : br.sah_cost;
  s->n_prims = int32_t(nPrims + d->n_csg + d->n_instances);
  std::memcpy(s->bounds, sb, sizeof sb);
  s->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = s;
  return GBRT_OK;
}

gbrt_status gbrt_scene_destroy(gbrt_scene* s) {
  if (!s) return GBRT_OK;
  // Touches no context state, so it stays safe in any destruction order.
  cudaSetDevice(s->device);
  free_scene(s);  // cudaFree waits for work using the memory
  delete s;
  return GBRT_OK;
}

gbrt_status gbrt_scene_bounds(const gbrt_scene* s, float bounds[6]) {
  if (!s || !bounds) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_scene_bounds: NULL argument");
  std::memcpy(bounds, s->bounds, sizeof s->bounds);
  return GBRT_OK;
}

gbrt_status gbrt_scene_info(const gbrt_scene* s, int64_t* n_nodes, int64_t* n_leaves, int32_t* max_depth,
                            double* sah_cost, double* build_ms) {
  if (!s) return fail(nullptr, GBRT_ERR_INVALID_ARG, "gbrt_scene_info: NULL scene");
  if (n_nodes) *n_nodes = s->view.n_nodes;
  if (n_leaves) *n_leaves = s->n_leaves;
  if (max_depth) *max_depth = s->max_depth;
  if (sah_cost) *sah_cost = s->sah_cost;
  if (build_ms) *build_ms = s->build_ms;
  return GBRT_OK;
}

void gbrt_free(void* p) { std::free(p); }

}  // extern "C"
