// shading.cuh — per-vertex material, light and sampling math of the renderer,
// restated for the GPU in FP32 (reference semantics, quirks included):
//   Sample::getCosinePowerWeightedDirection  src/sampler.cpp:48-76
//   DiffuseMaterial / AbstractDiffuse        src/diffusematerial.cpp:25-28, src/abstractdiffusematerial.cpp:8-14
//   MirrorMaterial                           src/mirrormaterial.cpp:31-41
//   PhongMaterial                            src/phongmaterial.cpp:31-81
//   BlinnMaterial                            src/blinnmaterial.cpp:34-84
//   TransparentMaterial                      src/transparentmaterial.cpp:34-75
//   AreaLight / PointLight intensity         src/arealight.cpp:35-59, src/pointlight.cpp:29-41
//   EnvironmentMap::get / getIntensity       src/environmentmap.cpp:40-65
// plus the counter-based random stream shared with the CPU oracle.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "gbrt_scene.h"

namespace gbrt {

constexpr float kEps = 0.001f;  // EPSILON, src/ray.h:34
constexpr float kInvPi = 0.318309886183790671537767526745028724f;
constexpr float kPiF = 3.14159265358979323846f;

struct V3f {
  float x, y, z;
};
__device__ __forceinline__ V3f v3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ V3f operator+(V3f a, V3f b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3f operator-(V3f a, V3f b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3f operator-(V3f a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3f operator*(float s, V3f a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3f mulc(V3f a, V3f b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot(V3f a, V3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3f cross(V3f a, V3f b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float len2(V3f a) { return dot(a, a); }
__device__ __forceinline__ float len(V3f a) { return sqrtf(dot(a, a)); }
// QVector3D::normalized: the zero vector stays zero.
__device__ __forceinline__ V3f normalize(V3f a) {
  float l2 = dot(a, a);
  if (!(l2 > 1e-24f)) return {0.f, 0.f, 0.f};
  float s = rsqrtf(l2);
  return {a.x * s, a.y * s, a.z * s};
}
__device__ __forceinline__ bool is_zero(V3f a) { return a.x == 0.f && a.y == 0.f && a.z == 0.f; }
__device__ __forceinline__ int signum(float x) { return (0.f < x) - (x < 0.f); }
__device__ __forceinline__ V3f reflect(V3f v, V3f n) { return v - (2.f * dot(v, n)) * n; }
__device__ __forceinline__ V3f ld3(const float* p) { return {p[0], p[1], p[2]}; }

// ---------------------------------------------------------------- RNG -----
// SplitMix64 output function (Steele, Lea, Flood 2014). One camera sample
// owns the stream key = mix64(seed ^ mix64(sample_id + c)); its d-th uniform
// is the top 24 bits of mix64(key + d * phi). The CPU oracle defines the same
// stream, so both can draw identical numbers.
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ unsigned long long stream_key(unsigned long long seed, unsigned long long sample_id) {
  return mix64(seed ^ mix64(sample_id + 0x632BE59BD9B4E019ull));
}
// The top 24 bits of the d-th draw; stream_u is this value / 2^24.
__host__ __device__ __forceinline__ unsigned stream_bits(unsigned long long key, unsigned dim) {
  return unsigned(mix64(key + (unsigned long long)dim * 0x9E3779B97F4A7C15ull) >> 40);
}
__host__ __device__ __forceinline__ float stream_u(unsigned long long key, unsigned dim) {
  return float(stream_bits(key, dim)) * (1.0f / 16777216.0f);
}
// floor(u * n) for u = bits / 2^24, exactly, in integer arithmetic.
__device__ __forceinline__ int stream_index(unsigned long long key, unsigned dim, int n) {
  return int((unsigned long long)stream_bits(key, dim) * unsigned(n) >> 24);
}
// Dimension layout per camera sample (D = max depth):
//   0,1 jitter | 2 path length | 3+2i, 4+2i path sample i |
//   3+2D+3k, +1 light sample k, +2 light index k
__device__ __forceinline__ unsigned dim_path(int i) { return 3u + 2u * unsigned(i); }
__device__ __forceinline__ unsigned dim_light(int D, int k) { return 3u + 2u * unsigned(D) + 3u * unsigned(k); }

// ----------------------------------------------------------- Sampling -----
// Cosine-power direction about w, src/sampler.cpp:48-76 (opening angle pi/2).
__device__ __forceinline__ V3f cosine_power_dir(V3f w, float sx, float sy, float e, float& pdf) {
  w = normalize(w);
  float ie = 1.f / (e + 1.f);
  float z = powf(sx, ie);
  float r = sqrtf(fmaxf(0.f, 1.f - powf(sx, 2.f * ie)));
  float sn, cs;
  sincospif(2.f * sy, &sn, &cs);
  V3f nd = v3(cs * r, sn * r, z);
  pdf = powf(z, e) * (e + 1.f) * (0.5f * kInvPi);
  V3f v;
  float ax = fabsf(w.x), ay = fabsf(w.y), az = fabsf(w.z);
  if (ax < ay && ax < az) v = v3(0.f, w.z, -w.y);
  else if (ay < az) v = v3(w.z, 0.f, -w.x);
  else v = v3(w.y, -w.x, 0.f);
  v = normalize(v);
  V3f u = cross(v, w);
  return normalize(nd.x * u + nd.y * v + nd.z * w);
}

// ---------------------------------------------------------------- CSG -----
// Surface of a CSG hit (leaf node index in the hit's u): the leaf's material;
// a sphere leaf's normal x - centre and texture coordinates as a sphere's
// (src/sphere.cpp:44-50); a box leaf's normal that of its slab entry face,
// also for the exit boundary, and texture coordinates (0, 0)
// (src/axisalignedbox.cpp:41-68). The slab is recomputed with the traversal's
// roundings so that the entry face is the one the hit came from.
__device__ __forceinline__ void csg_surface(const DeviceScene& S, int leaf, V3f o, V3f d, V3f x, V3f& n, int& mat,
                                            float& tu, float& tv) {
  const float4 A = __ldg(S.csg_nodes + 3 * leaf), B = __ldg(S.csg_nodes + 3 * leaf + 1);
  mat = __float_as_int(B.w);
  tu = 0.f;
  tv = 0.f;
  if (__float_as_int(A.w) == GBRT_CSG_SPHERE) {
    const V3f nn = x - v3(A.x, A.y, A.z);
    n = normalize(nn);
    tu = acosf(nn.z / B.x) * kInvPi;
    tv = atan2f(nn.x, nn.y) * (0.5f * kInvPi) + 0.5f;
    return;
  }
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  const float lo[3] = {A.x, A.y, A.z}, hi[3] = {B.x, B.y, B.z};
  float tmin = -CUDART_INF_F;
  float nr[3] = {0.f, 0.f, 0.f};
  for (int k = 0; k < 3; ++k) {
    const float inv = __fdiv_rn(1.f, dd[k]);
    const float tn = __fmul_rn(inv >= 0.f ? __fsub_rn(lo[k], oo[k]) : __fsub_rn(hi[k], oo[k]), inv);
    if (tn > tmin) {
      tmin = tn;
      nr[0] = nr[1] = nr[2] = 0.f;
      nr[k] = inv >= 0.f ? -1.f : 1.f;
    }
  }
  n = v3(nr[0], nr[1], nr[2]);
}

// --------------------------------------------------------- Materials -----
struct Vertex {
  V3f p;     // hit point
  V3f n;     // normalised surface normal (unflipped)
  V3f d;     // direction of the ray that hit it (unnormalised)
  int mat;   // material index, -1 = DarkMatter
  float tu, tv;  // texture coordinates (HitRecord::getTexCoords)
};

// ----------------------------------------------------------- Textures -----
// (The shading kernels take texture and CSG code only in their EXT
// instantiation, for scenes that have either: it costs registers.)
// Texture coordinates of a hit, HitRecord::getTexCoords: a triangle's
// (1 - u - v) t1 + u t2 + v t3 (src/triangle.cpp:54) in the renderer's
// operation order; a quad's halves carry the Triangle constructor's default
// (0,0), (0,1), (1,0) (src/triangle.h:35, src/quad.h:32); a sphere's
// (acos(n.z / r) / pi, atan2(n.x, n.y) / 2pi + 1/2) with n = x - centre
// (src/sphere.cpp:44-50); other primitives (0, 0).
__device__ __forceinline__ void hit_texcoords(const DeviceScene& S, int rec, float u, float v, V3f x, float& tu,
                                              float& tv) {
  tu = 0.f;
  tv = 0.f;
  if (!S.tri_uv || rec < 0) return;
  const float4* rp = S.recs + 3 * int64_t(rec);
  const float4 a = __ldg(rp);
  const int kind = __float_as_int(a.w);
  if (kind == kRecSphere) {
    const float r = __ldg(rp + 1).x;
    const V3f n = x - v3(a.x, a.y, a.z);
    tu = acosf(n.z / r) * kInvPi;
    tv = atan2f(n.x, n.y) * (0.5f * kInvPi) + 0.5f;
    return;
  }
  if (kind != kRecTriangle) return;
  const float w0 = __fsub_rn(__fsub_rn(1.f, u), v);
  if (__float_as_int(__ldg(rp + 1).w) != 0) {
    tu = __fadd_rn(__fadd_rn(__fmul_rn(w0, 0.f), __fmul_rn(u, 0.f)), __fmul_rn(v, 1.f));
    tv = __fadd_rn(__fadd_rn(__fmul_rn(w0, 0.f), __fmul_rn(u, 1.f)), __fmul_rn(v, 0.f));
    return;
  }
  const int64_t tri = int64_t(__ldg(&S.meta[rec]).x) - S.tri_pid0;
  if (tri < 0) {  // an instanced mesh's triangle: the default coordinates
    tu = v;
    tv = u;
    return;
  }
  const float* t = S.tri_uv + 6 * tri;
  tu = __fadd_rn(__fadd_rn(__fmul_rn(w0, t[0]), __fmul_rn(u, t[2])), __fmul_rn(v, t[4]));
  tv = __fadd_rn(__fadd_rn(__fmul_rn(w0, t[1]), __fmul_rn(u, t[3])), __fmul_rn(v, t[5]));
}

// HitRecord::transform's normal (src/hitrecord.h:79-84) for a hit on an
// instance's mesh: the inverse transpose of the instance's linear part, i.e.
// the transpose of its world-to-object rows, then normalised.
__device__ __forceinline__ V3f instance_normal(const DeviceScene& S, int in, V3f n) {
  const float4* M = S.inst + 4 * int64_t(in);
  const float4 m0 = __ldg(M), m1 = __ldg(M + 1), m2 = __ldg(M + 2);
  return normalize(v3(m0.x * n.x + m1.x * n.y + m2.x * n.z, m0.y * n.x + m1.y * n.y + m2.y * n.z,
                      m0.z * n.x + m1.z * n.y + m2.z * n.z));
}

// TextureMaterial::get + brdf's pow (src/texturematerial.cpp:62-74): the
// bilinear sample of the texture at (frac(u) (W - 1), frac(1 - v) (H - 1))
// (cv::getRectSubPix of a 1 x 1 patch, border replicated), times the
// coefficient kd, to the power gamma (the material's exponent).
__device__ __forceinline__ V3f texture_albedo(const DeviceScene& S, const DevMaterial& m, float u, float v) {
  const int4 ti = __ldg(&S.tex_info[m.tex]);
  const int W = ti.y, H = ti.z;
  float fu = fmodf(u, 1.f), fv = fmodf(1.f - v, 1.f);
  if (fu < 0.f) fu += 1.f;
  if (fv < 0.f) fv += 1.f;
  const float x = fu * float(W - 1), y = fv * float(H - 1);
  const float fx = floorf(x), fy = floorf(y);
  const float a = x - fx, b = y - fy;
  const int x0 = min(max(int(fx), 0), W - 1), y0 = min(max(int(fy), 0), H - 1);
  const int x1 = min(x0 + 1, W - 1), y1 = min(y0 + 1, H - 1);
  const float* T = S.tex_texels + 3 * int64_t(ti.x);
  const float w00 = (1.f - a) * (1.f - b), w10 = a * (1.f - b), w01 = (1.f - a) * b, w11 = a * b;
  V3f r;
  float* rr = &r.x;
  for (int c = 0; c < 3; ++c) {
    float s = __ldg(T + (int64_t(y0) * W + x0) * 3 + c) * w00 + __ldg(T + (int64_t(y0) * W + x1) * 3 + c) * w10 +
              __ldg(T + (int64_t(y1) * W + x0) * 3 + c) * w01 + __ldg(T + (int64_t(y1) * W + x1) * 3 + c) * w11;
    s *= m.kd[c];
    rr[c] = m.exponent == 1.f ? s : powf(s, m.exponent);
  }
  return r;
}

__device__ __forceinline__ V3f phong_spec(const DevMaterial& m, const Vertex& h, V3f dir) {
  V3f refl = reflect(dir, h.n);
  float dp = fmaxf(dot(normalize(refl), -normalize(h.d)), 0.f);
  float s = (m.exponent + 2.f) * (0.5f * kInvPi) * powf(dp, m.exponent);
  return v3(s * m.ks[0], s * m.ks[1], s * m.ks[2]);
}

__device__ __forceinline__ float blinn_G(V3f wi, V3f wo, V3f n) {
  V3f wh = normalize(wi + wo);
  return fminf(1.f, 2.f * dot(n, wh) * fminf(dot(n, wo), dot(n, wi)) / dot(wo, wh));
}

// Material::brdf(hit, direction): direction points from the light towards the
// surface (the renderer's convention).
template <bool EXT>
__device__ __forceinline__ V3f brdf_eval(const DeviceScene& S, const Vertex& h, V3f dir) {
  if (h.mat < 0) return v3(0.f, 0.f, 0.f);
  const DevMaterial& m = S.materials[h.mat];
  switch (m.type) {
    case kMatDiffuse:
      return v3(m.kd[0] * kInvPi, m.kd[1] * kInvPi, m.kd[2] * kInvPi);
    case kMatTexture:
      if (EXT) return kInvPi * texture_albedo(S, m, h.tu, h.tv);
      return v3(0.f, 0.f, 0.f);
    case kMatPhong: {
      V3f s = phong_spec(m, h, dir);
      return v3(m.kd[0] * kInvPi + s.x, m.kd[1] * kInvPi + s.y, m.kd[2] * kInvPi + s.z);
    }
    case kMatBlinn: {
      V3f n = h.n;
      V3f wo = -normalize(h.d);
      V3f wi = -normalize(dir);
      if (signum(dot(n, wo)) != signum(dot(n, wi))) return v3(0.f, 0.f, 0.f);
      if (dot(n, wo) < 0.f) n = -n;
      V3f wh = normalize(wi + wo);
      float D = (m.exponent + 2.f) * (0.5f * kInvPi) * powf(dot(wh, n), m.exponent);
      float f = D * blinn_G(wi, wo, n) / (4.f * dot(wo, n) * dot(wi, n));
      return v3(m.kd[0] * kInvPi + m.ks[0] * f, m.kd[1] * kInvPi + m.ks[1] * f, m.kd[2] * kInvPi + m.ks[2] * f);
    }
    default:
      return v3(0.f, 0.f, 0.f);
  }
}

__device__ __forceinline__ bool mat_specular(const DevMaterial* mats, int mat) {
  if (mat < 0) return false;
  int t = mats[mat].type;
  return t == kMatMirror || t == kMatTransparent;
}

// Material::outDirection(hit, sample, pdf, brdf).
template <bool EXT>
__device__ __forceinline__ V3f out_direction(const DeviceScene& S, const Vertex& h, float sx, float sy, float& pdf,
                                             V3f& brdf) {
  brdf = v3(0.f, 0.f, 0.f);
  pdf = 0.f;
  if (h.mat < 0) return v3(0.f, 0.f, 0.f);
  const DevMaterial& m = S.materials[h.mat];
  switch (m.type) {
    case kMatDiffuse:
    case kMatTexture: {  // AbstractDiffuseMaterial::outDirection
      V3f n = h.n;
      if (dot(n, normalize(h.d)) > 0.f) n = -n;
      V3f out = cosine_power_dir(n, sx, sy, 1.f, pdf);
      if (!EXT || m.type == kMatDiffuse) brdf = v3(m.kd[0] * kInvPi, m.kd[1] * kInvPi, m.kd[2] * kInvPi);
      else brdf = kInvPi * texture_albedo(S, m, h.tu, h.tv);
      return out;
    }
    case kMatMirror:
      pdf = 1.f;
      return reflect(h.d, h.n);
    case kMatPhong: {
      V3f n = h.n;
      if (dot(h.d, n) > 0.f) n = -n;
      V3f specDir = reflect(h.d, n);
      if (sx < m.rho_d) {
        V3f out = cosine_power_dir(n, sx / m.rho_d, sy, 1.f, pdf);
        brdf = v3(m.kd[0] * kInvPi, m.kd[1] * kInvPi, m.kd[2] * kInvPi);
        return out;
      } else if (sx < m.rho_d + m.rho_s) {
        V3f out = cosine_power_dir(specDir, (sx - m.rho_d) / m.rho_s, sy, m.exponent, pdf);
        if (dot(out, n) < 1.f) pdf = 0.f;  // the renderer's glossy-lobe quirk
        brdf = phong_spec(m, h, out);
        return out;
      }
      return v3(0.f, 0.f, 0.f);
    }
    case kMatBlinn: {
      V3f n = h.n;
      V3f wo = -normalize(h.d);
      if (dot(n, wo) < 0.f) n = -n;
      V3f wh = cosine_power_dir(n, sx, sy, m.exponent, pdf);
      if (dot(wo, wh) < 0.f) { pdf = 0.f; return v3(0.f, 0.f, 0.f); }
      V3f out = -reflect(wo, wh);
      pdf /= 4.f * fmaxf(dot(wo, wh), 0.0001f);
      brdf = brdf_eval<EXT>(S, h, out);
      return out;
    }
    case kMatTransparent: {
      pdf = 1.f;
      V3f d = normalize(h.d), n = h.n;
      float ratio;
      if (dot(-n, d) < 0.f) { n = -n; ratio = m.ior; } else { ratio = 1.f / m.ior; }
      float cosI = dot(-n, d);
      float s2 = fmaxf(0.f, 1.f - cosI * cosI);
      float sinO = ratio * sqrtf(s2);
      float cosO = sqrtf(fmaxf(0.f, 1.f - ratio * ratio * s2));
      float rPerp = (cosI - ratio * cosO) / (cosI + ratio * cosO);
      float rPara = (ratio * cosI - cosO) / (ratio * cosI + cosO);
      float R = 0.5f * (rPerp * rPerp + rPara * rPara);
      if (sinO > 1.f || sx < R) return reflect(d, n);
      return ratio * d + (ratio * cosI - float(signum(cosI)) * cosO) * n;
    }
    default:
      return v3(0.f, 0.f, 0.f);
  }
}

// ------------------------------------------------------------- Lights -----
// AreaLight::getIntensity(direction): Le * max(0, cos) * |u x v| / |d|^2.
__device__ __forceinline__ V3f area_intensity(const DevLight& L, V3f dir) {
  float c = dot(normalize(dir), ld3(L.nhat)) / len2(dir) * L.normal_len;
  if (!(c >= 0.f)) c = (c < 0.f) ? 0.f : c;
  return v3(c * L.intensity[0], c * L.intensity[1], c * L.intensity[2]);
}

// EnvironmentMap::get(direction). Angular light probe (+x at the centre) or
// equirectangular; nearest texel, indices clamped into the image.
__device__ __forceinline__ V3f env_get(const DeviceScene& S, V3f d) {
  int W = S.env_w, H = S.env_h;
  int row, col;
  if (S.env_mapping == GBRT_ENV_LATLONG) {
    float u = atan2f(d.x, -d.z) * (0.5f * kInvPi) + 0.5f;
    float v = acosf(fminf(1.f, fmaxf(-1.f, d.y))) * kInvPi;
    col = min(int(u * W), W - 1);
    row = min(int(v * H), H - 1);
  } else {
    float cx = d.y, cy = -d.z;
    float f = acosf(d.x) / (sqrtf(cx * cx + cy * cy) * CUDART_PI_F);
    cx *= f; cy *= f;
    int x = int((cx + 1.f) * 0.5f * float(W) - 1.f);
    int y = int((cy + 1.f) * 0.5f * float(H) - 1.f);
    row = min(y, W - 1);
    col = min(x, H - 1);
  }
  row = min(max(row, 0), H - 1);
  col = min(max(col, 0), W - 1);
  const float* p = S.env_texels + (size_t(row) * W + col) * 3;
  return v3(__ldg(p) * S.env_coef[0], __ldg(p + 1) * S.env_coef[1], __ldg(p + 2) * S.env_coef[2]);
}

// ---------------------------------------- environment importance sampling --
// Physical estimator only (the renderer samples the environment by the
// cosine, src/environmentmap.cpp:40-54). The environment is sampled from a
// piecewise-constant density over its mapping's parameter square [0,1)^2,
// env_h rows x env_w cells, each weighted by the luminance its centre looks
// up times the solid angle per unit parameter area there (the tables are
// built at scene creation, scene.cpp build_env_tables). The parameters:
//   lat-long  u = atan2(x, -z) / 2 pi + 1/2, v = acos(y) / pi (env_get's
//             own), solid angle per unit area J = 2 pi^2 sin(theta);
//   angular   u = (cx + 1) / 2, v = (cy + 1) / 2 with (cx, cy) the probe's
//             disc coordinates, r = |(cx, cy)| = theta / pi (theta measured
//             from +x), J = 4 pi^2 sin(theta) / theta; outside the disc there
//             is no direction.
// A direction's density per solid angle is dens(cell) / J.

// Direction of the parameter point (u, v) and J there; false where there is
// none (outside the angular disc, or a pole where J vanishes).
__device__ __forceinline__ bool env_param_dir(const DeviceScene& S, float u, float v, V3f& d, float& jac) {
  if (S.env_mapping == GBRT_ENV_LATLONG) {
    float sp, cp, st, ct;
    sincospif(2.f * u - 1.f, &sp, &cp);
    sincospif(v, &st, &ct);
    d = v3(st * sp, ct, -st * cp);
    jac = (2.f * kPiF * kPiF) * st;
  } else {
    const float cx = 2.f * u - 1.f, cy = 2.f * v - 1.f;
    const float r = sqrtf(cx * cx + cy * cy);
    if (!(r < 1.f)) return false;
    if (r == 0.f) {
      d = v3(1.f, 0.f, 0.f);
      jac = 4.f * kPiF * kPiF;
    } else {
      float st, ct;
      sincospif(r, &st, &ct);
      const float s = st / r;
      d = v3(ct, s * cx, -s * cy);
      jac = (4.f * kPiF) * s;  // 4 pi^2 sin(pi r) / (pi r)
    }
  }
  return jac > 0.f;
}

// Density per solid angle with which env_sample draws the unit direction d.
__device__ __forceinline__ float env_pdf(const DeviceScene& S, V3f d) {
  const int W = S.env_w, H = S.env_h;
  float u, v, jac;
  if (S.env_mapping == GBRT_ENV_LATLONG) {
    u = atan2f(d.x, -d.z) * (0.5f * kInvPi) + 0.5f;
    const float yc = fminf(1.f, fmaxf(-1.f, d.y));
    v = acosf(yc) * kInvPi;
    jac = (2.f * kPiF * kPiF) * sqrtf(fmaxf(0.f, 1.f - yc * yc));
  } else {
    const float th = acosf(fminf(1.f, fmaxf(-1.f, d.x)));
    const float q = sqrtf(d.y * d.y + d.z * d.z);
    const float f = q > 0.f ? th / (q * kPiF) : 0.f;
    u = (d.y * f + 1.f) * 0.5f;
    v = (-d.z * f + 1.f) * 0.5f;
    jac = th > 0.f ? (4.f * kPiF * kPiF) * q / th : 4.f * kPiF * kPiF;
  }
  if (!(jac > 0.f)) return 0.f;
  const int col = min(max(int(u * float(W)), 0), W - 1);
  const int row = min(max(int(v * float(H)), 0), H - 1);
  return __ldg(&S.env_dens[size_t(row) * W + col]) / jac;
}

// Index i in [0, n) with cdf[i] <= x < cdf[i + 1] (cdf[0] = 0, cdf[n] = 1,
// x in [0, 1)); cells of zero width are never returned.
__device__ __forceinline__ int cdf_find(const float* __restrict__ cdf, int n, float x) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&cdf[mid]) <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Draws a direction from the environment's density with u1 (row) and u2
// (cell within the row); its density per solid angle in pdf. False when the
// point has no direction (the angular disc's corners).
__device__ __forceinline__ bool env_sample(const DeviceScene& S, float u1, float u2, V3f& d, float& pdf) {
  const int W = S.env_w, H = S.env_h;
  const int row = cdf_find(S.env_marg, H, u1);
  const float m0 = __ldg(&S.env_marg[row]), m1 = __ldg(&S.env_marg[row + 1]);
  const float* cond = S.env_cond + size_t(row) * (W + 1);
  const int col = cdf_find(cond, W, u2);
  const float c0 = __ldg(&cond[col]), c1 = __ldg(&cond[col + 1]);
  const float fv = fminf((u1 - m0) / (m1 - m0), 0.99999994f);
  const float fu = fminf((u2 - c0) / (c1 - c0), 0.99999994f);
  float jac;
  if (!env_param_dir(S, (float(col) + fu) / float(W), (float(row) + fv) / float(H), d, jac)) return false;
  pdf = __ldg(&S.env_dens[size_t(row) * W + col]) / jac;
  return pdf > 0.f;
}

// ------------------------------------------------ physical semantics -----
// GBRT_SEM_PHYSICAL (not part of the renderer): modified Phong and Blinn with
// their sampling pdfs, perfect mirror and Fresnel-weighted glass. wo / wi
// point away from the surface, n faces wo (lobes are two-sided).
struct PhysBsdf {
  int kind;  // 0 none, 1 diffuse, 2 phong, 3 blinn, 4 mirror, 5 glass
  V3f kd, ks;
  float e, ior, pd;
};

template <bool EXT>
__device__ __forceinline__ PhysBsdf phys_bsdf(const DeviceScene& S, int mat, float tu, float tv) {
  PhysBsdf b;
  b.kind = 0; b.e = 0.f; b.ior = 1.f; b.pd = 1.f;
  b.kd = v3(0.f, 0.f, 0.f); b.ks = v3(0.f, 0.f, 0.f);
  if (mat < 0) return b;
  const DevMaterial& m = S.materials[mat];
  b.kd = ld3(m.kd); b.ks = ld3(m.ks); b.e = m.exponent; b.ior = m.ior;
  switch (m.type) {
    case kMatDiffuse: b.kind = 1; break;
    case kMatTexture:
      b.kind = 1;
      if (EXT) b.kd = texture_albedo(S, m, tu, tv);
      break;
    case kMatPhong: b.kind = 2; break;
    case kMatBlinn: b.kind = 3; break;
    case kMatMirror: b.kind = 4; break;
    case kMatTransparent: b.kind = 5; break;
    default: b.kind = 0;
  }
  if (b.kind == 2 || b.kind == 3) {
    float s = m.rho_d + m.rho_s;
    b.pd = s > 0.f ? m.rho_d / s : 1.f;
  }
  return b;
}

__device__ __forceinline__ float cos_power_pdf(float c, float e) {
  return c > 0.f ? (e + 1.f) * (0.5f * kInvPi) * powf(c, e) : 0.f;
}

// f(wo, wi) and the pdf of sampling wi, for the non-specular kinds.
__device__ __forceinline__ V3f phys_eval(const PhysBsdf& b, V3f n, V3f wo, V3f wi, float& pdf) {
  pdf = 0.f;
  float ci = dot(n, wi), co = dot(n, wo);
  if (b.kind < 1 || b.kind > 3 || ci <= 0.f || co <= 0.f) return v3(0.f, 0.f, 0.f);
  V3f diff = kInvPi * b.kd;
  if (b.kind == 1) {
    pdf = ci * kInvPi;
    return diff;
  }
  if (b.kind == 2) {
    V3f r = (2.f * co) * n - wo;
    float ca = fmaxf(0.f, dot(r, wi));
    float sp = (b.e + 2.f) * (0.5f * kInvPi) * powf(ca, b.e);
    pdf = b.pd * ci * kInvPi + (1.f - b.pd) * cos_power_pdf(ca, b.e);
    return diff + sp * b.ks;
  }
  V3f h = normalize(wi + wo);
  float nh = dot(n, h), oh = dot(wo, h);
  float D = (b.e + 2.f) * (0.5f * kInvPi) * powf(fmaxf(nh, 0.f), b.e);
  float G = fminf(1.f, fminf(2.f * nh * co / oh, 2.f * nh * ci / oh));
  pdf = b.pd * ci * kInvPi + (1.f - b.pd) * (oh > 0.f ? cos_power_pdf(nh, b.e) / (4.f * oh) : 0.f);
  return diff + (D * G / (4.f * ci * co)) * b.ks;
}

// Samples wi; weight = f * |cos| / pdf (1 for the specular kinds).
__device__ __forceinline__ bool phys_sample(const PhysBsdf& b, V3f n, V3f wo, bool exiting, float u0, float u1,
                                            float u2, V3f& wi, V3f& weight, float& pdf, bool& specular) {
  specular = false;
  pdf = 0.f;
  if (b.kind == 4) {
    wi = (2.f * dot(n, wo)) * n - wo;
    specular = true; weight = v3(1.f, 1.f, 1.f); pdf = 1.f;
    return true;
  }
  if (b.kind == 5) {
    // Leaving the medium the geometric normal points along the ray
    // (TransparentMaterial's test, src/transparentmaterial.cpp:43-51).
    V3f d = -wo;
    float ratio = exiting ? b.ior : 1.f / b.ior;
    float cosI = dot(-n, d);
    float s2 = fmaxf(0.f, 1.f - cosI * cosI);
    float sinO = ratio * sqrtf(s2);
    float cosO = sqrtf(fmaxf(0.f, 1.f - ratio * ratio * s2));
    float rPerp = (cosI - ratio * cosO) / (cosI + ratio * cosO);
    float rPara = (ratio * cosI - cosO) / (ratio * cosI + cosO);
    float R = 0.5f * (rPerp * rPerp + rPara * rPara);
    if (sinO > 1.f || u0 < R) wi = reflect(d, n);
    else wi = ratio * d + (ratio * cosI - float(signum(cosI)) * cosO) * n;
    specular = true; weight = v3(1.f, 1.f, 1.f); pdf = 1.f;
    return true;
  }
  if (b.kind < 1) return false;
  float tmp;
  if (b.kind == 1 || u0 < b.pd) {
    wi = cosine_power_dir(n, u1, u2, 1.f, tmp);
  } else if (b.kind == 2) {
    wi = cosine_power_dir((2.f * dot(n, wo)) * n - wo, u1, u2, b.e, tmp);
  } else {
    V3f h = cosine_power_dir(n, u1, u2, b.e, tmp);
    wi = (2.f * dot(wo, h)) * h - wo;
  }
  V3f f = phys_eval(b, n, wo, wi, pdf);
  if (!(pdf > 0.f)) return false;
  weight = (dot(n, wi) / pdf) * f;
  return true;
}

__device__ __forceinline__ float power_heuristic(float a, float b) { return a * a / (a * a + b * b); }

// Uniform direction on the sphere (Sample::getUniformSphereDirection,
// src/sampler.cpp:78-86).
__device__ __forceinline__ V3f uniform_sphere(float ux, float uy) {
  float z = 2.f * ux - 1.f;
  float f = sqrtf(fmaxf(0.f, 1.f - z * z));
  float sn, cs;
  sincospif(2.f * uy, &sn, &cs);
  return v3(f * cs, f * sn, z);
}

// Dimension layout of the physical estimator: per vertex i, base 2 + 8i:
// +0 lobe, +1/+2 BSDF direction, +3 light index, +4/+5 light sample, +6
// roulette (dims 0/1: pixel jitter).
__device__ __forceinline__ unsigned dim_phys(int i) { return 2u + 8u * unsigned(i); }

}  // namespace gbrt
