/*
 * oracle.cpp — TEST INFRASTRUCTURE ONLY: the CPU oracle for the GB300 path
 * tracer. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it; the product never links or calls it.
 *
 * It restates, class for class, the renderer's unidirectional path-tracing hot
 * path in plain C++17 (no Qt, GSL, OpenCV or Boost), quirks included, so that
 * it can check the CUDA path and serve as the timed CPU baseline:
 *   PerPixelRenderer::render        src/perpixelrenderer.cpp:43-101
 *   Renderer::createPath            src/renderer.cpp:47-106
 *   UniDiPathTracingIntegrator      src/unidipathtracingintegrator.cpp:34-107
 *   BVHNode::create / intersect     src/bvh.cpp:34-149
 *   AxisAlignedBox slab test        src/axisalignedbox.cpp:30-104
 *   IntersectableList               src/intersectablelist.cpp:30-78
 *   Triangle / Quad                 src/triangle.cpp:30-65, src/quad.cpp:23-41
 *   Sphere + CSGObject::intersect   src/sphere.cpp:29-62, src/csgobject.cpp:25-44
 *   Plane                           src/plane.cpp:27-46
 *   AreaLight / PointLight          src/arealight.cpp:31-118, src/pointlight.cpp:29-70
 *   ConeLight                       src/conelight.cpp:31-60
 *   EnvironmentMap / BlackLight     src/environmentmap.cpp:16-108, src/blacklight.cpp:5-24
 *   Materials                       src/darkmatter.cpp, src/abstractdiffusematerial.cpp,
 *                                   src/diffusematerial.cpp, src/mirrormaterial.cpp,
 *                                   src/phongmaterial.cpp, src/blinnmaterial.cpp,
 *                                   src/transparentmaterial.cpp
 *   Sample / JitteredSampler        src/sampler.cpp:33-86, src/jitteredsampler.cpp:23-35
 *   Camera                          src/camera.cpp:34-58
 *
 * Parity is unpinned by the renderer itself: it ships no tests, golden images
 * or scene files, and it cannot be built here (Qt5, GSL, OpenCV and Boost are
 * absent). Third-party arithmetic it relies on is restated: Qt's vector and
 * matrix operations (oracle_math.h); GSL's taus2 generator as L'Ecuyer's
 * published combined Tausworthe generator (taus88), GSL's negative binomial
 * with n = 1 as the geometric distribution drawn by inversion, and
 * gsl_rng_uniform_int as floor(u * n). These replace GSL's exact streams; the
 * reference's own argument-evaluation order in JitteredSampler is unspecified
 * anyway, so stream-level parity with the renderer is impossible and parity is
 * statistical. A second, counter-based generator (rng_mode 1) lets the oracle
 * draw exactly the numbers the CUDA path draws, for path-level comparisons.
 *
 * Deviations (all measure-zero or undefined behaviour in the renderer):
 *   - the end-of-path dereference of list end() (src/unidipathtracingintegrator.cpp:66-68)
 *     is read as "no next vertex";
 *   - environment-map texel indices are clamped into the image (the renderer
 *     can index row/column -1 at the rim and swaps width and height in its clamp,
 *     src/environmentmap.cpp:61-64);
 *   - BVH centroid sorting uses a NaN-safe key (infinite boxes of planes and the
 *     environment map give NaN centres, which makes std::sort's comparator
 *     invalid, src/bvh.cpp:52-57); the closest hit does not depend on the tree.
 */
#include "oracle_math.h"
#include "../include/gbrt.h"

#include <algorithm>
#include <cstring>
#include <list>
#include <functional>
#include <memory>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

M4 inverted(const M4& a) {
  double m[16], inv[16];
  for (int c = 0; c < 4; ++c)
    for (int r = 0; r < 4; ++r) m[c * 4 + r] = a.m[c][r];
  inv[0] = m[5] * m[10] * m[15] - m[5] * m[11] * m[14] - m[9] * m[6] * m[15] + m[9] * m[7] * m[14] + m[13] * m[6] * m[11] - m[13] * m[7] * m[10];
  inv[4] = -m[4] * m[10] * m[15] + m[4] * m[11] * m[14] + m[8] * m[6] * m[15] - m[8] * m[7] * m[14] - m[12] * m[6] * m[11] + m[12] * m[7] * m[10];
  inv[8] = m[4] * m[9] * m[15] - m[4] * m[11] * m[13] - m[8] * m[5] * m[15] + m[8] * m[7] * m[13] + m[12] * m[5] * m[11] - m[12] * m[7] * m[9];
  inv[12] = -m[4] * m[9] * m[14] + m[4] * m[10] * m[13] + m[8] * m[5] * m[14] - m[8] * m[6] * m[13] - m[12] * m[5] * m[10] + m[12] * m[6] * m[9];
  inv[1] = -m[1] * m[10] * m[15] + m[1] * m[11] * m[14] + m[9] * m[2] * m[15] - m[9] * m[3] * m[14] - m[13] * m[2] * m[11] + m[13] * m[3] * m[10];
  inv[5] = m[0] * m[10] * m[15] - m[0] * m[11] * m[14] - m[8] * m[2] * m[15] + m[8] * m[3] * m[14] + m[12] * m[2] * m[11] - m[12] * m[3] * m[10];
  inv[9] = -m[0] * m[9] * m[15] + m[0] * m[11] * m[13] + m[8] * m[1] * m[15] - m[8] * m[3] * m[13] - m[12] * m[1] * m[11] + m[12] * m[3] * m[9];
  inv[13] = m[0] * m[9] * m[14] - m[0] * m[10] * m[13] - m[8] * m[1] * m[14] + m[8] * m[2] * m[13] + m[12] * m[1] * m[10] - m[12] * m[2] * m[9];
  inv[2] = m[1] * m[6] * m[15] - m[1] * m[7] * m[14] - m[5] * m[2] * m[15] + m[5] * m[3] * m[14] + m[13] * m[2] * m[7] - m[13] * m[3] * m[6];
  inv[6] = -m[0] * m[6] * m[15] + m[0] * m[7] * m[14] + m[4] * m[2] * m[15] - m[4] * m[3] * m[14] - m[12] * m[2] * m[7] + m[12] * m[3] * m[6];
  inv[10] = m[0] * m[5] * m[15] - m[0] * m[7] * m[13] - m[4] * m[1] * m[15] + m[4] * m[3] * m[13] + m[12] * m[1] * m[7] - m[12] * m[3] * m[5];
  inv[14] = -m[0] * m[5] * m[14] + m[0] * m[6] * m[13] + m[4] * m[1] * m[14] - m[4] * m[2] * m[13] - m[12] * m[1] * m[6] + m[12] * m[2] * m[5];
  inv[3] = -m[1] * m[6] * m[11] + m[1] * m[7] * m[10] + m[5] * m[2] * m[11] - m[5] * m[3] * m[10] - m[9] * m[2] * m[7] + m[9] * m[3] * m[6];
  inv[7] = m[0] * m[6] * m[11] - m[0] * m[7] * m[10] - m[4] * m[2] * m[11] + m[4] * m[3] * m[10] + m[8] * m[2] * m[7] - m[8] * m[3] * m[6];
  inv[11] = -m[0] * m[5] * m[11] + m[0] * m[7] * m[9] + m[4] * m[1] * m[11] - m[4] * m[3] * m[9] - m[8] * m[1] * m[7] + m[8] * m[3] * m[5];
  inv[15] = m[0] * m[5] * m[10] - m[0] * m[6] * m[9] - m[4] * m[1] * m[10] + m[4] * m[2] * m[9] + m[8] * m[1] * m[6] - m[8] * m[2] * m[5];
  double det = m[0] * inv[0] + m[1] * inv[4] + m[2] * inv[8] + m[3] * inv[12];
  M4 out;
  if (det == 0) return out;
  for (int i = 0; i < 16; ++i) out.m[i / 4][i % 4] = float(inv[i] / det);
  return out;
}

M4 normalMatrix(const M4& a) {
  M4 inv = inverted(a);
  M4 out;
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) out.m[c][r] = inv.m[r][c];
  return out;
}

/* ------------------------------------------------------------------ RNG -- */

/* SplitMix64 output function (Steele, Lea, Flood 2014): the mixer of the
 * counter-based stream shared by the oracle and the CUDA path. */
static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Rng {
  virtual ~Rng() {}
  virtual double uniform() = 0;                   /* [0,1) */
};

/* L'Ecuyer's maximally equidistributed combined Tausworthe generator (1996),
 * the algorithm behind GSL's taus2. Seeding through an LCG keeps every
 * component above its minimum. */
struct TausRng : Rng {
  uint32_t s1, s2, s3;
  explicit TausRng(uint64_t seed) {
    uint32_t x = uint32_t(seed ^ (seed >> 32)) ;
    if (x == 0) x = 1;
    auto lcg = [&]() { x = 69069u * x + 1u; return x; };
    s1 = lcg(); if (s1 < 2) s1 += 2;
    s2 = lcg(); if (s2 < 8) s2 += 8;
    s3 = lcg(); if (s3 < 16) s3 += 16;
    for (int i = 0; i < 6; ++i) next();
  }
  uint32_t next() {
    uint32_t b;
    b = ((s1 << 13) ^ s1) >> 19; s1 = ((s1 & 4294967294u) << 12) ^ b;
    b = ((s2 << 2) ^ s2) >> 25;  s2 = ((s2 & 4294967288u) << 4) ^ b;
    b = ((s3 << 3) ^ s3) >> 11;  s3 = ((s3 & 4294967280u) << 17) ^ b;
    return s1 ^ s2 ^ s3;
  }
  double uniform() override { return next() / 4294967296.0; }
};

/* Counter-based stream: u(key, dim) = top 24 bits of mix64(key + dim * phi).
 * key = mix64(seed ^ mix64(sample_id + c)), sample_id = pixel * spp + s. */
static inline uint64_t streamKey(uint64_t seed, uint64_t sample_id) {
  return mix64(seed ^ mix64(sample_id + 0x632BE59BD9B4E019ull));
}
static inline float streamU(uint64_t key, uint32_t dim) {
  uint64_t h = mix64(key + uint64_t(dim) * 0x9E3779B97F4A7C15ull);
  return float(h >> 40) * (1.0f / 16777216.0f);
}

/* --------------------------------------------------------------- Sample -- */

struct Sample {
  double x = 0, y = 0; /* QPointF */
  Sample() = default;
  Sample(double a, double b) : x(a), y(b) {}

  /* Sample::getCosinePowerWeightedDirection, src/sampler.cpp:48-76. */
  V3 cosinePowerDirection(V3 w, float& pdf, float e, float openingAngle = float(M_PI / 2)) const {
    float radiusFactor = float(std::sin(double(openingAngle)));
    w.normalize();
    /* 2 / (e + 1) and 1 / (e + 1) are float expressions in the renderer. */
    double pw = std::pow(x, double(2 / (e + 1)));
    V3 nd(float(std::cos(2 * M_PI * y) * std::sqrt(1 - pw * radiusFactor * radiusFactor)),
          float(std::sin(2 * M_PI * y) * std::sqrt(1 - pw * radiusFactor * radiusFactor)),
          float(std::pow(x, double(1 / (e + 1))) * radiusFactor));
    pdf = float(std::pow(double(nd.z), double(e)) * (double(e) + 1) / (2 * M_PI));
    V3 v;
    if (std::fabs(w.x) < std::fabs(w.y) && std::fabs(w.x) < std::fabs(w.z)) v = V3(0, w.z, -w.y);
    else if (std::fabs(w.y) < std::fabs(w.z)) v = V3(w.z, 0, -w.x);
    else v = V3(w.y, -w.x, 0);
    v.normalize();
    V3 u = cross(v, w);
    M4 t;
    t.setColumn(0, V4(u, 0)); t.setColumn(1, V4(v, 0)); t.setColumn(2, V4(w, 0));
    V3 d = t.mapPoint(nd);
    return d.normalized();
  }
  V3 cosineDirection(V3 w, float& pdf) const { return cosinePowerDirection(w, pdf, 1.f); }
  /* getUniformSphereDirection, src/sampler.cpp:78-86. */
  V3 uniformSphere() const {
    float z = float(2 * x - 1);
    float t = float(2 * M_PI * y);
    float f = std::sqrt(1 - z * z);
    return V3(f * std::cos(t), f * std::sin(t), z);
  }
};

/* ------------------------------------------------------------------ Ray -- */

struct Ray {
  V3 o, d;
  float from = kEpsilon, to = kInf;
  Ray() = default;
  Ray(V3 origin, V3 dir, float f = kEpsilon, float t = kInf) : o(origin), d(dir), from(f), to(t) {}
  /* Ray::evaluate, src/ray.h:91-101. */
  V4 evaluate(float u) const {
    if (std::isinf(u)) {
      V3 n = d.normalized();
      float s = float(signum(u));
      return V4(s * n.x, s * n.y, s * n.z, s * 0.f);
    }
    return V4(o + u * d, 1);
  }
  bool inRange(float u) const { return from <= u && u <= to; }
  Ray transform(const M4& m) const {
    V4 no = m.map4(V4(o, 1)), nd = m.map4(V4(d, 0));
    return Ray(no.affine(), nd.xyz(), from, to);
  }
};

struct Material;
struct Intersectable;

/* HitRecord, src/hitrecord.h:35-121 (+ the leaf's primitive id and the
 * triangle barycentrics for the ray-level oracle). */
struct Hit {
  const Material* mat = nullptr;
  float t = kNaN;
  V4 point;
  V3 normal;
  Ray ray;
  int prim = -1;
  float bu = 0, bv = 0;
  float tu = 0, tv = 0;  /* texcoords, src/hitrecord.h:59 (default (0, 0)) */
  Hit() = default;
  Hit(float tt, const Ray& r, const Material* m, V3 n, int p, float u = 0, float v = 0)
      : mat(m), t(tt), point(r.evaluate(tt)), normal(n.normalized()), ray(r), prim(p), bu(u), bv(v) {}
  bool intersects() const { return !std::isnan(t); }
  void transform(const M4& m, const M4& nm) {
    point = m.map4(point);
    ray = ray.transform(m);
    normal = nm.mapPoint(normal);
  }
};

/* ------------------------------------------------------------- Material -- */

struct Material {
  virtual ~Material() {}
  virtual C3 brdf(const Hit&, V3) const { return C3(); }
  virtual bool isSpecular() const { return false; }
  virtual C3 emission(const Hit&) const { return C3(); }
  virtual bool emitsLight() const { return false; }
  virtual V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& brdf) const = 0;
};

struct DiffuseMaterial;

/* DarkMatter, src/darkmatter.cpp:32-39. */
struct DarkMatter : Material {
  V3 outDirection(const Hit&, Sample, float& pdf, C3& brdf) const override {
    brdf = C3(); pdf = 0; return V3();
  }
};
static DarkMatter gDark;

/* AbstractDiffuseMaterial + DiffuseMaterial, src/abstractdiffusematerial.cpp:8-14,
 * src/diffusematerial.cpp:25-28. */
struct DiffuseMaterial : Material {
  C3 color;
  explicit DiffuseMaterial(C3 c) : color(c) {}
  C3 brdf(const Hit&, V3) const override { return color * float(1 / M_PI); }
  V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& b) const override {
    V3 n = hit.normal;
    if (dot(n.normalized(), hit.ray.d.normalized()) > 0) n = n * -1.f;
    V3 out = s.cosineDirection(n, pdf);
    b = brdf(hit, out);
    return out;
  }
};

/* TextureMaterial, src/texturematerial.cpp:33-74: AbstractDiffuseMaterial
 * whose brdf is pow(get(texcoords), gamma) / pi, get = the bilinear sample
 * of a 1 x 1 cv::getRectSubPix patch at (frac(u) (W - 1), frac(1 - v) (H - 1))
 * (border replicated) times the coefficient. The texels are those of
 * cv::imread scaled by 1/255 (load, :48-60), given here already scaled. */
struct TextureMaterial : Material {
  int W, H;
  std::vector<float> tex;
  C3 coef;
  float gamma;
  TextureMaterial(int w, int h, const float* texels, C3 c, float g)
      : W(w), H(h), tex(texels, texels + size_t(w) * h * 3), coef(c), gamma(g) {}
  static float wrap(float x) {
    float f = std::fmod(x, 1.f);
    if (f < 0) f += 1;
    return f;
  }
  C3 get(float u, float v) const {
    float x = wrap(u) * float(W - 1), y = wrap(1 - v) * float(H - 1);
    float fx = std::floor(x), fy = std::floor(y);
    float a = x - fx, b = y - fy;
    int x0 = std::min(std::max(int(fx), 0), W - 1), y0 = std::min(std::max(int(fy), 0), H - 1);
    int x1 = std::min(x0 + 1, W - 1), y1 = std::min(y0 + 1, H - 1);
    float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
    float r[3];
    for (int c = 0; c < 3; ++c)
      r[c] = tex[(size_t(y0) * W + x0) * 3 + c] * w00 + tex[(size_t(y0) * W + x1) * 3 + c] * w10 +
             tex[(size_t(y1) * W + x0) * 3 + c] * w01 + tex[(size_t(y1) * W + x1) * 3 + c] * w11;
    return C3(r[0] * coef.b, r[1] * coef.g, r[2] * coef.r);
  }
  C3 albedo(const Hit& h) const {
    C3 g = get(h.tu, h.tv);
    if (gamma == 1.f) return g;
    return C3(std::pow(g.b, gamma), std::pow(g.g, gamma), std::pow(g.r, gamma));
  }
  C3 brdf(const Hit& h, V3) const override { return albedo(h) * float(1 / M_PI); }
  V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& b) const override {
    V3 n = hit.normal;
    if (dot(n.normalized(), hit.ray.d.normalized()) > 0) n = n * -1.f;
    V3 out = s.cosineDirection(n, pdf);
    b = brdf(hit, out);
    return out;
  }
};

/* MirrorMaterial, src/mirrormaterial.cpp:31-41. */
struct MirrorMaterial : Material {
  bool isSpecular() const override { return true; }
  V3 outDirection(const Hit& hit, Sample, float& pdf, C3& b) const override {
    pdf = 1; b = C3();
    return reflect(hit.ray.d, hit.normal.normalized());
  }
};

/* PhongMaterial, src/phongmaterial.cpp:31-81. */
struct PhongMaterial : Material {
  C3 color, spec; float e;
  PhongMaterial(C3 kd, C3 ks, float ex) : color(kd), spec(ks), e(ex) {}
  C3 diffuseBrdf() const { return color * float(1 / M_PI); }
  C3 specularBrdf(const Hit& hit, V3 direction) const {
    V3 normal = hit.normal.normalized();
    V3 reflected = reflect(direction, normal);
    float dp = std::max(dot(reflected.normalized(), -hit.ray.d.normalized()), 0.f);
    float sp = float((e + 2) / (2 * M_PI) * std::pow(dp, e));
    return sp * spec;
  }
  C3 brdf(const Hit& hit, V3 d) const override { return diffuseBrdf() + specularBrdf(hit, d); }
  V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& b) const override {
    V3 n = hit.normal;
    if (dot(hit.ray.d, n) > 0) n = n * -1.f;
    n.normalize();
    V3 specDir = reflect(hit.ray.d, n);
    float rho_d = lum(color), rho_s = lum(spec);
    if (s.x < rho_d) {
      s.x /= rho_d;
      V3 out = s.cosineDirection(n, pdf);
      b = diffuseBrdf();
      return out;
    } else if (s.x < rho_d + rho_s) {
      s.x = (s.x - rho_d) / rho_s;
      V3 out = s.cosinePowerDirection(specDir, pdf, e);
      if (dot(out, n) < 1) pdf = 0; /* the renderer's glossy-lobe quirk */
      b = specularBrdf(hit, out);
      return out;
    }
    pdf = 0; b = C3();
    return V3();
  }
};

/* BlinnMaterial, src/blinnmaterial.cpp:30-84. */
static float blinnG(V3 wi, V3 wo, V3 n) {
  V3 wh = wi + wo; wh.normalize();
  return std::min(1.f, 2 * dot(n, wh) * std::min(dot(n, wo), dot(n, wi)) / dot(wo, wh));
}
struct BlinnMaterial : Material {
  C3 kd, ks; float e;
  BlinnMaterial(C3 a, C3 b, float ex) : kd(a), ks(b), e(ex) {}
  float D(V3 wh, V3 n) const { return float((e + 2) / (2 * M_PI) * std::pow(dot(wh, n), e)); }
  C3 brdf(const Hit& hit, V3 direction) const override {
    V3 n = hit.normal; n.normalize();
    V3 wo = -hit.ray.d.normalized();
    V3 wi = -direction.normalized();
    if (signum(dot(n, wo)) != signum(dot(n, wi))) return C3();
    if (dot(n, wo) < 0) n = n * -1.f;
    V3 wh = wi + wo; wh.normalize();
    return kd * float(1 / M_PI) + ks * (D(wh, n) * blinnG(wi, wo, n) / (4 * dot(wo, n) * dot(wi, n)));
  }
  V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& b) const override {
    V3 n = hit.normal; n.normalize();
    V3 wo = -hit.ray.d.normalized();
    if (dot(n, wo) < 0) n = n * -1.f;
    V3 wh = s.cosinePowerDirection(n, pdf, e);
    if (dot(wo, wh) < 0) { pdf = 0; b = C3(); return V3(); }
    V3 out = -reflect(wo, wh);
    pdf /= 4 * std::max(dot(wo, wh), .0001f);
    b = brdf(hit, out);
    return out;
  }
};

/* TransparentMaterial, src/transparentmaterial.cpp:34-80. */
struct TransparentMaterial : Material {
  float k;
  explicit TransparentMaterial(float c) : k(c) {}
  bool isSpecular() const override { return true; }
  V3 outDirection(const Hit& hit, Sample s, float& pdf, C3& b) const override {
    pdf = 1; b = C3();
    V3 d = hit.ray.d, n = hit.normal;
    d.normalize(); n.normalize();
    float ratio;
    if (dot(-n, d) < 0.) { n = n * -1.f; ratio = k; } else { ratio = 1 / k; }
    float cosI = dot(-n, d);
    float cc = cosI * cosI;
    float sinO = float(ratio * std::sqrt(std::max(0., 1. - cc)));
    float cosO = float(std::sqrt(std::max(0., 1 - (ratio * ratio) * std::max(0., 1. - cc))));
    float rPerp = (cosI - ratio * cosO) / (cosI + ratio * cosO);
    float rPara = (ratio * cosI - cosO) / (ratio * cosI + cosO);
    float R = float(1 / 2. * (rPerp * rPerp + rPara * rPara));
    if (sinO > 1 || s.x < R) return reflect(d, n);
    return ratio * d + (ratio * cosI - signum(cosI) * cosO) * n;
  }
};

/* -------------------------------------------------------- Intersectable -- */

struct AABB {
  V3 mn{kInf, kInf, kInf}, mx{-kInf, -kInf, -kInf};
  AABB() = default;
  AABB(V3 a, V3 b) : mn(a), mx(b) {}
  void includePoint(V3 p) {
    for (int i = 0; i < 3; ++i) {
      if (p[i] < mn[i]) mn[i] = p[i];
      if (p[i] > mx[i]) mx[i] = p[i];
    }
  }
  void includeOther(const AABB& b) { includePoint(b.mn); includePoint(b.mx); }
  struct Param { float t; V3 normal; };
  /* AxisAlignedBox::getCSGIntersection, src/axisalignedbox.cpp:30-73: a
   * heap-allocated entry/exit list per call, kept for a faithful CPU cost. */
  std::list<Param> csgIntersection(const Ray& ray) const {
    std::list<Param> result;
    Param p;
    float tmin = -kInf, tmax = kInf;
    for (int i = 0; i < 3; ++i) {
      float a = 1 / ray.d[i];
      float t0, t1;
      V3 nrm;
      if (a >= 0) { t0 = mn[i] - ray.o[i]; t1 = mx[i] - ray.o[i]; nrm[i] = -1; }
      else { t0 = mx[i] - ray.o[i]; t1 = mn[i] - ray.o[i]; nrm[i] = 1; }
      t0 *= a; t1 *= a;
      if (t0 > tmin) { tmin = t0; p.normal = nrm; }
      if (t1 < tmax) tmax = t1;
      if (tmin > tmax) return result;
    }
    p.t = tmin; result.push_back(p);
    p.t = tmax; result.push_back(p);
    return result;
  }
};

/* The prim id a leaf must skip (any-hit queries only). */
static thread_local int tIgnorePrim = -1;

struct Intersectable {
  int prim = -1;
  virtual ~Intersectable() {}
  virtual Hit intersect(const Ray& ray) const = 0;
  virtual AABB bbox() const = 0;
  virtual void contained(std::vector<Intersectable*>& out) { out.push_back(this); }
};

/* Triangle, src/triangle.h:35-38, src/triangle.cpp:30-65. Texture
 * coordinates default to (0,0), (0,1), (1,0) as in the constructors without
 * them. */
struct Triangle : Intersectable {
  V3 p1, p2, p3, n1, n2, n3;
  float t1[2] = {0, 0}, t2[2] = {0, 1}, t3[2] = {1, 0};
  const Material* mat;
  Triangle(V3 a, V3 b, V3 c, const Material* m) : p1(a), p2(b), p3(c), mat(m) {
    n1 = cross(a - b, a - c).normalized(); n2 = n1; n3 = n1;
  }
  Triangle(V3 a, V3 b, V3 c, V3 na, V3 nb, V3 nc, const Material* m)
      : p1(a), p2(b), p3(c), n1(na.normalized()), n2(nb.normalized()), n3(nc.normalized()), mat(m) {}
  Hit intersect(const Ray& ray) const override {
    if (prim == tIgnorePrim) return Hit();
    V3 ad = ray.o - p1;
    V3 abxac = cross(p2 - p1, p3 - p1);
    float w = -dot(abxac, ray.d);
    if (w == 0) return Hit();
    float t = dot(abxac, ad) / w;
    if (!ray.inRange(t)) return Hit();
    V3 adxde = cross(ad, ray.d);
    float u = dot(adxde, p3 - p1) / w;
    if (u < 0 || u > 1) return Hit();
    float v = -dot(adxde, p2 - p1) / w;
    if (v < 0 || u + v > 1) return Hit();
    V3 normal = (1 - u - v) * n1 + u * n2 + v * n3;
    if (normal == V3()) return Hit();
    Hit h(t, ray, mat, normal, prim, u, v);
    /* (1 - u - v) * t1 + u * t2 + v * t3 (cv::Point2f arithmetic) */
    float w0 = 1 - u - v;
    h.tu = w0 * t1[0] + u * t2[0] + v * t3[0];
    h.tv = w0 * t1[1] + u * t2[1] + v * t3[1];
    return h;
  }
  AABB bbox() const override { AABB b; b.includePoint(p1); b.includePoint(p2); b.includePoint(p3); return b; }
};

/* Quad(p1..p4) = Triangle(p1,p2,p4) then Triangle(p4,p2,p3), src/quad.h:32,
 * src/quad.cpp:23-41: the first triangle's hit wins without a t comparison. */
struct Quad : Intersectable {
  Triangle t1, t2;
  Quad(V3 a, V3 b, V3 c, V3 d, const Material* m) : t1(a, b, d, m), t2(d, b, c, m) {}
  void setPrim(int p) { prim = p; t1.prim = p; t2.prim = p; }
  Hit intersect(const Ray& ray) const override {
    Hit h = t1.intersect(ray);
    if (h.intersects()) return h;
    return t2.intersect(ray);
  }
  AABB bbox() const override { AABB b = t1.bbox(); b.includeOther(t2.bbox()); return b; }
};

/* Sphere as a CSG leaf, src/sphere.cpp:29-62 + CSGObject::intersect,
 * src/csgobject.cpp:25-44 (two-entry list per test, kept). */
struct Sphere : Intersectable {
  V3 c; float r; const Material* mat;
  Sphere(V3 cc, float rr, const Material* m) : c(cc), r(rr), mat(m) {}
  Hit intersect(const Ray& ray) const override {
    if (prim == tIgnorePrim) return Hit();
    struct P { float t; V3 n; float tu, tv; };
    std::list<P> params;
    V3 diff = ray.o - c;
    float r2 = r * r;
    float a = ray.d.lengthSquared();
    float b = 2 * dot(ray.d, diff);
    float cc = diff.lengthSquared() - r2;
    float disc = b * b - 4 * a * cc;
    if (disc >= 0) {
      float rd = std::sqrt(disc);
      P p;
      /* texcoord (acos(n.z / r) / pi, atan2(n.x, n.y) / pi / 2 + 0.5), src/sphere.cpp:44-50 */
      auto uvOf = [&](P& q) {
        q.tu = float(std::acos(double(q.n.z / r)) / M_PI);
        q.tv = float(std::atan2(double(q.n.x), double(q.n.y)) / M_PI / 2 + 0.5);
      };
      p.t = (-b - rd) / (2 * a); p.n = ray.evaluate(p.t).affine() - c; uvOf(p); params.push_back(p);
      p.t = (-b + rd) / (2 * a); p.n = ray.evaluate(p.t).affine() - c; uvOf(p); params.push_back(p);
    }
    if (params.empty() || ray.from > params.back().t) return Hit();
    for (auto& p : params) {
      if (p.t >= ray.from) {
        if (p.t > ray.to) return Hit();
        Hit h(p.t, ray, mat, p.n, prim);
        h.tu = p.tu;
        h.tv = p.tv;
        return h;
      }
    }
    return Hit();
  }
  AABB bbox() const override { V3 rv(r, r, r); return AABB(c - rv, c + rv); }
};

/* ------------------------------------------------------------------ CSG --
 * IntersectionParameter (src/csgobject.h:32-43), the leaves' interval lists
 * (Sphere::getCSGIntersection, src/sphere.cpp:29-56; AxisAlignedBox::
 * getCSGIntersection, src/axisalignedbox.cpp:30-73), CSGOperation (src/
 * csgoperation.cpp:27-97) and CSGObject::intersect (src/csgobject.cpp:25-44),
 * with std::list as in the renderer. */
struct CsgParam {
  float t = 0;
  V3 normal;
  float tu = 0, tv = 0;
  const Material* mat = nullptr;
};

struct CsgNode {
  virtual ~CsgNode() {}
  virtual std::list<CsgParam> params(const Ray& ray) const = 0;
  virtual AABB box() const = 0;
};

struct CsgSphere : CsgNode {
  V3 c; float r; const Material* mat;
  CsgSphere(V3 cc, float rr, const Material* m) : c(cc), r(rr), mat(m) {}
  std::list<CsgParam> params(const Ray& ray) const override {
    std::list<CsgParam> out;
    V3 diff = ray.o - c;
    float a = ray.d.lengthSquared();
    float b = 2 * dot(ray.d, diff);
    float cc = diff.lengthSquared() - r * r;
    float disc = b * b - 4 * a * cc;
    if (disc >= 0) {
      float rd = std::sqrt(disc);
      CsgParam p;
      p.mat = mat;
      for (int k = 0; k < 2; ++k) {
        p.t = (k == 0 ? (-b - rd) : (-b + rd)) / (2 * a);
        p.normal = ray.evaluate(p.t).affine() - c;
        p.tu = float(std::acos(double(p.normal.z / r)) / M_PI);
        p.tv = float(std::atan2(double(p.normal.x), double(p.normal.y)) / M_PI / 2 + 0.5);
        out.push_back(p);
      }
    }
    return out;
  }
  AABB box() const override { V3 rv(r, r, r); return AABB(c - rv, c + rv); }
};

struct CsgBox : CsgNode {
  V3 lo, hi; const Material* mat;
  CsgBox(V3 a, V3 b, const Material* m) : lo(a), hi(b), mat(m) {}
  std::list<CsgParam> params(const Ray& ray) const override {
    std::list<CsgParam> out;
    CsgParam p;
    p.mat = mat;
    float tmin = -kInf, tmax = kInf;
    for (int i = 0; i < 3; ++i) {
      float a = 1 / ray.d[i];
      V3 n;
      float tn, tx;
      if (a >= 0) { tn = (lo - ray.o)[i]; tx = (hi - ray.o)[i]; n.set(i, -1); }
      else { tn = (hi - ray.o)[i]; tx = (lo - ray.o)[i]; n.set(i, 1); }
      tn *= a;
      tx *= a;
      if (tn > tmin) { tmin = tn; p.normal = n; }
      if (tx < tmax) tmax = tx;
      if (tmin > tmax) return out;
    }
    p.t = tmin;
    out.push_back(p);
    p.t = tmax;  /* the exit keeps the entry face's normal */
    out.push_back(p);
    return out;
  }
  AABB box() const override { return AABB(lo, hi); }
};

struct CsgOp : CsgNode {
  int op;  /* gbrt_csg_op */
  std::unique_ptr<CsgNode> left, right;
  bool inside(bool l, bool r) const {
    switch (op) {
      case GBRT_CSG_ISECT: return l && r;
      case GBRT_CSG_UNION: return l || r;
      case GBRT_CSG_DIFF: return l && !r;
      default: return l != r;
    }
  }
  std::list<CsgParam> params(const Ray& ray) const override {
    bool li = false, ri = false;
    std::list<CsgParam> L = left->params(ray), R = right->params(ray), out;
    auto i = L.begin();
    auto j = R.begin();
    while (i != L.end() || j != R.end()) {
      bool takeL = i != L.end() && (j == R.end() || i->t <= j->t);
      bool was = inside(li, ri);
      bool& cur = takeL ? li : ri;
      cur = !cur;
      if (was != inside(li, ri)) out.push_back(takeL ? *i : *j);
      if (takeL) ++i; else ++j;
    }
    return out;
  }
  AABB box() const override { AABB b = left->box(); AABB c = right->box(); b.includeOther(c); return b; }
};

struct CsgObject : Intersectable {
  std::unique_ptr<CsgNode> root;
  Hit intersect(const Ray& ray) const override {
    std::list<CsgParam> ps = root->params(ray);
    if (ps.empty() || ray.from > ps.back().t) return Hit();
    for (auto& p : ps) {
      if (p.t >= ray.from) {
        if (p.t > ray.to) return Hit();
        Hit h(p.t, ray, p.mat, p.normal, prim);
        h.tu = p.tu;
        h.tv = p.tv;
        return h;
      }
    }
    return Hit();
  }
  AABB bbox() const override { return root->box(); }
};

/* Plane, src/plane.cpp:27-46. */
struct Plane : Intersectable {
  V4 P; const Material* mat;
  Plane(V4 p, const Material* m) : P(p), mat(m) {}
  Hit intersect(const Ray& ray) const override {
    if (prim == tIgnorePrim) return Hit();
    float d = -dot(ray.d, P.xyz());
    float u = dot4(V4(ray.o, 1), P);
    float t = u / d;
    if (ray.inRange(t)) return Hit(t, ray, mat, P.xyz(), prim);
    return Hit();
  }
  AABB bbox() const override { return AABB(V3(-kInf, -kInf, -kInf), V3(kInf, kInf, kInf)); }
};

/* IntersectableList, src/intersectablelist.cpp:30-78. */
struct IntersectableList : Intersectable {
  std::vector<Intersectable*> comps;
  Hit intersect(const Ray& r) const override {
    Ray ray = r;
    Hit hit;
    for (auto* c : comps) {
      Hit cur = c->intersect(ray);
      if (cur.intersects()) {
        ray = Ray(ray.o, ray.d, ray.from, cur.t);
        hit = cur;
      }
    }
    return hit;
  }
  AABB bbox() const override { AABB b; for (auto* c : comps) b.includeOther(c->bbox()); return b; }
  void contained(std::vector<Intersectable*>& out) override { for (auto* c : comps) c->contained(out); }
};

/* BVHNode, src/bvh.cpp:62-149: median split by box centre on the longest
 * axis; traversal visits both children and keeps the closer hit, the right
 * child winning ties. */
struct BVHNode : Intersectable {
  Intersectable *left, *right;
  AABB bb;
  BVHNode(Intersectable* l, Intersectable* r, AABB b) : left(l), right(r), bb(b) {}
  Hit intersect(const Ray& ray) const override {
    std::list<AABB::Param> params = bb.csgIntersection(ray);
    if (params.empty() || params.front().t > ray.to || params.back().t < ray.from) return Hit();
    Hit lh = left->intersect(ray);
    Hit rh = right->intersect(ray);
    if (!rh.intersects() || lh.t < rh.t) return lh;
    return rh;
  }
  AABB bbox() const override { return bb; }
  void contained(std::vector<Intersectable*>& out) override { left->contained(out); right->contained(out); }
};

static Intersectable* buildBVH(std::vector<Intersectable*> items, std::vector<std::unique_ptr<Intersectable>>& pool) {
  if (items.size() == 1) return items.front();
  AABB bb;
  for (auto* it : items) bb.includeOther(it->bbox());
  V3 diff = bb.mx - bb.mn;
  int axis = (diff.x > diff.y && diff.x > diff.z) ? 0 : (diff.y > diff.z ? 1 : 2);
  std::vector<std::pair<float, Intersectable*>> keyed;
  keyed.reserve(items.size());
  for (auto* it : items) {
    AABB b = it->bbox();
    float k = (b.mx + b.mn)[axis];
    if (std::isnan(k)) k = -kInf; /* NaN-safe stand-in for unbounded boxes */
    keyed.push_back({k, it});
  }
  std::stable_sort(keyed.begin(), keyed.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
  size_t half = keyed.size() / 2;
  std::vector<Intersectable*> l, r;
  for (size_t i = 0; i < keyed.size(); ++i) (i < half ? l : r).push_back(keyed[i].second);
  if (l.empty() || r.empty()) {
    auto* list = new IntersectableList();
    list->comps = items;
    pool.emplace_back(list);
    return list;
  }
  Intersectable* L = buildBVH(l, pool);
  Intersectable* R = buildBVH(r, pool);
  auto* node = new BVHNode(L, R, bb);
  pool.emplace_back(node);
  return node;
}

/* IntersectableInstance, src/intersectableinstance.cpp:24-46 with
 * HitRecord::transform, src/hitrecord.h:79-84: the ray moved into the
 * child's space by the inverse transform (origin as a point, direction as a
 * vector, not renormalised, each row summed left to right), the hit point
 * mapped back, the normal by the inverse transpose. Here the inverse is the
 * affine one computed in double from the cofactors (as the CUDA path does)
 * and the mapped normal is normalised; the hit reports the instance's id. */
struct IntersectableInstance : Intersectable {
  float fwd[12], inv[12];  /* row-major 3 x 4: object -> world, world -> object */
  Intersectable* child = nullptr;
  static V3 mapP(const float* m, V3 p) {
    return V3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
  }
  static V3 mapV(const float* m, V3 v) {
    return V3((m[0] * v.x + m[1] * v.y) + m[2] * v.z, (m[4] * v.x + m[5] * v.y) + m[6] * v.z,
              (m[8] * v.x + m[9] * v.y) + m[10] * v.z);
  }
  Hit intersect(const Ray& ray) const override {
    Ray tr(mapP(inv, ray.o), mapV(inv, ray.d), ray.from, ray.to);
    Hit h = child->intersect(tr);
    if (!h.intersects()) return h;
    h.point = V4(mapP(fwd, h.point.affine()), 1);
    h.ray = ray;
    V3 n = h.normal;
    h.normal = V3(inv[0] * n.x + inv[4] * n.y + inv[8] * n.z, inv[1] * n.x + inv[5] * n.y + inv[9] * n.z,
                  inv[2] * n.x + inv[6] * n.y + inv[10] * n.z).normalized();
    h.prim = prim;
    return h;
  }
  /* IntersectableInstance::createBoundingBox: the child's box corners mapped */
  AABB bbox() const override {
    AABB c = child->bbox(), b;
    for (int k = 0; k < 8; ++k)
      b.includePoint(mapP(fwd, V3((k & 1) ? c.mx.x : c.mn.x, (k & 2) ? c.mx.y : c.mn.y, (k & 4) ? c.mx.z : c.mn.z)));
    return b;
  }
};

/* The prim id of an instanced mesh's triangles: never an ignored prim. */
static const int kMeshTrianglePrim = -0x7ffffff0;

/* Inverse of an affine row-major 3 x 4 matrix in double, rounded to float. */
static bool affineInverse(const float in[12], float out[12]) {
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

/* ---------------------------------------------------------------- Light -- */

struct Light : Intersectable {
  virtual C3 intensity(const Hit& hit, V3& direction, const Intersectable& scene, const Sample& s) const = 0;
};

/* AreaLight, src/arealight.cpp:31-118: a one-sided parallelogram emitter
 * that is also geometry and its own material. */
struct AreaLight : Light, Material {
  V3 origin, u, v, normal; C3 Le;
  AreaLight(V3 o, V3 uu, V3 vv, C3 le) : origin(o), u(uu), v(vv), normal(cross(uu, vv)), Le(le) {}
  V3 location(double px, double py) const { return origin + float(px) * u + float(py) * v; }
  C3 intensityDir(V3 direction) const {
    float c = dot(direction.normalized(), normal.normalized()) / direction.lengthSquared() * normal.length();
    if (c < 0) c = 0;
    return c * Le;
  }
  C3 intensity(const Hit& hit, V3& direction, const Intersectable& scene, const Sample& s) const override {
    V3 at = hit.point.affine();
    V3 lp = location(s.x, s.y);
    direction = at - lp;
    Hit sh = scene.intersect(Ray(at, -direction.normalized(), kEpsilon, direction.length() - kEpsilon));
    if (sh.intersects() && sh.mat != static_cast<const Material*>(this)) return C3();
    return intensityDir(direction);
  }
  Hit intersect(const Ray& ray) const override {
    if (prim == tIgnorePrim) return Hit();
    V3 ad = ray.o - origin;
    V3 abxac = cross(u, v);
    float w = -dot(abxac, ray.d);
    if (w == 0) return Hit();
    float t = dot(abxac, ad) / w;
    if (!ray.inRange(t)) return Hit();
    V3 adxde = cross(ad, ray.d);
    float uu = dot(adxde, v) / w;
    if (uu < 0 || uu > 1) return Hit();
    float vv = -dot(adxde, u) / w;
    if (vv < 0 || vv > 1) return Hit();
    return Hit(t, ray, this, normal, prim, uu, vv);
  }
  AABB bbox() const override {
    AABB b; b.includePoint(origin); b.includePoint(origin + u); b.includePoint(origin + v); b.includePoint(origin + u + v);
    return b;
  }
  C3 emission(const Hit& hit) const override { return intensityDir(-hit.ray.d); }
  bool emitsLight() const override { return true; }
  V3 outDirection(const Hit&, Sample, float& pdf, C3& b) const override { b = C3(); pdf = 0; return V3(); }
};

/* PointLight, src/pointlight.cpp:29-70: never hit; bbox at the origin. */
struct PointLight : Light {
  V3 loc; C3 I;
  PointLight(V3 l, C3 i) : loc(l), I(i) {}
  C3 intensity(const Hit& hit, V3& direction, const Intersectable& scene, const Sample&) const override {
    V3 at = hit.point.affine();
    direction = at - loc;
    V3 dd = at - loc;
    Hit h = scene.intersect(Ray(at, -dd.normalized(), kEpsilon, dd.length() - kEpsilon));
    if (h.intersects()) return C3();
    return I * (1 / direction.lengthSquared());
  }
  Hit intersect(const Ray&) const override { return Hit(); }
  AABB bbox() const override { return AABB(V3(), V3()); }
};

/* ConeLight, src/conelight.cpp:31-60: a point light limited to a cone. */
struct ConeLight : Light {
  V3 loc, axis; float angle; C3 I;
  ConeLight(V3 l, V3 a, float ang, C3 i) : loc(l), axis(a), angle(ang), I(i) {}
  C3 intensity(const Hit& hit, V3& direction, const Intersectable& scene, const Sample&) const override {
    V3 at = hit.point.affine();
    direction = at - loc;
    Hit sh = scene.intersect(Ray(at, -direction.normalized(), kEpsilon, direction.length() - kEpsilon));
    float rayAngle = float(std::acos(double(dot(direction.normalized(), axis.normalized()))));
    if (0 <= rayAngle && rayAngle <= angle && !sh.intersects()) return I * (1 / direction.lengthSquared());
    return C3();
  }
  Hit intersect(const Ray&) const override { return Hit(); }
  AABB bbox() const override { return AABB(V3(), V3()); }
};

/* BlackLight, src/blacklight.cpp:5-24. */
struct BlackLight : Light {
  C3 intensity(const Hit&, V3&, const Intersectable&, const Sample&) const override { return C3(); }
  Hit intersect(const Ray&) const override { return Hit(); }
  AABB bbox() const override { return AABB(V3(), V3()); }
};

/* EnvironmentMap, src/environmentmap.cpp:16-108: an angular light probe (or,
 * as an extension, an equirectangular map) at infinity. */
struct EnvironmentMap : Light, Material {
  int W, H, mapping; std::vector<float> tex; C3 coef;
  C3 texel(int row, int col) const {
    row = std::min(std::max(row, 0), H - 1);
    col = std::min(std::max(col, 0), W - 1);
    const float* p = &tex[(size_t(row) * W + col) * 3];
    return C3(p[0], p[1], p[2]);
  }
  C3 get(V3 d) const {
    if (mapping == GBRT_ENV_LATLONG) {
      float u = float(std::atan2(double(d.x), double(-d.z)) / (2 * M_PI) + 0.5);
      float v = float(std::acos(double(std::min(1.f, std::max(-1.f, d.y)))) / M_PI);
      int x = std::min(int(u * W), W - 1), y = std::min(int(v * H), H - 1);
      return mul(texel(y, x), coef);
    }
    float cx = d.y, cy = -d.z;
    float len = float(std::sqrt(double(cx) * cx + double(cy) * cy));
    float f = float(std::acos(double(d.x)) / (len * M_PI));
    cx *= f; cy *= f;
    int x = int(float(((cx + 1.0) / 2.0) * W - 1));
    int y = int(float(((cy + 1.0) / 2.0) * H - 1));
    return mul(texel(std::min(y, W - 1), std::min(x, H - 1)), coef);
  }
  C3 intensity(const Hit& hit, V3& direction, const Intersectable& scene, const Sample& s) const override {
    V3 at = hit.point.affine();
    float pdf;
    direction = -s.cosineDirection(hit.normal, pdf);
    Hit sh = scene.intersect(Ray(at, direction, -kInf, -kEpsilon));
    if (sh.intersects()) return C3();
    return (1 / pdf) * get(direction);
  }
  Hit intersect(const Ray& ray) const override {
    if (prim == tIgnorePrim) return Hit();
    if (std::isinf(ray.to)) return Hit(ray.to, ray, this, -ray.d.normalized(), prim);
    return Hit();
  }
  AABB bbox() const override { return AABB(V3(-kInf, -kInf, -kInf), V3(kInf, kInf, kInf)); }
  C3 emission(const Hit& hit) const override { return get(hit.ray.d.normalized()); }
  bool emitsLight() const override { return true; }
  V3 outDirection(const Hit&, Sample, float& pdf, C3& b) const override { b = C3(); pdf = 0; return V3(); }

  /* Importance sampling for the physical estimator (not in the renderer,
   * whose NEE draws the cosine, :40-54). A piecewise-constant density over
   * the mapping's parameter square, H rows x W cells: lat-long (u, v) =
   * (atan2(x, -z) / 2 pi + 1/2, acos(y) / pi) with 2 pi^2 sin(theta) of solid
   * angle per unit area; the angular probe's disc (u, v) = ((cx + 1) / 2,
   * (cy + 1) / 2), r = theta / pi, 4 pi^2 sin(theta) / theta. A cell weighs
   * the luminance get() returns for its centre times that factor there; row
   * and cell CDFs are summed in double and stored in float, and a cell's
   * density is the product of its float CDF steps times W H. */
  std::vector<float> marg, cond, dens;
  bool sampled = false;

  void buildTables() {
    const double pi = M_PI;
    std::vector<double> w(size_t(W) * H, 0.0), rs(size_t(H), 0.0);
    double tot = 0;
    for (int r = 0; r < H; ++r) {
      for (int c = 0; c < W; ++c) {
        double u = (c + 0.5) / W, v = (r + 0.5) / H, jac;
        V3 d;
        if (mapping == GBRT_ENV_LATLONG) {
          double ph = 2 * pi * (u - 0.5), th = pi * v;
          d = V3(float(std::sin(th) * std::sin(ph)), float(std::cos(th)), float(-std::sin(th) * std::cos(ph)));
          jac = 2 * pi * pi * std::sin(th);
        } else {
          double cx = 2 * u - 1, cy = 2 * v - 1, rr = std::sqrt(cx * cx + cy * cy);
          if (!(rr < 1)) continue;
          double th = pi * rr, k = rr > 0 ? std::sin(th) / rr : 0;
          d = rr > 0 ? V3(float(std::cos(th)), float(k * cx), float(-k * cy)) : V3(1, 0, 0);
          jac = rr > 0 ? 4 * pi * pi * std::sin(th) / th : 4 * pi * pi;
        }
        C3 L = get(d);
        double l = 0.299 * L.r + 0.587 * L.g + 0.114 * L.b;
        double x = (l > 0 && std::isfinite(l)) ? l * jac : 0.0;
        w[size_t(r) * W + c] = x;
        rs[r] += x;
      }
      tot += rs[r];
    }
    if (!(tot > 0) || !std::isfinite(tot)) return;
    marg.assign(size_t(H) + 1, 0.f);
    cond.assign(size_t(H) * (W + 1), 0.f);
    dens.assign(size_t(H) * W, 0.f);
    double acc = 0;
    for (int r = 0; r < H; ++r) {
      marg[r] = float(acc / tot);
      acc += rs[r];
      double a = 0;
      for (int c = 0; c < W; ++c) {
        cond[size_t(r) * (W + 1) + c] = rs[r] > 0 ? float(a / rs[r]) : float(c) / float(W);
        a += w[size_t(r) * W + c];
      }
      cond[size_t(r) * (W + 1) + W] = 1.f;
    }
    marg[H] = 1.f;
    for (int r = 0; r < H; ++r)
      for (int c = 0; c < W; ++c)
        dens[size_t(r) * W + c] = (marg[r + 1] - marg[r]) *
                                  (cond[size_t(r) * (W + 1) + c + 1] - cond[size_t(r) * (W + 1) + c]) * float(W) *
                                  float(H);
    sampled = true;
  }
  /* Density per solid angle of the unit direction d. */
  float pdf(V3 d) const {
    double u, v, jac;
    if (mapping == GBRT_ENV_LATLONG) {
      double y = std::min(1.0, std::max(-1.0, double(d.y)));
      u = std::atan2(double(d.x), double(-d.z)) / (2 * M_PI) + 0.5;
      v = std::acos(y) / M_PI;
      jac = 2 * M_PI * M_PI * std::sqrt(std::max(0.0, 1 - y * y));
    } else {
      double th = std::acos(std::min(1.0, std::max(-1.0, double(d.x))));
      double q = std::sqrt(double(d.y) * d.y + double(d.z) * d.z);
      double f = q > 0 ? th / (q * M_PI) : 0;
      u = (d.y * f + 1) / 2;
      v = (-d.z * f + 1) / 2;
      jac = th > 0 ? 4 * M_PI * M_PI * q / th : 4 * M_PI * M_PI;
    }
    if (!(jac > 0)) return 0;
    int c = std::min(std::max(int(float(u) * W), 0), W - 1), r = std::min(std::max(int(float(v) * H), 0), H - 1);
    return float(dens[size_t(r) * W + c] / jac);
  }
  static int cdfFind(const float* cdf, int n, float x) {
    int lo = 0, hi = n;
    while (hi - lo > 1) {
      int mid = (lo + hi) / 2;
      if (cdf[mid] <= x) lo = mid; else hi = mid;
    }
    return lo;
  }
  /* Draws a direction with u1 (row) and u2 (cell); false outside the disc. */
  bool sample(float u1, float u2, V3& d, float& p) const {
    int r = cdfFind(marg.data(), H, u1);
    const float* cr = &cond[size_t(r) * (W + 1)];
    int c = cdfFind(cr, W, u2);
    float fv = std::min((u1 - marg[r]) / (marg[r + 1] - marg[r]), 0.99999994f);
    float fu = std::min((u2 - cr[c]) / (cr[c + 1] - cr[c]), 0.99999994f);
    double u = (float(c) + fu) / float(W), v = (float(r) + fv) / float(H), jac;
    if (mapping == GBRT_ENV_LATLONG) {
      double ph = M_PI * (2 * u - 1), th = M_PI * v;
      d = V3(float(std::sin(th) * std::sin(ph)), float(std::cos(th)), float(-std::sin(th) * std::cos(ph)));
      jac = 2 * M_PI * M_PI * std::sin(th);
    } else {
      double cx = 2 * u - 1, cy = 2 * v - 1, rr = std::sqrt(cx * cx + cy * cy);
      if (!(rr < 1)) return false;
      double th = M_PI * rr, k = rr > 0 ? std::sin(th) / rr : 0;
      d = rr > 0 ? V3(float(std::cos(th)), float(k * cx), float(-k * cy)) : V3(1, 0, 0);
      jac = rr > 0 ? 4 * M_PI * M_PI * std::sin(th) / th : 4 * M_PI * M_PI;
    }
    if (!(jac > 0)) return false;
    p = float(dens[size_t(r) * W + c] / jac);
    return p > 0;
  }
};

/* --------------------------------------------------------------- Camera -- */

/* Camera::init / getRay, src/camera.cpp:34-58. */
struct Camera {
  float t, b, l, r, aspect;
  int W, H;
  M4 ext;
  void init(V3 cop, V3 lookAt, V3 up, float fov, int w, int h) {
    W = w; H = h;
    V3 ww = (cop - lookAt).normalized();
    V3 uu = normalOf(up, ww);
    V3 vv = cross(ww, uu);
    aspect = float(w) / h;
    t = float(std::tan(double(fov / 2))); b = -t; r = aspect * t; l = -r;
    ext.setColumn(0, V4(uu, 0)); ext.setColumn(1, V4(vv, 0)); ext.setColumn(2, V4(ww, 0)); ext.setColumn(3, V4(cop, 1));
  }
  Ray getRay(double px, double py) const {
    V4 pl(float(l + (r - l) * (px + 0.5) / W), float(t + (b - t) * (py + 0.5) / H), -1, 0);
    return Ray(V3(0, 0, 0), pl.xyz()).transform(ext);
  }
};

/* ---------------------------------------------------------------- Scene -- */

struct Scene {
  std::vector<std::unique_ptr<Intersectable>> pool;
  std::vector<std::unique_ptr<Material>> mats;
  std::vector<const Material*> matTable;
  std::vector<const Light*> lights;
  Intersectable* root = nullptr;
  int nPrims = 0;
};

static C3 spec3(const float* p) { return C3(p[0], p[1], p[2]); }
static V3 vec3(const float* p) { return V3(p[0], p[1], p[2]); }

/* scene_builder::getScene, src/sceneast.cpp:673-695: the root is
 * IntersectableList(lights..., scene contents), then createBVH() flattens
 * nested lists into leaves (src/intersectable.cpp:11-14). */
static Scene* buildScene(const gbrt_scene_desc* d, bool useBVH) {
  auto* s = new Scene();
  for (int i = 0; i < d->n_materials; ++i) {
    const gbrt_material& m = d->materials[i];
    Material* mm = nullptr;
    switch (m.type) {
      case GBRT_MAT_DIFFUSE: mm = new DiffuseMaterial(spec3(m.kd)); break;
      case GBRT_MAT_MIRROR: mm = new MirrorMaterial(); break;
      case GBRT_MAT_PHONG: mm = new PhongMaterial(spec3(m.kd), spec3(m.ks), m.exponent); break;
      case GBRT_MAT_BLINN: mm = new BlinnMaterial(spec3(m.kd), spec3(m.ks), m.exponent); break;
      case GBRT_MAT_TRANSPARENT: mm = new TransparentMaterial(m.ior); break;
      case GBRT_MAT_TEXTURE:
        if (m.texture >= 0 && m.texture < d->n_textures) {
          const gbrt_texture& tx = d->textures[m.texture];
          mm = new TextureMaterial(tx.width, tx.height, tx.texels, spec3(m.kd), m.exponent);
        }
        break;
      default: mm = nullptr;
    }
    if (mm) { s->mats.emplace_back(mm); s->matTable.push_back(mm); }
    else s->matTable.push_back(&gDark);
  }
  auto mat = [&](int i) -> const Material* {
    if (i < 0 || i >= int(s->matTable.size())) return &gDark;
    return s->matTable[i];
  };
  std::vector<Intersectable*> top;
  int pid = 0;
  for (int i = 0; i < d->n_lights; ++i, ++pid) {
    const gbrt_light& L = d->lights[i];
    Light* l = nullptr;
    if (L.type == GBRT_LIGHT_AREA) l = new AreaLight(vec3(L.origin), vec3(L.u), vec3(L.v), spec3(L.intensity));
    else if (L.type == GBRT_LIGHT_POINT) l = new PointLight(vec3(L.origin), spec3(L.intensity));
    else if (L.type == GBRT_LIGHT_CONE) l = new ConeLight(vec3(L.origin), vec3(L.u), L.v[0], spec3(L.intensity));
    else if (L.type == GBRT_LIGHT_ENV && d->env && d->env->texels) {
      auto* e = new EnvironmentMap();
      e->W = d->env->width; e->H = d->env->height; e->mapping = d->env->mapping;
      e->tex.assign(d->env->texels, d->env->texels + size_t(e->W) * e->H * 3);
      e->coef = spec3(L.intensity);
      if (!(d->flags & GBRT_SCENE_ENV_UNIFORM)) e->buildTables();
      l = e;
    } else l = new BlackLight();
    l->prim = pid;
    s->pool.emplace_back(l);
    s->lights.push_back(l);
    top.push_back(l);
  }
  for (int64_t i = 0; i < d->n_tri; ++i, ++pid) {
    const float* p = d->tri_pos + 9 * i;
    const Material* m = mat(d->tri_mat ? d->tri_mat[i] : 0);
    Triangle* t;
    bool useN = false;
    if (d->tri_nrm) {
      const float* n = d->tri_nrm + 9 * i;
      useN = !(vec3(n).isNull() || vec3(n + 3).isNull() || vec3(n + 6).isNull());
      if (useN) t = new Triangle(vec3(p), vec3(p + 3), vec3(p + 6), vec3(n), vec3(n + 3), vec3(n + 6), m);
    }
    if (!useN) t = new Triangle(vec3(p), vec3(p + 3), vec3(p + 6), m);
    if (d->tri_uv) {
      const float* uv = d->tri_uv + 6 * i;
      t->t1[0] = uv[0]; t->t1[1] = uv[1];
      t->t2[0] = uv[2]; t->t2[1] = uv[3];
      t->t3[0] = uv[4]; t->t3[1] = uv[5];
    }
    t->prim = pid;
    s->pool.emplace_back(t);
    top.push_back(t);
  }
  for (int i = 0; i < d->n_quads; ++i, ++pid) {
    const gbrt_quad& q = d->quads[i];
    auto* qq = new Quad(vec3(q.p[0]), vec3(q.p[1]), vec3(q.p[2]), vec3(q.p[3]), mat(q.material));
    qq->setPrim(pid);
    s->pool.emplace_back(qq);
    top.push_back(qq);
  }
  for (int i = 0; i < d->n_spheres; ++i, ++pid) {
    const gbrt_sphere& q = d->spheres[i];
    auto* sp = new Sphere(vec3(q.center), q.radius, mat(q.material));
    sp->prim = pid;
    s->pool.emplace_back(sp);
    top.push_back(sp);
  }
  for (int i = 0; i < d->n_planes; ++i, ++pid) {
    const gbrt_plane& q = d->planes[i];
    auto* pl = new Plane(V4(q.plane[0], q.plane[1], q.plane[2], q.plane[3]), mat(q.material));
    pl->prim = pid;
    s->pool.emplace_back(pl);
    top.push_back(pl);
  }
  std::function<CsgNode*(int)> csgBuild = [&](int i) -> CsgNode* {
    const gbrt_csg_node& nd = d->csg_nodes[i];
    if (nd.op == GBRT_CSG_SPHERE) return new CsgSphere(vec3(nd.a), nd.b[0], mat(nd.material));
    if (nd.op == GBRT_CSG_BOX) return new CsgBox(vec3(nd.a), vec3(nd.b), mat(nd.material));
    auto* op = new CsgOp();
    op->op = nd.op;
    op->left.reset(csgBuild(nd.left));
    op->right.reset(csgBuild(nd.right));
    return op;
  };
  for (int i = 0; i < d->n_csg; ++i, ++pid) {
    auto* o = new CsgObject();
    o->root.reset(csgBuild(d->csg_roots[i]));
    o->prim = pid;
    s->pool.emplace_back(o);
    top.push_back(o);
  }
  /* Instanced meshes: each instance gets a BVH of its mesh's triangles (the
   * renderer's BVHCreator builds one per instance node, sceneast.cpp:
   * 184-205). */
  for (int i = 0; i < d->n_instances; ++i, ++pid) {
    const gbrt_instance& in = d->instances[i];
    const gbrt_mesh& gm = d->meshes[in.mesh];
    std::vector<Intersectable*> tris;
    for (int64_t k = 0; k < gm.n_tri; ++k) {
      const float* p = gm.tri_pos + 9 * k;
      const Material* m = mat(gm.tri_mat ? gm.tri_mat[k] : 0);
      Triangle* t = nullptr;
      if (gm.tri_nrm) {
        const float* n = gm.tri_nrm + 9 * k;
        if (!(vec3(n).isNull() || vec3(n + 3).isNull() || vec3(n + 6).isNull()))
          t = new Triangle(vec3(p), vec3(p + 3), vec3(p + 6), vec3(n), vec3(n + 3), vec3(n + 6), m);
      }
      if (!t) t = new Triangle(vec3(p), vec3(p + 3), vec3(p + 6), m);
      t->prim = kMeshTrianglePrim;
      s->pool.emplace_back(t);
      tris.push_back(t);
    }
    auto* inst = new IntersectableInstance();
    std::memcpy(inst->fwd, in.transform, sizeof inst->fwd);
    if (!affineInverse(in.transform, inst->inv)) { delete inst; continue; }
    if (useBVH) {
      inst->child = buildBVH(tris, s->pool);
    } else {  /* --no-bvh: the mesh's triangles as a list, in file order */
      auto* ml = new IntersectableList();
      ml->comps = tris;
      s->pool.emplace_back(ml);
      inst->child = ml;
    }
    inst->prim = pid;
    s->pool.emplace_back(inst);
    top.push_back(inst);
  }
  s->nPrims = pid;
  /* The root list in the scene's list order (gbrt_scene_desc.list_rank):
   * with --no-bvh the renderer tests it in that order and the later entry
   * wins exact ties (src/intersectablelist.cpp:29-47). */
  if (d->list_rank) {
    std::stable_sort(top.begin(), top.end(), [&](const Intersectable* a, const Intersectable* b) {
      return d->list_rank[a->prim] < d->list_rank[b->prim];
    });
  }
  if (useBVH && !top.empty()) {
    s->root = buildBVH(top, s->pool);
  } else {
    auto* list = new IntersectableList();
    list->comps = top;
    s->pool.emplace_back(list);
    s->root = list;
  }
  return s;
}

/* ------------------------------------------------------- createPath etc. -- */

struct PathVertex { C3 alpha; Hit hit; };
using Path = std::list<PathVertex>;

struct Draws {
  /* one camera sample's random numbers */
  int pathLength;
  std::vector<Sample> pathSamples, lightSamples;
  std::vector<int> lightIndex;
};

/* Renderer::createPath(primaryRay, scene, samples, ...), src/renderer.cpp:69-106,
 * with MAX_DEPTH (src/renderer.h:38) a run-time value. */
static Path createPath(const Ray& primary, const Intersectable& scene, const Draws& dr, int maxDepth,
                       float rrPdf, int rrStart, uint64_t* rays) {
  Path result;
  int pathLength = dr.pathLength;
  C3 alpha(1, 1, 1);
  Hit hit = scene.intersect(primary);
  ++*rays;
  for (int i = 0; i < pathLength; ++i) {
    if (!hit.intersects()) return result;
    float pdf; C3 brdf;
    V3 out = hit.mat->outDirection(hit, dr.pathSamples[i], pdf, brdf);
    if (hit.mat->emitsLight()) {
      result.push_back({alpha, hit});
      return result;
    } else if (hit.mat->isSpecular()) {
      if (i == pathLength - 1 && pathLength < maxDepth) pathLength++;
    } else {
      result.push_back({alpha, hit});
      if (pdf == 0 || alpha.isZero()) return result;
      float c = std::fabs(dot(out.normalized(), hit.normal.normalized()));
      alpha = mul(alpha, brdf) * (c / pdf);
      if (i > rrStart) alpha = alpha * (1 / rrPdf);
    }
    hit = scene.intersect(Ray(hit.point.affine(), out));
    ++*rays;
  }
  return result;
}

/* UniDiPathTracingIntegrator::integrate(path, ...),
 * src/unidipathtracingintegrator.cpp:48-107. */
static C3 integratePath(const Path& path, const Intersectable& scene, const std::vector<const Light*>& lights,
                        const Draws& dr, uint64_t* shadowRays) {
  C3 color;
  auto it = path.begin();
  if (it != path.end()) {
    C3 e = it->hit.mat->emission(it->hit);
    if (e != C3()) return e;
  }
  int i = 0;
  for (; it != path.end(); ++it, ++i) {
    V3 direction;
    C3 L;
    auto next = std::next(it);
    const Hit& h = it->hit;
    if (next != path.end() && next->hit.mat->emitsLight()) {
      L = next->hit.mat->emission(next->hit);
      V4 lp = next->hit.point;
      if (lp.w == 0) direction = -lp.xyz();
      else direction = h.point.affine() - lp.affine();
    } else {
      if (lights.empty()) continue;
      L = lights[dr.lightIndex[i]]->intensity(h, direction, scene, dr.lightSamples[i]);
      ++*shadowRays;
    }
    C3 brdf = h.mat->brdf(h, direction);
    float inCos = dot(-direction.normalized(), h.normal.normalized());
    float outCos = dot(-h.ray.d.normalized(), h.normal.normalized());
    if (signum(inCos) == signum(outCos)) color = color + mul(mul(it->alpha, brdf), L) * std::fabs(inCos);
  }
  return color;
}

/* Draws of one camera sample. Mode 0: the renderer's order on a per-row
 * generator (src/renderer.cpp:47-66, src/unidipathtracingintegrator.cpp:36-44).
 * Mode 1: the counter-based stream, dimension layout
 *   0,1 jitter | 2 path length | 3+2i,4+2i path sample i |
 *   3+2D+3k, +1 light sample k, +2 light index k       (D = max depth). */
static void drawPath(Draws& dr, int maxDepth, float p, int nLights, Rng* rng, uint64_t key) {
  dr.pathSamples.resize(maxDepth);
  dr.lightSamples.resize(maxDepth);
  dr.lightIndex.resize(maxDepth);
  double ul = rng ? rng->uniform() : double(streamU(key, 2));
  if (p > 0) {
    int k = 0;
    if (p < 1) k = int(std::floor(std::log(1.0 - ul) / std::log(1.0 - double(p))));
    dr.pathLength = std::min(3 + std::max(k, 0), maxDepth);
  } else dr.pathLength = maxDepth;
  for (int i = 0; i < maxDepth; ++i) {
    if (rng) { double a = rng->uniform(), b = rng->uniform(); dr.pathSamples[i] = Sample(a, b); }
    else dr.pathSamples[i] = Sample(streamU(key, 3 + 2 * i), streamU(key, 4 + 2 * i));
  }
  for (int k = 0; k < maxDepth; ++k) {
    double a, b, c;
    if (rng) { a = rng->uniform(); b = rng->uniform(); c = rng->uniform(); }
    else {
      uint32_t base = 3 + 2 * maxDepth + 3 * k;
      a = streamU(key, base); b = streamU(key, base + 1); c = streamU(key, base + 2);
    }
    dr.lightSamples[k] = Sample(a, b);
    int li = nLights > 0 ? int(c * nLights) : 0;
    dr.lightIndex[k] = std::min(li, std::max(nLights - 1, 0));
  }
}


/* ===================================================== physical semantics ==
 * Not part of the renderer: the physically based estimator the GPU path
 * offers as GBRT_SEM_PHYSICAL, restated here from the same specification to
 * check it. Unbiased Russian roulette (survival 1 - p from the fourth vertex
 * on), emission on direct view and on BSDF-sampled hits weighted by the power
 * heuristic against next-event estimation (light chosen uniformly, with the
 * light-count factor), modified Phong and Blinn with their sampling pdfs, the
 * environment looked up in the direction the light arrives from, sampled
 * uniformly over the sphere for NEE. Directions wo / wi point away from the
 * surface; lobes are two-sided (the normal is flipped towards wo). Random
 * numbers per vertex i: dims 2+8i lobe, +1/+2 BSDF direction, +3 light index,
 * +4/+5 light sample, +6 roulette (dims 0/1: pixel jitter). */

struct PhysBsdf {
  int kind = -1;  /* 0 none, 1 diffuse, 2 phong, 3 blinn, 4 mirror, 5 glass */
  C3 kd, ks;
  float e = 0, ior = 1, pd = 1;
};

static PhysBsdf physOf(const Hit& h) {
  const Material* m = h.mat;
  PhysBsdf b;
  if (auto* d = dynamic_cast<const DiffuseMaterial*>(m)) { b.kind = 1; b.kd = d->color; }
  else if (auto* tx = dynamic_cast<const TextureMaterial*>(m)) { b.kind = 1; b.kd = tx->albedo(h); }
  else if (auto* ph = dynamic_cast<const PhongMaterial*>(m)) { b.kind = 2; b.kd = ph->color; b.ks = ph->spec; b.e = ph->e; }
  else if (auto* bl = dynamic_cast<const BlinnMaterial*>(m)) { b.kind = 3; b.kd = bl->kd; b.ks = bl->ks; b.e = bl->e; }
  else if (dynamic_cast<const MirrorMaterial*>(m)) b.kind = 4;
  else if (auto* t = dynamic_cast<const TransparentMaterial*>(m)) { b.kind = 5; b.ior = t->k; }
  else b.kind = 0;
  if (b.kind == 2 || b.kind == 3) {
    float rd = lum(b.kd), rs = lum(b.ks);
    b.pd = (rd + rs) > 0 ? rd / (rd + rs) : 1.f;
  }
  return b;
}

static float cosPowerPdf(float c, float e) { return c > 0 ? float((e + 1) / (2 * M_PI) * std::pow(double(c), double(e))) : 0.f; }

/* f(wo, wi) and pdf(wi) of a non-specular lobe; n faces wo. */
static C3 physEval(const PhysBsdf& b, V3 n, V3 wo, V3 wi, float& pdf) {
  pdf = 0;
  float ci = dot(n, wi), co = dot(n, wo);
  if (b.kind < 1 || b.kind > 3 || ci <= 0 || co <= 0) return C3();
  C3 diff = b.kd * float(1 / M_PI);
  if (b.kind == 1) { pdf = float(ci / M_PI); return diff; }
  if (b.kind == 2) {
    V3 r = 2 * co * n - wo;
    float ca = std::max(0.f, dot(r, wi));
    float sp = float((b.e + 2) / (2 * M_PI) * std::pow(double(ca), double(b.e)));
    pdf = float(b.pd * ci / M_PI) + (1 - b.pd) * cosPowerPdf(ca, b.e);
    return diff + b.ks * sp;
  }
  V3 h = (wi + wo).normalized();
  float nh = dot(n, h), oh = dot(wo, h);
  float D = float((b.e + 2) / (2 * M_PI) * std::pow(double(std::max(nh, 0.f)), double(b.e)));
  float G = std::min(1.f, std::min(2 * nh * co / oh, 2 * nh * ci / oh));
  pdf = float(b.pd * ci / M_PI) + (1 - b.pd) * (oh > 0 ? cosPowerPdf(nh, b.e) / (4 * oh) : 0.f);
  return diff + b.ks * (D * G / (4 * ci * co));
}

/* Samples wi; returns f * |cos| / pdf in weight (or 1 for specular lobes). */
static bool physSample(const PhysBsdf& b, V3 n, V3 wo, bool exiting, float u0, float u1, float u2, V3& wi, C3& weight,
                       float& pdf, bool& specular) {
  specular = false;
  pdf = 0;
  if (b.kind == 4) {
    wi = 2 * dot(n, wo) * n - wo;
    specular = true; weight = C3(1, 1, 1); pdf = 1;
    return true;
  }
  if (b.kind == 5) {
    /* n faces wo; leaving the medium the geometric normal points along the
     * ray (TransparentMaterial's test, src/transparentmaterial.cpp:43-51). */
    V3 d = -wo;
    float ratio = exiting ? b.ior : 1 / b.ior;
    float cosI = dot(-n, d);
    float cc = cosI * cosI;
    float sinO = float(ratio * std::sqrt(std::max(0., 1. - cc)));
    float cosO = float(std::sqrt(std::max(0., 1 - (ratio * ratio) * std::max(0., 1. - cc))));
    float rPerp = (cosI - ratio * cosO) / (cosI + ratio * cosO);
    float rPara = (ratio * cosI - cosO) / (ratio * cosI + cosO);
    float R = float(0.5 * (rPerp * rPerp + rPara * rPara));
    if (sinO > 1 || u0 < R) wi = reflect(d, n);
    else wi = ratio * d + (ratio * cosI - signum(cosI) * cosO) * n;
    specular = true; weight = C3(1, 1, 1); pdf = 1;
    return true;
  }
  if (b.kind < 1) return false;
  Sample s(u1, u2);
  float tmp;
  if (b.kind == 1 || u0 < b.pd) {
    wi = s.cosineDirection(n, tmp);
  } else if (b.kind == 2) {
    wi = s.cosinePowerDirection(2 * dot(n, wo) * n - wo, tmp, b.e);
  } else {
    V3 h = s.cosinePowerDirection(n, tmp, b.e);
    wi = 2 * dot(wo, h) * h - wo;
  }
  C3 f = physEval(b, n, wo, wi, pdf);
  if (!(pdf > 0)) return false;
  weight = f * (dot(n, wi) / pdf);
  return true;
}

static float powerHeuristic(float a, float b) { return a * a / (a * a + b * b); }

struct PhysStats { uint64_t rays = 0, shadow = 0; };

/* One camera sample under the physical estimator. u(dim) draws the numbers. */
template <typename U>
static C3 physRadiance(const Scene& s, const Ray& primary, int D, float p, U&& u, PhysStats& st) {
  C3 Lsum, alpha(1, 1, 1);
  Ray ray = primary;
  float prevPdf = 0;
  bool prevSpec = true;
  const int nL = int(s.lights.size());
  const float pChoose = nL > 0 ? 1.f / nL : 0.f;
  for (int i = 0; i < D; ++i) {
    Hit h = s.root->intersect(ray);
    ++st.rays;
    if (!h.intersects()) break;
    const uint32_t base = 2 + 8 * uint32_t(i);
    if (auto* al = dynamic_cast<const AreaLight*>(h.mat)) {
      V3 dn = ray.d.normalized();
      float cl = dot(-dn, al->normal.normalized());
      if (cl > 0) {
        float w = 1;
        if (!prevSpec) {
          float dist = h.t * ray.d.length();
          float pl = pChoose * dist * dist / (cl * al->normal.length());
          w = powerHeuristic(prevPdf, pl);
        }
        Lsum = Lsum + mul(alpha, al->Le) * w;
      }
      break;
    }
    if (auto* em = dynamic_cast<const EnvironmentMap*>(h.mat)) {
      V3 dn = ray.d.normalized();
      float pe = em->sampled ? em->pdf(dn) : float(1 / (4 * M_PI));
      float w = prevSpec ? 1.f : powerHeuristic(prevPdf, pChoose * pe);
      Lsum = Lsum + mul(alpha, em->get(dn)) * w;
      break;
    }
    PhysBsdf b = physOf(h);
    if (b.kind <= 0) break;
    V3 x = h.point.affine();
    V3 wo = -ray.d.normalized();
    V3 n = h.normal.normalized();
    bool flipped = dot(n, wo) < 0;
    if (flipped) n = -n;
    /* next-event estimation at non-specular vertices */
    if (b.kind <= 3 && nL > 0) {
      int li = std::min(int(double(u(base + 3)) * nL), nL - 1);
      const Light* L = s.lights[li];
      float lx = u(base + 4), ly = u(base + 5);
      V3 wi; float dist = 0, pl = 0; C3 Le; bool delta = false; int ignore = -1;
      bool ok = true;
      if (auto* a = dynamic_cast<const AreaLight*>(L)) {
        V3 y = a->origin + lx * a->u + ly * a->v;
        V3 d = y - x;
        dist = d.length();
        wi = d.normalized();
        float cl = dot(-wi, a->normal.normalized());
        if (cl > 0) { Le = a->Le; pl = pChoose * dist * dist / (cl * a->normal.length()); }
        else ok = false;
        ignore = a->prim;
      } else if (auto* pt = dynamic_cast<const PointLight*>(L)) {
        V3 d = pt->loc - x; dist = d.length(); wi = d.normalized();
        Le = pt->I * (1 / d.lengthSquared()); pl = pChoose; delta = true;
      } else if (auto* cn = dynamic_cast<const ConeLight*>(L)) {
        V3 d = cn->loc - x; dist = d.length(); wi = d.normalized();
        float ang = float(std::acos(double(dot(-wi, cn->axis.normalized()))));
        if (ang <= cn->angle) { Le = cn->I * (1 / d.lengthSquared()); pl = pChoose; delta = true; }
        else ok = false;
      } else if (auto* em = dynamic_cast<const EnvironmentMap*>(L)) {
        float pe = float(1 / (4 * M_PI));
        if (em->sampled) ok = em->sample(lx, ly, wi, pe);
        else wi = Sample(lx, ly).uniformSphere();
        dist = kInf;
        if (ok) Le = em->get(wi);
        pl = pChoose * pe;
      } else ok = false;
      if (ok && !Le.isZero()) {
        float pb;
        C3 f = physEval(b, n, wo, wi, pb);
        float ci = std::fabs(dot(n, wi));
        if (!f.isZero()) {
          float w = delta ? 1.f : powerHeuristic(pl, pb);
          C3 c = mul(mul(alpha, f), Le) * (ci * w / pl);
          ++st.shadow;
          Ray sr(x, wi, kEpsilon, std::isinf(dist) ? kInf : dist - kEpsilon);
          tIgnorePrim = ignore;
          Hit sh = s.root->intersect(sr);
          tIgnorePrim = -1;
          bool occluded = sh.intersects() && !std::isinf(sh.t);
          if (!occluded) Lsum = Lsum + c;
        }
      }
    }
    /* continue the path */
    V3 wi; C3 wgt; float pdf; bool spec;
    if (!physSample(b, n, wo, flipped, u(base + 0), u(base + 1), u(base + 2), wi, wgt, pdf, spec)) break;
    alpha = mul(alpha, wgt);
    if (i + 1 >= 3 && p > 0) {
      if (u(base + 6) < p) break;
      alpha = alpha * (1 / (1 - p));
    }
    prevPdf = pdf;
    prevSpec = spec;
    ray = Ray(x, wi);
  }
  return Lsum;
}
}  // namespace orc

/* ================================================================ C API == */

using namespace orc;

extern "C" {

void* orc_scene_create(const gbrt_scene_desc* desc, int use_bvh) {
  if (!desc) return nullptr;
  return buildScene(desc, use_bvh != 0);
}

void orc_scene_destroy(void* s) { delete static_cast<Scene*>(s); }

int orc_scene_prims(void* s) { return static_cast<Scene*>(s)->nPrims; }

static void fillHit(const Hit& h, gbrt_hit* o) {
  o->t = h.t;
  o->prim = h.intersects() ? h.prim : -1;
  o->u = h.bu;
  o->v = h.bv;
}

/* Closest hit of each ray: scene.object->intersect(Ray), src/scene.h:36. */
void orc_trace_closest(void* sp, const gbrt_ray* rays, int64_t n, gbrt_hit* hits, int threads) {
  Scene* s = static_cast<Scene*>(sp);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t i = 0; i < n; ++i) {
    const gbrt_ray& r = rays[i];
    Ray ray(V3(r.org[0], r.org[1], r.org[2]), V3(r.dir[0], r.dir[1], r.dir[2]), r.tmin, r.tmax);
    fillHit(s->root->intersect(ray), &hits[i]);
  }
}

/* Occlusion: some primitive other than ignore[i] hit in [tmin, tmax]; the
 * environment map (hit only at t = inf) never occludes. */
void orc_trace_any(void* sp, const gbrt_ray* rays, const int32_t* ignore, int64_t n, uint8_t* occ, int threads) {
  Scene* s = static_cast<Scene*>(sp);
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
#endif
  for (int64_t i = 0; i < n; ++i) {
    const gbrt_ray& r = rays[i];
    Ray ray(V3(r.org[0], r.org[1], r.org[2]), V3(r.dir[0], r.dir[1], r.dir[2]), r.tmin, r.tmax);
    tIgnorePrim = ignore ? ignore[i] : -1;
    Hit h = s->root->intersect(ray);
    tIgnorePrim = -1;
    occ[i] = (h.intersects() && !std::isinf(h.t)) ? 1 : 0;
  }
}

/* PerPixelRenderer::render, src/perpixelrenderer.cpp:43-101, over rows
 * [row_begin, row_end). film receives the per-pixel mean (BGR); sum / sumsq
 * (optional, double) the per-pixel sum and sum of squares of the per-sample
 * radiance. rng_mode 0: per-row combined Tausworthe generator seeded
 * height * seed + row; rng_mode 1: the counter-based stream shared with the
 * CUDA path. Returns 0 on success. */
int orc_render(void* sp, const gbrt_camera* cam, const gbrt_render_params* prm, int rng_mode, int row_begin,
               int row_end, int row_step, float* film, double* sum, double* sumsq, int threads,
               uint64_t* out_paths, uint64_t* out_rays, uint64_t* out_shadow) {
  Scene* s = static_cast<Scene*>(sp);
  if (!s || !cam || !prm) return 1;
  Camera camera;
  camera.init(vec3(cam->eye), vec3(cam->look_at), vec3(cam->up), cam->fov, cam->width, cam->height);
  const int W = cam->width, H = cam->height;
  const int xs = prm->x_samples, ys = prm->y_samples, spp = xs * ys;
  const int D = prm->max_depth;
  float p = prm->termination_prob;
  float rrPdf = p > 0 ? p : 1.f;
  const int rrStart = 3;
  if (row_begin < 0) row_begin = 0;
  if (row_end > H || row_end < 0) row_end = H;
  if (row_step < 1) row_step = 1;
  const int nRows = row_end > row_begin ? (row_end - row_begin + row_step - 1) / row_step : 0;
  uint64_t totRays = 0, totShadow = 0, totPaths = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic) reduction(+ : totRays, totShadow, totPaths)
#endif
  for (int ri = 0; ri < nRows; ++ri) {
    const int i = row_begin + ri * row_step;
    std::unique_ptr<TausRng> rng;
    if (rng_mode == 0) rng.reset(new TausRng(uint64_t(H) * prm->seed + uint64_t(i)));
    Draws dr;
    for (int j = 0; j < W; ++j) {
      /* JitteredSampler(xs, ys).getSamples(), src/jitteredsampler.cpp:23-35:
       * stratum (a, b) for a < xs (x, outer), b < ys (y, inner). */
      std::list<Sample> samples;
      std::vector<uint64_t> keys;
      for (int a = 0; a < xs; ++a)
        for (int b = 0; b < ys; ++b) {
          int sidx = a * ys + b;
          if (rng) {
            double ux = rng->uniform(), uy = rng->uniform();
            samples.push_back(Sample((ux + a) / xs, (uy + b) / ys));
          } else {
            uint64_t key = streamKey(prm->seed, (uint64_t(i) * W + j) * spp + sidx);
            keys.push_back(key);
            samples.push_back(Sample((streamU(key, 0) + a) / double(xs), (streamU(key, 1) + b) / double(ys)));
          }
        }
      double accB = 0, accG = 0, accR = 0, sqB = 0, sqG = 0, sqR = 0;
      float fB = 0, fG = 0, fR = 0;
      int sidx = 0;
      for (auto& smp : samples) {
        Ray ray = camera.getRay(double(j) + smp.x, double(i) + smp.y);
        uint64_t r = 0, sh = 0;
        C3 c;
        if (prm->semantics == GBRT_SEM_PHYSICAL) {
          PhysStats ps;
          uint64_t key = rng ? 0 : keys[sidx];
          TausRng* tr = rng.get();
          c = physRadiance(*s, ray, D, p, [&](uint32_t dim) -> float {
            return tr ? float(tr->uniform()) : streamU(key, dim);
          }, ps);
          r = ps.rays; sh = ps.shadow;
        } else {
          drawPath(dr, D, p, int(s->lights.size()), rng.get(), rng ? 0 : keys[sidx]);
          Path path = createPath(ray, *s->root, dr, D, rrPdf, rrStart, &r);
          c = integratePath(path, *s->root, s->lights, dr, &sh);
        }
        totRays += r; totShadow += sh; totPaths += 1;
        float inv = 1.f / spp;
        fB += c.b * inv; fG += c.g * inv; fR += c.r * inv;
        accB += c.b; accG += c.g; accR += c.r;
        sqB += double(c.b) * c.b; sqG += double(c.g) * c.g; sqR += double(c.r) * c.r;
        ++sidx;
      }
      size_t o = (size_t(i) * W + j) * 3;
      if (film) { film[o] = fB; film[o + 1] = fG; film[o + 2] = fR; }
      if (sum) { sum[o] = accB; sum[o + 1] = accG; sum[o + 2] = accR; }
      if (sumsq) { sumsq[o] = sqB; sumsq[o + 1] = sqG; sumsq[o + 2] = sqR; }
    }
  }
  if (out_paths) *out_paths = totPaths;
  if (out_rays) *out_rays = totRays;
  if (out_shadow) *out_shadow = totShadow;
  return 0;
}

/* Camera ray of a pixel sample point (px, py) in pixel units, for tests of
 * Camera::getRay (src/camera.cpp:50-58). */
void orc_camera_ray(const gbrt_camera* cam, double px, double py, gbrt_ray* out) {
  Camera camera;
  camera.init(vec3(cam->eye), vec3(cam->look_at), vec3(cam->up), cam->fov, cam->width, cam->height);
  Ray r = camera.getRay(px, py);
  out->org[0] = r.o.x; out->org[1] = r.o.y; out->org[2] = r.o.z; out->tmin = r.from;
  out->dir[0] = r.d.x; out->dir[1] = r.d.y; out->dir[2] = r.d.z; out->tmax = r.to;
}

/* The counter-based stream, exposed for tests. */
float orc_stream_u(uint64_t seed, uint64_t sample_id, uint32_t dim) {
  return streamU(streamKey(seed, sample_id), dim);
}

}  // extern "C"

/* ================================================= Markov-chain renderers ==
 * MetropolisRenderer::render (src/metropolisrenderer.cpp:56-201) and
 * EnergyRedistributionRenderer::render (src/energyredistributionrenderer.cpp:
 * 38-135) with MetropolisSample (src/metropolissample.cpp:33-121), restated
 * with the counter-based stream in place of GSL and float primary-sample
 * coordinates in place of QPointF's doubles. A sample is the vector
 *   0,1 camera point over the image | 2 path length | 3+2i,4+2i direction
 *   sample i | 3+2D+3k,+1 light sample k | 3+2D+3k+2 light choice k
 * (D = max depth). The renderer's lightPathSamples and lightSample2 feed no
 * computation of the unidirectional integrator and are not kept. The chains
 * of the CUDA path run in parallel; here they run one after the other with
 * the same keys, so both produce the same chains. */
namespace chains {

enum : uint64_t { kBoot = 1, kMutate = 2, kPick = 3, kEd = 4, kInit = 5, kFlow = 6 };
inline uint64_t key(uint64_t seed, uint64_t tag, uint64_t id) { return streamKey(seed, (tag << 56) | id); }
inline int dims(int D) { return 3 + 5 * D; }
/* dimensions a small step moves: camera point, direction and light samples */
inline bool moves(int d, int D) {
  if (d == 2) return false;
  if (d >= 3 + 2 * D) return (d - 3 - 2 * D) % 3 != 2;
  return true;
}

/* mutate(qreal&, rng), src/metropolissample.cpp:62-78: a step of
 * b exp(-log(b / a) u) (a = 1/1024, b = 1/64), negative when the second
 * number is below 1/2, wrapped into [0, 1]. -log(16) rounded to float. */
inline float mutateCoord(float s, float ux, float uy) {
  const float b = 1.f / 64.f, logRatio = -2.772588722239781f;
  float delta = b * std::exp(logRatio * ux);
  if (uy < 0.5f) delta = -delta;
  s += delta;
  if (s < 0.f) s += 1.f;
  if (s > 1.f) s -= 1.f;
  return s;
}

/* cv::norm of a Vec3f: square root of the squares summed in double. */
inline double cvNorm(C3 c) {
  double s = double(c.b) * c.b;
  s += double(c.g) * c.g;
  s += double(c.r) * c.r;
  return std::sqrt(s);
}

inline bool finite3(C3 c) { return std::isfinite(c.b) && std::isfinite(c.g) && std::isfinite(c.r); }

struct Tracer {
  Scene* s;
  Camera camera;
  int W, H, D, nL;
  uint64_t paths = 0, rays = 0, shadow = 0, nonfinite = 0;
  /* MetropolisSample::cameraPathFromSample (src/metropolissample.cpp:
   * 120-127) + UniDiPathTracingIntegrator::integrate(path, ...): the path
   * length from dimension 2 when p > 0 (MetropolisSample::mutatePathLength,
   * :32-44), else D with Russian-roulette pdf 1. */
  C3 trace(const float* u, float p) {
    Draws dr;
    dr.pathSamples.resize(D);
    dr.lightSamples.resize(D);
    dr.lightIndex.resize(D);
    if (p > 0) {
      int k = 0;
      if (p < 1) k = int(std::floor(std::log(1.0 - double(u[2])) / std::log(1.0 - double(p))));
      dr.pathLength = std::min(3 + std::max(k, 0), D);
    } else dr.pathLength = D;
    for (int i = 0; i < D; ++i) dr.pathSamples[i] = Sample(u[3 + 2 * i], u[4 + 2 * i]);
    for (int k = 0; k < D; ++k) {
      const float* l = u + 3 + 2 * D + 3 * k;
      dr.lightSamples[k] = Sample(l[0], l[1]);
      int li = nL > 0 ? int(l[2] * float(nL)) : 0;
      dr.lightIndex[k] = std::min(li, std::max(nL - 1, 0));
    }
    float sx = u[0] * float(W), sy = u[1] * float(H);
    Ray ray = camera.getRay(double(sx), double(sy));
    Path path = createPath(ray, *s->root, dr, D, p > 0 ? p : 1.f, 3, &rays);
    C3 c = integratePath(path, *s->root, s->lights, dr, &shadow);
    ++paths;
    if (!finite3(c)) { ++nonfinite; return C3(); }
    return c;
  }
};

/* MetropolisSample::getPos (src/metropolissample.cpp:129-136): the pixel of
 * the camera point, clamped. */
inline int pixelOf(float u, int n) { return std::max(0, std::min(int(double(u) * n), n - 1)); }

}  // namespace chains

extern "C" {

/* MetropolisRenderer::render with `chains` parallel chains (the renderer: one
 * per OpenMP thread). counts: paths traced, mutations, accepted, chains. */
int orc_render_mlt(void* sp, const gbrt_camera* cam, const gbrt_render_params* prm, const gbrt_mlt_params* mp,
                   int64_t chains_n, float* film, double* out_b, uint64_t* counts) {
  using namespace chains;
  Scene* s = static_cast<Scene*>(sp);
  if (!s || !cam || !prm || !mp || chains_n <= 0 || mp->bootstrap <= 0 || mp->mutations <= 0) return 1;
  Tracer tr;
  tr.s = s;
  tr.camera.init(vec3(cam->eye), vec3(cam->look_at), vec3(cam->up), cam->fov, cam->width, cam->height);
  tr.W = cam->width; tr.H = cam->height; tr.D = prm->max_depth; tr.nL = int(s->lights.size());
  const int D = tr.D, nd = dims(D), W = tr.W, H = tr.H;
  const uint64_t seed = prm->seed;
  /* Bootstrap (lines 77-100): large steps traced at full length
   * (MetropolisSample starts with pathLength MAX_DEPTH, terminationProb 1). */
  const int nb = mp->bootstrap;
  std::vector<float> bootI(nb), u(nd);
  std::vector<C3> bootL(nb);
  float sumI = 0;
  for (int i = 0; i < nb; ++i) {
    uint64_t k = key(seed, kBoot, uint64_t(i));
    for (int d = 0; d < nd; ++d) u[d] = streamU(k, d);
    bootL[i] = tr.trace(u.data(), 0.f);
    bootI[i] = lum(bootL[i]);
    sumI += bootI[i];
  }
  const float b = sumI / nb;
  /* Initial samples (lines 102-113) by systematic resampling: chain c takes
   * the first bootstrap sample whose running sum exceeds (u + c) / chains of
   * the total; with one chain this is the renderer's choice. */
  std::vector<float> cum(nb);
  float run = 0;
  for (int i = 0; i < nb; ++i) { run += bootI[i]; cum[i] = run; }
  const double u0 = streamU(key(seed, kPick, 0), 0);
  const int64_t N = chains_n;
  const int64_t total = int64_t(mp->mutations) * W * H;
  const int64_t M = std::max<int64_t>(1, total / N);
  std::vector<double> acc(size_t(W) * H * 3, 0.0);
  auto deposit = [&](const float* su, float weight, C3 v) {
    int x = pixelOf(su[0], W), y = pixelOf(su[1], H);
    C3 dv = weight * v;
    size_t o = (size_t(y) * W + x) * 3;
    acc[o] += dv.b; acc[o + 1] += dv.g; acc[o + 2] += dv.r;
  };
  uint64_t accepted = 0;
  std::vector<float> cur(nd), prop(nd);
  for (int64_t c = 0; c < N; ++c) {
    float off = float((u0 + double(c)) / double(N) * double(sumI));
    int bi = int(std::upper_bound(cum.begin(), cum.end(), off) - cum.begin());
    if (bi >= nb) bi = nb - 1;
    uint64_t kb = key(seed, kBoot, uint64_t(bi));
    for (int d = 0; d < nd; ++d) cur[d] = streamU(kb, d);
    C3 curV = bootL[bi];
    /* the chain (lines 131-190) */
    for (int64_t t = 0; t < M; ++t) {
      uint64_t k = key(seed, kMutate, uint64_t(t) * uint64_t(N) + uint64_t(c));
      const bool large = streamU(k, 0) < mp->large_step_prob;
      for (int d = 0; d < nd; ++d) {
        if (d == 2) prop[d] = streamU(k, 2);
        else if (large) prop[d] = streamU(k, 3 + 2 * d);
        else prop[d] = moves(d, D) ? mutateCoord(cur[d], streamU(k, 3 + 2 * d), streamU(k, 4 + 2 * d)) : cur[d];
      }
      C3 newV = tr.trace(prop.data(), mp->termination_prob);
      const float lc = lum(curV), ln = lum(newV);
      float ratio = ln / lc;
      float a = ratio < 1.f ? ratio : 1.f;  /* std::min<float>(1, ratio): NaN gives 1 */
      if (lc > 0) deposit(cur.data(), 1 - a, curV * (1.f / lc * b / float(mp->mutations)));
      if (ln > 0) deposit(prop.data(), a, newV * (1.f / ln * b / float(mp->mutations)));
      if (streamU(k, 1) < a) { cur.swap(prop); curV = newV; ++accepted; }
    }
  }
  for (size_t i = 0; i < acc.size(); ++i) film[i] = float(acc[i]);
  if (out_b) *out_b = b;
  if (counts) { counts[0] = tr.paths; counts[1] = uint64_t(N * M); counts[2] = accepted; counts[3] = uint64_t(N); }
  return 0;
}

/* EnergyRedistributionRenderer::render. counts: paths traced, mutations,
 * accepted, chains. */
int orc_render_erpt(void* sp, const gbrt_camera* cam, const gbrt_render_params* prm, const gbrt_erpt_params* ep,
                    float* film, double* out_ed, uint64_t* counts) {
  using namespace chains;
  Scene* s = static_cast<Scene*>(sp);
  if (!s || !cam || !prm || !ep || ep->mutations <= 0 || ep->x_samples <= 0 || ep->y_samples <= 0) return 1;
  Tracer tr;
  tr.s = s;
  tr.camera.init(vec3(cam->eye), vec3(cam->look_at), vec3(cam->up), cam->fov, cam->width, cam->height);
  tr.W = cam->width; tr.H = cam->height; tr.D = prm->max_depth; tr.nL = int(s->lights.size());
  const int D = tr.D, nd = dims(D), W = tr.W, H = tr.H, M = ep->mutations;
  const int xs = ep->x_samples, ys = ep->y_samples, spp = xs * ys;
  const uint64_t seed = prm->seed;
  /* computeEd (lines 120-135): one path through each pixel corner with the
   * integrator's termination probability 0.1, summed (here in double). */
  double Sb = 0, Sg = 0, Sr = 0;
  Draws dr;
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j) {
      uint64_t k = key(seed, kEd, uint64_t(i) * W + j);
      Ray ray = tr.camera.getRay(double(j), double(i));
      drawPath(dr, D, 0.1f, tr.nL, nullptr, k);
      Path path = createPath(ray, *s->root, dr, D, 0.1f, 3, &tr.rays);
      C3 c = integratePath(path, *s->root, s->lights, dr, &tr.shadow);
      ++tr.paths;
      if (!finite3(c)) { ++tr.nonfinite; continue; }
      Sb += c.b; Sg += c.g; Sr += c.r;
    }
  const float ed = float(cvNorm(C3(float(Sb), float(Sg), float(Sr))) / double(H * W * M));
  std::vector<double> acc(size_t(W) * H * 3, 0.0);
  std::vector<float> u(nd), y(nd), z(nd);
  uint64_t chainId = 0, accepted = 0, mutations = 0;
  for (int i = 0; i < H; ++i)
    for (int j = 0; j < W; ++j)
      for (int a = 0; a < xs; ++a)
        for (int bb = 0; bb < ys; ++bb) {
          /* JitteredSampler(xs, ys) point and MetropolisSample::initAtPixel */
          const uint64_t g = (uint64_t(i) * W + j) * spp + uint64_t(a * ys + bb);
          const uint64_t k = key(seed, kInit, g);
          const double jx = (double(streamU(k, 0)) + a) / xs, jy = (double(streamU(k, 1)) + bb) / ys;
          u[0] = float((j + jx) / W);
          u[1] = float((i + jy) / H);
          for (int d = 2; d < nd; ++d) u[d] = streamU(k, d);
          const C3 c = tr.trace(u.data(), 0.f);
          /* equalDispositionFlow (lines 83-118) */
          const double nc = cvNorm(c);
          const float me = float(M) * ed;
          const double xc = double(streamU(k, nd)) + nc / double(me);
          const int numChains = xc > 0.0 ? int(xc) : 0;  /* a black scene gives 0 / 0 */
          if (numChains <= 0) continue;
          const double sc = double(ed) / nc / numChains;
          const C3 depVal(float(c.b * sc), float(c.g * sc), float(c.r * sc));
          const double depNorm = cvNorm(depVal);
          for (int r = 0; r < numChains; ++r, ++chainId) {
            y = u;
            C3 yV = c;
            for (int m = 0; m < M; ++m) {
              const uint64_t kk = key(seed, kFlow, chainId * uint64_t(M) + uint64_t(m));
              for (int d = 0; d < nd; ++d)
                z[d] = moves(d, D) ? mutateCoord(y[d], streamU(kk, 3 + 2 * d), streamU(kk, 4 + 2 * d)) : y[d];
              const C3 zV = tr.trace(z.data(), 0.f);
              ++mutations;
              const float yLum = float(cvNorm(yV)), zLum = float(cvNorm(zV));
              const float ratio = zLum / yLum;
              const float q = ratio < 1.f ? ratio : 1.f;
              const C3 yOld = yV;
              if (q > streamU(kk, 1)) { y.swap(z); yV = zV; ++accepted; }
              const int px = pixelOf(y[0], W), py = pixelOf(y[1], H);
              const double in = 1.0 / cvNorm(yOld);
              const float isp = 1.f / float(spp);
              C3 t(float(depNorm * yOld.b), float(depNorm * yOld.g), float(depNorm * yOld.r));
              t = C3(float(t.b * in), float(t.g * in), float(t.r * in));
              t = t * isp;
              size_t o = (size_t(py) * W + px) * 3;
              acc[o] += t.b; acc[o + 1] += t.g; acc[o + 2] += t.r;
            }
          }
        }
  for (size_t i = 0; i < acc.size(); ++i) film[i] = float(acc[i]);
  if (out_ed) *out_ed = ed;
  if (counts) { counts[0] = tr.paths; counts[1] = mutations; counts[2] = accepted; counts[3] = chainId; }
  return 0;
}

}  // extern "C"

/* Tonemapper::map, src/tonemapper.cpp:31-56: RGB bytes of a BGR film. */
extern "C" void orc_tonemap(const float* film, int w, int h, float gamma, unsigned char* rgb) {
  double ig = 1. / gamma;
  auto ch = [&](float c) -> unsigned char {
    float x = float(255 * std::pow(double(c), ig));
    if (!(x > 0)) return 0;
    if (x >= 255) return 255;
    return (unsigned char)int(x);
  };
  for (size_t i = 0; i < size_t(w) * h; ++i) {
    rgb[3 * i] = ch(film[3 * i + 2]);
    rgb[3 * i + 1] = ch(film[3 * i + 1]);
    rgb[3 * i + 2] = ch(film[3 * i]);
  }
}
