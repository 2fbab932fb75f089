/*
 * oracle_math.h — TEST INFRASTRUCTURE ONLY (the CPU oracle). Nothing in the
 * product imports this file.
 *
 * Small float vector/matrix types that restate, operation for operation, the
 * Qt arithmetic the renderer relies on (QVector3D / QVector4D / QMatrix4x4):
 *   - dot and cross products and lengthSquared in float, left to right;
 *   - length and normalized computed through double, with normalized() leaving
 *     a vector whose double squared length is within 1e-12 of 1 unchanged and
 *     mapping one whose squared length is within 1e-12 of 0 to the zero vector
 *     (Qt 5 semantics for QVector3D::normalized);
 *   - toVector3DAffine returning the zero vector when w is exactly zero;
 *   - column-major 4x4 matrices, map() of points (w = 1, then divided by w when
 *     w != 1) and of 4-vectors.
 * The oracle is compiled with -ffp-contract=off so that no multiply-add is
 * fused on any host: results are bit-identical on x86-64 and aarch64.
 */
#ifndef ORACLE_MATH_H
#define ORACLE_MATH_H

#include <cmath>
#include <cstdint>
#include <limits>

namespace orc {

static const float kInf = std::numeric_limits<float>::infinity();
static const float kNaN = std::numeric_limits<float>::quiet_NaN();
static const float kEpsilon = 0.001f; /* EPSILON, src/ray.h:34 */

struct V3 {
  float x = 0, y = 0, z = 0;
  V3() = default;
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  void set(int i, float v) { (i == 0 ? x : (i == 1 ? y : z)) = v; }
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
  bool isNull() const { return x == 0.f && y == 0.f && z == 0.f; }
  float lengthSquared() const { return x * x + y * y + z * z; }
  float length() const {
    double l = double(x) * double(x) + double(y) * double(y) + double(z) * double(z);
    return float(std::sqrt(l));
  }
  V3 normalized() const {
    double l = double(x) * double(x) + double(y) * double(y) + double(z) * double(z);
    if (std::fabs(l - 1.0) <= 1e-12) return *this;
    if (std::fabs(l) > 1e-12) {
      double s = std::sqrt(l);
      return V3(float(double(x) / s), float(double(y) / s), float(double(z) / s));
    }
    return V3();
  }
  void normalize() { *this = normalized(); }
};

inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
inline bool operator==(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return V3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* QVector3D::normal(a, b) = normalized cross product. */
inline V3 normalOf(V3 a, V3 b) { return cross(a, b).normalized(); }

struct V4 {
  float x = 0, y = 0, z = 0, w = 0;
  V4() = default;
  V4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
  V4(V3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
  V3 xyz() const { return V3(x, y, z); }
  /* QVector4D::toVector3DAffine: zero vector when w is zero. */
  V3 affine() const {
    if (w == 0.f) return V3();
    return V3(x / w, y / w, z / w);
  }
};
inline float dot4(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }

/* Spectrum in BGR order (cv::Vec3f in the renderer). */
struct C3 {
  float b = 0, g = 0, r = 0;
  C3() = default;
  C3(float x, float y, float z) : b(x), g(y), r(z) {}
  float operator[](int i) const { return i == 0 ? b : (i == 1 ? g : r); }
  bool isZero() const { return b == 0.f && g == 0.f && r == 0.f; }
};
inline C3 operator+(C3 a, C3 c) { return C3(a.b + c.b, a.g + c.g, a.r + c.r); }
inline C3 operator*(C3 a, float s) { return C3(a.b * s, a.g * s, a.r * s); }
inline C3 operator*(float s, C3 a) { return C3(s * a.b, s * a.g, s * a.r); }
inline C3 mul(C3 a, C3 c) { return C3(a.b * c.b, a.g * c.g, a.r * c.r); }
inline bool operator!=(C3 a, C3 c) { return !(a.b == c.b && a.g == c.g && a.r == c.r); }
/* lum(), src/mathhelper.cpp:102-105: index 2 is red. */
inline float lum(C3 c) { return float(.299 * c.r + .587 * c.g + .114 * c.b); }

/* signum for signed types, src/mathhelper.h:44-47. */
inline int signum(float x) { return (0.f < x) - (x < 0.f); }

/* reflect(v, n) = v - 2 dot(v,n) n, src/vechelper.cpp:3-6. */
inline V3 reflect(V3 v, V3 n) { return v - 2 * dot(v, n) * n; }

/* 4x4 float matrix, column-major storage m[col][row] like QMatrix4x4. */
struct M4 {
  float m[4][4];
  M4() { setIdentity(); }
  void setIdentity() {
    for (int c = 0; c < 4; ++c)
      for (int r = 0; r < 4; ++r) m[c][r] = (c == r) ? 1.f : 0.f;
  }
  void setColumn(int c, V4 v) { m[c][0] = v.x; m[c][1] = v.y; m[c][2] = v.z; m[c][3] = v.w; }
  void setRow(int r, V4 v) { m[0][r] = v.x; m[1][r] = v.y; m[2][r] = v.z; m[3][r] = v.w; }
  V4 map4(V4 v) const {
    return V4(v.x * m[0][0] + v.y * m[1][0] + v.z * m[2][0] + v.w * m[3][0],
              v.x * m[0][1] + v.y * m[1][1] + v.z * m[2][1] + v.w * m[3][1],
              v.x * m[0][2] + v.y * m[1][2] + v.z * m[2][2] + v.w * m[3][2],
              v.x * m[0][3] + v.y * m[1][3] + v.z * m[2][3] + v.w * m[3][3]);
  }
  /* map of a point: w = 1, divided by w when w != 1. */
  V3 mapPoint(V3 p) const {
    V4 r = map4(V4(p, 1.f));
    if (r.w == 1.f || r.w == 0.f) return r.xyz();
    return V3(r.x / r.w, r.y / r.w, r.z / r.w);
  }
  M4 operator*(const M4& o) const {
    M4 r;
    for (int c = 0; c < 4; ++c)
      for (int rr = 0; rr < 4; ++rr) {
        float s = 0;
        for (int k = 0; k < 4; ++k) s += m[k][rr] * o.m[c][k];
        r.m[c][rr] = s;
      }
    return r;
  }
};

/* General 4x4 inverse by cofactors (double), returned in float. */
M4 inverted(const M4& a);
/* Normal matrix: inverse transpose of the upper-left 3x3, as a 4x4 with the
 * last row/column of the identity. */
M4 normalMatrix(const M4& a);

}  // namespace orc

#endif
