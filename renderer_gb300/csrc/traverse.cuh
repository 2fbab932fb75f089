// traverse.cuh — closest-hit and any-hit BVH traversal for sm_103a.
//
// Replaces the renderer's per-ray virtual intersect chain:
//   BVHNode::intersect                 src/bvh.cpp:135-149
//   AxisAlignedBox::getCSGIntersection src/axisalignedbox.cpp:30-73
//   Triangle::intersect                src/triangle.cpp:30-56
//   Quad::intersect                    src/quad.cpp:23-34 (as two triangles)
//   Sphere + CSGObject::intersect      src/sphere.cpp:29-56, src/csgobject.cpp:25-44
//   Plane::intersect                   src/plane.cpp:27-40
//   AreaLight::intersect               src/arealight.cpp:73-90
//   EnvironmentMap::intersect          src/environmentmap.cpp:73-83 (as "no hit, tmax = inf")
//
// Structure: ordered (nearest child first) traversal of a 4-wide BVH with tmax
// shrinking. A node is 128 bytes; a ray fetches the six box planes it needs in
// near/far order (chosen once per ray by the signs of its direction) and the
// child references as seven 128-bit non-coherent loads, tests the four child
// boxes, sorts the hit children by entry distance with a 4-key sorting
// network, descends into the nearest and pushes the others far-to-near on a
// per-thread stack (local memory, L1-resident). A 4-wide tree halves the chain
// of dependent node fetches of a binary one, which is what bounds traversal:
// the nodes of a 1.3M-triangle scene sit in L1/L2, so the kernel is
// latency-bound rather than DRAM-bound.
//
// Numerics. By default a triangle is tested with the renderer's own formulas
// (src/triangle.cpp:32-44: Cramer's rule, t first, then u in [0,1], v >= 0,
// u + v <= 1) evaluated in the renderer's operation order with every product,
// sum and quotient rounded separately (no fused multiply-adds), so the hit
// decision and t are bit-identical to the renderer's float arithmetic for the
// same ray. That test is not watertight: its barycentrics carry a rounding
// error of about eps * |origin - vertex| / |edge|, so near a shared edge a ray
// can miss both triangles or hit both. With GBRT_SCENE_WATERTIGHT the inside
// decision instead uses the watertight test of Woop, Benthin and Wald (JCGT
// 2013): vertices are translated to the ray origin and sheared so the ray runs
// along +z, and the three 2D edge functions are evaluated without fused
// multiply-adds (the two triangles sharing an edge then evaluate it as exact
// negations of each other), with a double-precision re-evaluation when one is
// exactly zero; t still comes from the renderer's formula. Spheres, planes and
// parallelograms always use the renderer's formulas the same way. Box tests
// are conservative (box_entry; Ize 2013, "Robust BVH Ray Traversal").
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>

#include "gbrt_scene.h"

namespace gbrt {

// Stack entries: at most three pushes per level of the 4-wide tree, whose
// depth is at most the binary tree's (<= 62, kept by the builder).
constexpr int kStackSize = 190;  // any tree
constexpr int kShortStack = 64;  // trees of 4-wide depth <= 21
constexpr int kFaultStack = 4;   // injected fault (GBRT_FAULT_SMALL_STACK): overflows on most trees
__host__ __device__ constexpr int stack_need(int depth4) { return 3 * depth4 + 1; }
constexpr int kTraceBlock = 128;

// Exactly rounded, never-contracted float operations.
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fdv(float a, float b) { return __fdiv_rn(a, b); }
// (a*b) - (c*d) with both products rounded, like the renderer's cross product.
__device__ __forceinline__ float dmd(float a, float b, float c, float d) { return fs(fm(a, b), fm(c, d)); }
// x1*x2 + y1*y2 + z1*z2 evaluated left to right (QVector3D::dotProduct).
__device__ __forceinline__ float dot3x(float ax, float ay, float az, float bx, float by, float bz) {
  return fa(fa(fm(ax, bx), fm(ay, by)), fm(az, bz));
}

struct TRay {
  float ox, oy, oz, tmin;
  float dx, dy, dz, tmax;
  float ix, iy, iz;        // 1 / d
  float sx0, sx1, sx2;     // shear row for the 2D x coordinate
  float sy0, sy1, sy2;     // shear row for the 2D y coordinate
};

__device__ __forceinline__ TRay make_tray(float4 a, float4 b) {
  TRay r;
  r.ox = a.x; r.oy = a.y; r.oz = a.z; r.tmin = a.w;
  r.dx = b.x; r.dy = b.y; r.dz = b.z; r.tmax = b.w;
  r.ix = 1.0f / r.dx; r.iy = 1.0f / r.dy; r.iz = 1.0f / r.dz;
  // Watertight shear: kz = dominant axis, (kx, ky) the two others in cyclic
  // order. A vertex A (relative to the origin) maps to
  //   (A[kx] - Sx A[kz], A[ky] - Sy A[kz]),  Sx = d[kx]/d[kz], Sy = d[ky]/d[kz].
  // Both signs of the edge functions are accepted (two-sided), so the
  // winding-preserving swap of kx and ky is not needed.
  float ax = fabsf(r.dx), ay = fabsf(r.dy), az = fabsf(r.dz);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  float dkz = kz == 0 ? r.dx : (kz == 1 ? r.dy : r.dz);
  float sx0 = 0, sx1 = 0, sx2 = 0, sy0 = 0, sy1 = 0, sy2 = 0;
  if (kz == 0) {        // kx = 1, ky = 2
    sx1 = 1.f; sx0 = -r.dy / dkz;
    sy2 = 1.f; sy0 = -r.dz / dkz;
  } else if (kz == 1) { // kx = 2, ky = 0
    sx2 = 1.f; sx1 = -r.dz / dkz;
    sy0 = 1.f; sy1 = -r.dx / dkz;
  } else {              // kx = 0, ky = 1
    sx0 = 1.f; sx2 = -r.dx / dkz;
    sy1 = 1.f; sy2 = -r.dy / dkz;
  }
  r.sx0 = sx0; r.sx1 = sx1; r.sx2 = sx2;
  r.sy0 = sy0; r.sy1 = sy1; r.sy2 = sy2;
  return r;
}

// Entry distance of one child box, or +inf when the ray misses it inside
// [tmin, tcur]. n* / f* are the box's near and far planes for this ray (picked
// by the signs of 1/d, as AxisAlignedBox::getCSGIntersection does,
// src/axisalignedbox.cpp:41-66). A plane distance that is NaN (a zero
// direction component with the origin on that plane: 0 * inf) constrains
// nothing, because fmaxf / fminf ignore NaN. Each distance (p - o) * (1/d) has
// a relative error below 2^-23, so enlarging the far distance by
// 1 + 6.7 * 2^-24 (Ize 2013, "Robust BVH Ray Traversal") never loses a box.
__device__ __forceinline__ float box_entry(const TRay& r, float nx, float fx, float ny, float fy, float nz, float fz,
                                           float tcur) {
  float tn = fmaxf(fmaxf((nx - r.ox) * r.ix, (ny - r.oy) * r.iy), fmaxf((nz - r.oz) * r.iz, r.tmin));
  float tf = fminf(fminf((fx - r.ox) * r.ix, (fy - r.oy) * r.iy), (fz - r.oz) * r.iz);
  tf = fminf(tf * 1.0000004f, tcur);
  return tn <= tf ? tn : CUDART_INF_F;
}

__device__ __forceinline__ void cswap(float& ka, int& ra, float& kb, int& rb) {
  bool sw = kb < ka;
  float k = sw ? kb : ka;
  int rr = sw ? rb : ra;
  kb = sw ? ka : kb;
  rb = sw ? ra : rb;
  ka = k;
  ra = rr;
}

// Accepts t against the current best: inclusive of tmax for the first hit
// (the renderer's Ray::inRange), strictly closer afterwards.
__device__ __forceinline__ bool accept_t(float t, float tmin, float tcur, bool found) {
  return t >= tmin && (found ? t < tcur : t <= tcur);
}

// Triangle p1 p2 p3, the renderer's test (src/triangle.cpp:30-56). Returns
// true and t/u/v when the ray hits it inside [tmin, tlim].
__device__ __forceinline__ bool tri_test_ref(const TRay& r, float4 v0, float4 v1, float4 v2, float tlim,
                                             float& t_out, float& u_out, float& v_out) {
  float e1x = fs(v1.x, v0.x), e1y = fs(v1.y, v0.y), e1z = fs(v1.z, v0.z);
  float e2x = fs(v2.x, v0.x), e2y = fs(v2.y, v0.y), e2z = fs(v2.z, v0.z);
  float nx = dmd(e1y, e2z, e1z, e2y);
  float ny = dmd(e1z, e2x, e1x, e2z);
  float nz = dmd(e1x, e2y, e1y, e2x);
  float w = -dot3x(nx, ny, nz, r.dx, r.dy, r.dz);
  if (w == 0.f) return false;
  float adx = fs(r.ox, v0.x), ady = fs(r.oy, v0.y), adz = fs(r.oz, v0.z);
  float t = fdv(dot3x(nx, ny, nz, adx, ady, adz), w);
  if (!(t >= r.tmin && t <= tlim)) return false;
  float qx = dmd(ady, r.dz, adz, r.dy);
  float qy = dmd(adz, r.dx, adx, r.dz);
  float qz = dmd(adx, r.dy, ady, r.dx);
  float u = fdv(dot3x(qx, qy, qz, e2x, e2y, e2z), w);
  if (u < 0.f || u > 1.f) return false;
  float v = fdv(-dot3x(qx, qy, qz, e1x, e1y, e1z), w);
  if (v < 0.f || fa(u, v) > 1.f) return false;
  t_out = t; u_out = u; v_out = v;
  return true;
}

// Triangle p1 p2 p3 with the watertight inside test; t and the barycentrics by
// the renderer's formulas. Returns true when the ray hits it inside [tmin, tlim].
__device__ __forceinline__ bool tri_test_wt(const TRay& r, float4 v0, float4 v1, float4 v2, float tlim,
                                            float& t_out, float& u_out, float& v_out) {
  // Watertight inside test.
  float Ax = v0.x - r.ox, Ay = v0.y - r.oy, Az = v0.z - r.oz;
  float Bx = v1.x - r.ox, By = v1.y - r.oy, Bz = v1.z - r.oz;
  float Cx = v2.x - r.ox, Cy = v2.y - r.oy, Cz = v2.z - r.oz;
  float ax = fmaf(r.sx2, Az, fmaf(r.sx1, Ay, r.sx0 * Ax));
  float ay = fmaf(r.sy2, Az, fmaf(r.sy1, Ay, r.sy0 * Ax));
  float bx = fmaf(r.sx2, Bz, fmaf(r.sx1, By, r.sx0 * Bx));
  float by = fmaf(r.sy2, Bz, fmaf(r.sy1, By, r.sy0 * Bx));
  float cx = fmaf(r.sx2, Cz, fmaf(r.sx1, Cy, r.sx0 * Cx));
  float cy = fmaf(r.sy2, Cz, fmaf(r.sy1, Cy, r.sy0 * Cx));
  float U = dmd(cx, by, cy, bx);
  float V = dmd(ax, cy, ay, cx);
  float W = dmd(bx, ay, by, ax);
  if (U == 0.f || V == 0.f || W == 0.f) {
    U = float(double(cx) * double(by) - double(cy) * double(bx));
    V = float(double(ax) * double(cy) - double(ay) * double(cx));
    W = float(double(bx) * double(ay) - double(by) * double(ax));
  }
  if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
  if (U + V + W == 0.f) return false;
  // t by the renderer's formula (src/triangle.cpp:32-37).
  float e1x = fs(v1.x, v0.x), e1y = fs(v1.y, v0.y), e1z = fs(v1.z, v0.z);
  float e2x = fs(v2.x, v0.x), e2y = fs(v2.y, v0.y), e2z = fs(v2.z, v0.z);
  float nx = dmd(e1y, e2z, e1z, e2y);
  float ny = dmd(e1z, e2x, e1x, e2z);
  float nz = dmd(e1x, e2y, e1y, e2x);
  float w = -dot3x(nx, ny, nz, r.dx, r.dy, r.dz);
  if (w == 0.f) return false;
  float adx = fs(r.ox, v0.x), ady = fs(r.oy, v0.y), adz = fs(r.oz, v0.z);
  float t = fdv(dot3x(nx, ny, nz, adx, ady, adz), w);
  if (!(t >= r.tmin && t <= tlim)) return false;
  // Barycentrics by the renderer's formula (src/triangle.cpp:40-43).
  float qx = dmd(ady, r.dz, adz, r.dy);
  float qy = dmd(adz, r.dx, adx, r.dz);
  float qz = dmd(adx, r.dy, ady, r.dx);
  u_out = fdv(dot3x(qx, qy, qz, e2x, e2y, e2z), w);
  v_out = fdv(-dot3x(qx, qy, qz, e1x, e1y, e1z), w);
  t_out = t;
  return true;
}

// Parallelogram origin + a u + b v, a, b in [0, 1] (AreaLight::intersect).
__device__ __forceinline__ bool pgram_test(const TRay& r, float4 o, float4 eu, float4 ev, float tlim,
                                           float& t_out, float& u_out, float& v_out) {
  float nx = dmd(eu.y, ev.z, eu.z, ev.y);
  float ny = dmd(eu.z, ev.x, eu.x, ev.z);
  float nz = dmd(eu.x, ev.y, eu.y, ev.x);
  float w = -dot3x(nx, ny, nz, r.dx, r.dy, r.dz);
  if (w == 0.f) return false;
  float adx = fs(r.ox, o.x), ady = fs(r.oy, o.y), adz = fs(r.oz, o.z);
  float t = fdv(dot3x(nx, ny, nz, adx, ady, adz), w);
  if (!(t >= r.tmin && t <= r.tmax)) return false;
  float qx = dmd(ady, r.dz, adz, r.dy);
  float qy = dmd(adz, r.dx, adx, r.dz);
  float qz = dmd(adx, r.dy, ady, r.dx);
  float u = fdv(dot3x(qx, qy, qz, ev.x, ev.y, ev.z), w);
  if (u < 0.f || u > 1.f) return false;
  float v = fdv(-dot3x(qx, qy, qz, eu.x, eu.y, eu.z), w);
  if (v < 0.f || v > 1.f) return false;
  if (!(t <= tlim)) return false;
  t_out = t; u_out = u; v_out = v;
  return true;
}

// Sphere, first intersection parameter at or beyond tmin (CSGObject rule).
__device__ __forceinline__ bool sphere_test(const TRay& r, float4 c, float rad, float tlim, float& t_out) {
  float dfx = fs(r.ox, c.x), dfy = fs(r.oy, c.y), dfz = fs(r.oz, c.z);
  float r2 = fm(rad, rad);
  float a = dot3x(r.dx, r.dy, r.dz, r.dx, r.dy, r.dz);
  float b = fm(2.f, dot3x(r.dx, r.dy, r.dz, dfx, dfy, dfz));
  float cc = fs(dot3x(dfx, dfy, dfz, dfx, dfy, dfz), r2);
  float disc = fs(fm(b, b), fm(fm(4.f, a), cc));
  if (!(disc >= 0.f)) return false;
  float rd = __fsqrt_rn(disc);
  float a2 = fm(2.f, a);
  float t1 = fdv(fs(-b, rd), a2);
  float t2 = fdv(fa(-b, rd), a2);
  if (r.tmin > t2) return false;
  float t = (t1 >= r.tmin) ? t1 : t2;
  if (!(t >= r.tmin)) return false;  // NaN guard
  if (t > r.tmax) return false;
  if (!(t <= tlim)) return false;
  t_out = t;
  return true;
}

// ------------------------------------------------------------------ CSG --
// CSGObject::intersect over the interval lists of CSGOperation::
// getCSGIntersection (src/csgobject.cpp:25-44, src/csgoperation.cpp:27-64):
// the object's postfix program evaluates leaf lists (a sphere's two roots,
// src/sphere.cpp:29-56; a box's slab entry and exit, src/axisalignedbox.cpp:
// 30-73) and merges them in t order, keeping a boundary where the
// operation's inside state changes. At most GBRT_CSG_MAX_LEAVES leaves, so
// lists hold at most twice as many boundaries. Not inlined: its lists live
// in local memory only while a CSG record is tested.
struct CsgParam {
  float t;
  int leaf;  // node index of the leaf that produced the boundary
};
constexpr int kCsgList = 2 * GBRT_CSG_MAX_LEAVES;

__device__ __forceinline__ bool csg_inside(int op, bool l, bool r) {
  return op == GBRT_CSG_ISECT ? (l && r) : op == GBRT_CSG_UNION ? (l || r) : op == GBRT_CSG_DIFF ? (l && !r) : (l != r);
}

static __device__ __noinline__ bool csg_test(const DeviceScene& S, const TRay& r, int start, int len, float tlim,
                                      float& t_out, int& leaf_out) {
  CsgParam lists[GBRT_CSG_MAX_LEAVES][kCsgList];
  int cnt[GBRT_CSG_MAX_LEAVES];
  int sp = 0;
  for (int i = 0; i < len; ++i) {
    const int nidx = __ldg(S.csg_prog + start + i);
    const float4 A = __ldg(S.csg_nodes + 3 * nidx), B = __ldg(S.csg_nodes + 3 * nidx + 1);
    const int op = __float_as_int(A.w);
    if (op == GBRT_CSG_SPHERE || op == GBRT_CSG_BOX) {
      if (sp >= GBRT_CSG_MAX_LEAVES) return false;
      CsgParam* out = lists[sp];
      int n = 0;
      if (op == GBRT_CSG_SPHERE) {
        float dfx = fs(r.ox, A.x), dfy = fs(r.oy, A.y), dfz = fs(r.oz, A.z);
        float a = dot3x(r.dx, r.dy, r.dz, r.dx, r.dy, r.dz);
        float b = fm(2.f, dot3x(r.dx, r.dy, r.dz, dfx, dfy, dfz));
        float c = fs(dot3x(dfx, dfy, dfz, dfx, dfy, dfz), fm(B.x, B.x));
        float disc = fs(fm(b, b), fm(fm(4.f, a), c));
        if (disc >= 0.f) {
          float rd = __fsqrt_rn(disc), a2 = fm(2.f, a);
          out[0] = CsgParam{fdv(fs(-b, rd), a2), nidx};
          out[1] = CsgParam{fdv(fa(-b, rd), a2), nidx};
          n = 2;
        }
      } else {
        const float o[3] = {r.ox, r.oy, r.oz}, d[3] = {r.dx, r.dy, r.dz};
        const float lo[3] = {A.x, A.y, A.z}, hi[3] = {B.x, B.y, B.z};
        float tmin = -CUDART_INF_F, tmax = CUDART_INF_F;
        bool empty = false;
        for (int k = 0; k < 3 && !empty; ++k) {
          float inv = fdv(1.f, d[k]);
          float tn = inv >= 0.f ? fs(lo[k], o[k]) : fs(hi[k], o[k]);
          float tx = inv >= 0.f ? fs(hi[k], o[k]) : fs(lo[k], o[k]);
          tn = fm(tn, inv);
          tx = fm(tx, inv);
          if (tn > tmin) tmin = tn;
          if (tx < tmax) tmax = tx;
          if (tmin > tmax) empty = true;
        }
        if (!empty) {
          out[0] = CsgParam{tmin, nidx};
          out[1] = CsgParam{tmax, nidx};
          n = 2;
        }
      }
      cnt[sp++] = n;
    } else {
      if (sp < 2) return false;
      const CsgParam* L = lists[sp - 2];
      const CsgParam* R = lists[sp - 1];
      const int nl = cnt[sp - 2], nr = cnt[sp - 1];
      CsgParam tmp[kCsgList];
      int n = 0, i0 = 0, j0 = 0;
      bool li = false, ri = false;
      while (i0 < nl || j0 < nr) {
        const bool was = csg_inside(op, li, ri);
        const bool takeL = i0 < nl && (j0 >= nr || L[i0].t <= R[j0].t);
        const CsgParam p = takeL ? L[i0++] : R[j0++];
        if (takeL) li = !li; else ri = !ri;
        if (was != csg_inside(op, li, ri) && n < kCsgList) tmp[n++] = p;
      }
      for (int k = 0; k < n; ++k) lists[sp - 2][k] = tmp[k];
      cnt[sp - 2] = n;
      --sp;
    }
  }
  if (sp != 1) return false;
  const CsgParam* P = lists[0];
  const int n = cnt[0];
  if (n == 0 || r.tmin > P[n - 1].t) return false;
  for (int k = 0; k < n; ++k) {
    if (P[k].t >= r.tmin) {
      if (P[k].t > r.tmax || !(P[k].t <= tlim)) return false;
      t_out = P[k].t;
      leaf_out = P[k].leaf;
      return true;
    }
  }
  return false;
}

// Plane (src/plane.cpp:29-31): t = dot((o,1), P) / -dot(d, P.xyz).
__device__ __forceinline__ float plane_t(const TRay& r, float4 P) {
  float d = -dot3x(r.dx, r.dy, r.dz, P.x, P.y, P.z);
  float u = fa(dot3x(r.ox, r.oy, r.oz, P.x, P.y, P.z), P.w);
  return fdv(u, d);
}

struct TraceCounters {
  unsigned long long nodes, prims;
};

// Traversal state of one ray between steps (see trace_step).
struct TState {
  int32_t node;      // next node or leaf to visit
  int sp;            // stack depth
  float tcur;        // current far limit
  int32_t best;      // internal hit encoding of the best hit so far
  int32_t bestPrim;
  int32_t bestQuad;  // 0: not a quad half, 1: first half, 2: second half
  float bu, bv;
  bool found;
  // Two-level scenes (GEN traversal only): the instance whose mesh is being
  // traversed (-1: world space), the instance of the best hit, and the ray in
  // that instance's space.
  int32_t inst, bestInst;
  TRay oray;
};

// IntersectableInstance::intersect's Ray::transform(inverseTransform)
// (src/intersectableinstance.cpp:24-30): the origin mapped as a point, the
// direction as a vector (not renormalised), each row summed left to right.
__device__ __forceinline__ TRay instance_ray(const TRay& r, float4 m0, float4 m1, float4 m2) {
  auto pt = [&](float4 m) { return fa(fa(fa(fm(m.x, r.ox), fm(m.y, r.oy)), fm(m.z, r.oz)), m.w); };
  auto vec = [&](float4 m) { return fa(fa(fm(m.x, r.dx), fm(m.y, r.dy)), fm(m.z, r.dz)); };
  return make_tray(make_float4(pt(m0), pt(m1), pt(m2), r.tmin), make_float4(vec(m0), vec(m1), vec(m2), r.tmax));
}

// Starts a ray: tests the planes (unbounded, kept out of the BVH; testing them
// first gives the tree a tighter tmax). Returns true when the ray is already
// finished (an any-hit ray that hit a plane, or an empty tree).
template <bool ANY>
__device__ __forceinline__ bool trace_init(const DeviceScene& S, const TRay& r, int ignore_prim, TState& ts) {
  ts.tcur = r.tmax;
  ts.found = false;
  ts.best = -1;
  ts.bestPrim = -1;
  ts.bestQuad = 0;
  ts.bu = 0.f;
  ts.bv = 0.f;
  ts.sp = 0;
  ts.node = 0;
  ts.inst = -1;
  ts.bestInst = -1;
  for (int k = 0; k < S.n_planes; ++k) {
    if (ANY && S.plane_meta[k].x == ignore_prim) continue;
    float t = plane_t(r, __ldg(&S.planes[k]));
    bool take = t >= r.tmin && t <= r.tmax && accept_t(t, r.tmin, ts.tcur, ts.found);
    if (!ANY && !take && S.prim_rank && ts.found && t == ts.tcur)
      take = S.prim_rank[S.plane_meta[k].x] > S.prim_rank[ts.bestPrim];  // list order: the later plane
    if (take) {
      ts.tcur = t; ts.found = true; ts.best = -2 - k; ts.bu = 0.f; ts.bv = 0.f;
      if (S.prim_rank) ts.bestPrim = S.plane_meta[k].x;
      if (ANY) return true;
    }
  }
  return S.n_nodes <= 0;
}

// GBRT_SCENE_LIST_ORDER: whether a hit on record rec (primitive prim, in the
// instance being traversed) at exactly the best t so far comes later in the
// scene's list than the best hit: by the primitives' (or instances') ranks,
// then, within one mesh instance, by the mesh triangles' indices. Reached
// only on exact ties.
template <bool GEN>
__device__ __noinline__ bool list_later(const DeviceScene& S, int32_t prim, int32_t rec, const TState& ts) {
  int32_t top = prim, btop = ts.bestPrim, sub = 0, bsub = 0;
  if (GEN && ts.inst >= 0) {
    top = __float_as_int(__ldg(S.inst + 4 * int64_t(ts.inst) + 3).y);
    sub = S.rec_sub ? S.rec_sub[rec] : 0;
  }
  if (GEN && ts.bestInst >= 0) {
    btop = __float_as_int(__ldg(S.inst + 4 * int64_t(ts.bestInst) + 3).y);
    bsub = S.rec_sub ? S.rec_sub[ts.best] : 0;
  }
  const int32_t a = S.prim_rank[top], b = S.prim_rank[btop];
  return a != b ? a > b : sub > bsub;
}

// One traversal step: one 4-wide node or one leaf. ANY: stop at the first
// accepted hit and skip records whose prim id equals ignore_prim. WT:
// watertight triangle test. GEN: the general leaves, CSG objects and
// instances (entering an instance pushes the rest of its leaf and a return
// marker, then walks the mesh's tree with the ray in the mesh's space).
// Returns true when the ray is finished.
//
// Acceptance: the first hit may lie anywhere in [tmin, tmax] (Ray::inRange is
// inclusive); later hits must be strictly closer. One exception keeps
// Quad::intersect's rule (src/quad.cpp:23-34) that the first triangle of a
// quad wins over the second whenever it is hit: the first half replaces a
// current best that is the same quad's second half even at a larger t, and the
// second half never replaces the first.
template <bool ANY, bool COUNT, bool WT, int STACK, bool GEN>
__device__ __forceinline__ bool trace_step(const DeviceScene& S, const TRay& wr, int ignore_prim, TState& ts,
                                           int* stack, int* err, TraceCounters* cnt) {
  const int32_t node = ts.node;
  const TRay& r = (GEN && ts.inst >= 0) ? ts.oray : wr;
  if (node >= 0) {
    if (!in_range(node < S.n_nodes, err)) return true;
    // Offsets (in float4) of the near and far planes of each axis.
    const int nxo = r.ix >= 0.f ? 0 : 1, nyo = r.iy >= 0.f ? 2 : 3, nzo = r.iz >= 0.f ? 4 : 5;
    const float4* np = S.nodes + 8 * int64_t(node);
    const float4 nx = __ldg(np + nxo), fx = __ldg(np + (1 - nxo));
    const float4 ny = __ldg(np + nyo), fy = __ldg(np + (5 - nyo));
    const float4 nz = __ldg(np + nzo), fz = __ldg(np + (9 - nzo));
    const int4 rf = __ldg(reinterpret_cast<const int4*>(np + 6));
    if (COUNT) cnt->nodes++;
    const float tcur = ts.tcur;
    float k0 = box_entry(r, nx.x, fx.x, ny.x, fy.x, nz.x, fz.x, tcur);
    float k1 = box_entry(r, nx.y, fx.y, ny.y, fy.y, nz.y, fz.y, tcur);
    float k2 = box_entry(r, nx.z, fx.z, ny.z, fy.z, nz.z, fz.z, tcur);
    float k3 = box_entry(r, nx.w, fx.w, ny.w, fy.w, nz.w, fz.w, tcur);
    int r0 = rf.x, r1 = rf.y, r2 = rf.z, r3 = rf.w;
    // Ascending entry distance (sorting network for four keys).
    cswap(k0, r0, k1, r1);
    cswap(k2, r2, k3, r3);
    cswap(k0, r0, k2, r2);
    cswap(k1, r1, k3, r3);
    cswap(k1, r1, k2, r2);
    if (k1 != CUDART_INF_F) {
      if (ts.sp + 3 > STACK) { atomicOr(err, kErrStack); return true; }
      if (k3 != CUDART_INF_F) stack[ts.sp++] = r3;
      if (k2 != CUDART_INF_F) stack[ts.sp++] = r2;
      stack[ts.sp++] = r1;
    }
    if (k0 != CUDART_INF_F) {
      ts.node = r0;
      return false;
    }
  } else {
    // Leaf.
    uint32_t lv = ~uint32_t(node);
    int64_t first = int64_t(lv >> 4), count = int64_t(lv & 15u) + 1;
    if (!in_range(first + count <= S.n_recs, err)) return true;
    for (int64_t k = first; k < first + count; ++k) {
      const float4* rp = S.recs + 3 * k;
      float4 a = __ldg(rp + 0), b = __ldg(rp + 1), c = __ldg(rp + 2);
      if (COUNT) cnt->prims++;
      int kind = __float_as_int(a.w);
      int prim = __float_as_int(c.w);
      if (ANY && prim == ignore_prim) continue;
      int quad = kind == kRecTriangle ? __float_as_int(b.w) : 0;
      // The first half of a quad may displace its own second half at any t.
      bool displace = !ANY && quad == 1 && ts.found && ts.bestPrim == prim && ts.bestQuad == 2;
      float tlim = displace ? r.tmax : ts.tcur;
      float t, u = 0.f, v = 0.f;
      bool hit;
      if (kind == kRecTriangle) {
        if (WT) hit = tri_test_wt(r, a, b, c, tlim, t, u, v);
        else hit = tri_test_ref(r, a, b, c, tlim, t, u, v);
      } else if (kind == kRecSphere) {
        hit = sphere_test(r, a, b.x, tlim, t);
      } else if (!GEN || kind == kRecParallelogram) {
        hit = pgram_test(r, a, b, c, tlim, t, u, v);
      } else if (kind == kRecInstance) {
        // The rest of this leaf after the instance, then the way back.
        if (ts.sp + 2 > STACK) { atomicOr(err, kErrStack); return true; }
        const int64_t rest = first + count - (k + 1);
        if (rest > 0) stack[ts.sp++] = ~int32_t(uint32_t(k + 1) << 4 | uint32_t(rest - 1));
        stack[ts.sp++] = kInstPop;
        const int in = __float_as_int(b.x);
        if (!in_range(in >= 0 && in < S.n_inst, err)) return true;
        const float4* M = S.inst + 4 * int64_t(in);
        ts.oray = instance_ray(wr, __ldg(M), __ldg(M + 1), __ldg(M + 2));
        ts.inst = in;
        ts.node = __float_as_int(__ldg(M + 3).x);
        return false;
      } else {
        int leaf = -1;
        hit = csg_test(S, r, __float_as_int(b.w), __float_as_int(c.x), tlim, t, leaf);
        u = __int_as_float(leaf);
      }
      if (hit && ts.found && !displace) {
        // strictly closer (or, under GBRT_SCENE_LIST_ORDER, as close and later
        // in the list), and a second half never displaces its first half
        bool closer = t < ts.tcur;
        if (!ANY && !closer && t == ts.tcur && S.prim_rank) closer = list_later<GEN>(S, prim, int32_t(k), ts);
        hit = closer && !(quad == 2 && ts.bestPrim == prim && ts.bestQuad == 1);
      }
      if (hit) {
        ts.tcur = t; ts.found = true; ts.best = int32_t(k); ts.bu = u; ts.bv = v;
        ts.bestPrim = prim; ts.bestQuad = quad;
        if (GEN) ts.bestInst = ts.inst;
        if (ANY) return true;
      }
    }
  }
  if (ts.sp == 0) return true;
  ts.node = stack[--ts.sp];
  if (GEN && ts.node == kInstPop) {  // back from a mesh to world space
    ts.inst = -1;
    if (ts.sp == 0) return true;
    ts.node = stack[--ts.sp];
  }
  return false;
}

// A whole ray in one call (the ray-query entry points). Returns the internal
// hit encoding (RawHit::rec) and fills t/u/v, and with GEN the instance of the
// hit (-1: none). STACK is the capacity of the traversal stack
// (stack_need(depth of the 4-wide tree), both levels for two-level scenes).
template <bool ANY, bool COUNT, bool WT, int STACK, bool GEN>
__device__ __forceinline__ int32_t trace_ray(const DeviceScene& S, const TRay& r, int ignore_prim,
                                             float& t_best, float& u_best, float& v_best, int* err,
                                             TraceCounters* cnt, int32_t* inst_out = nullptr) {
  TState ts;
  int stack[STACK];
  if (!trace_init<ANY>(S, r, ignore_prim, ts)) {
    while (!trace_step<ANY, COUNT, WT, STACK, GEN>(S, r, ignore_prim, ts, stack, err, cnt)) {
    }
  }
  t_best = ts.found ? ts.tcur : CUDART_NAN_F;
  u_best = ts.bu;
  v_best = ts.bv;
  if (GEN && inst_out) *inst_out = ts.bestInst;
  return ts.best;
}

}  // namespace gbrt
