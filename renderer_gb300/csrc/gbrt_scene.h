// gbrt_scene.h — device layout of a flattened scene, shared by the host code
// that builds it and the kernels that read it.
//
// HBM layout (all arrays 16-byte aligned, read through the non-coherent
// 128-bit load path):
//   nodes  : n_nodes x 128 B  4-wide BVH nodes (bvh_build.h Node4), root at 0
//   recs   : n_recs x 48 B    primitive records in BVH leaf order, 3 float4:
//              triangle      (p1, kind) (p2, -) (p3, prim)
//              sphere        (centre, kind) (radius, 0, 0, -) (0, 0, 0, prim)
//              parallelogram (origin, kind) (u, -) (v, prim)
//              CSG object    (box lo, kind) (box hi, program start) (program length, 0, 0, prim)
//              instance      (box lo, kind) (instance, 0, 0, 0) (0, 0, 0, prim)
//            kind and prim are int bit patterns in the w lanes.
//   Two-level scenes: the nodes and records of every instanced mesh follow
//   the top-level ones in the same arrays (absolute indices); a mesh's
//   triangle records carry the prim id kMeshTriangle.
//   inst   : n_inst x 64 B    world-to-object 3 x 4 rows (3 float4), then
//                             (mesh root node, prim id, mesh, -) as ints
//   meta   : n_recs x 16 B    (prim id, material, normal index or -1, light)
//   tri_nrm: per smooth triangle 3 normals (9 floats, padded to 12)
//   planes : n_planes x float4 plane vector; plane_meta (prim, material)
//   materials, lights: small tables; env texels H x W x 3 float (BGR)
//   textures: texels of every texture (BGR), their table, per-triangle uv
// Planes have unbounded boxes and live outside the BVH; the environment map is
// what a ray with tmax = +inf sees when it hits nothing else.
#pragma once

#include <cstdint>

#include "../../include/gbrt.h"

namespace gbrt {

enum RecKind : int32_t { kRecTriangle = 0, kRecSphere = 1, kRecParallelogram = 2, kRecCSG = 3, kRecInstance = 4 };

// Prim id of an instanced mesh's triangle records (a hit reports its
// instance's id instead); never equal to a shadow ray's ignored prim.
constexpr int32_t kMeshTriangle = -0x7ffffff0;
// Traversal stack entry that returns from an instance's mesh to world space
// (no leaf encoding reaches it: records are fewer than 2^27).
constexpr int32_t kInstPop = -0x7fffffff - 1;

// Material kinds on the device (gbrt_material_type plus the two emitters that
// are their own material in the renderer: AreaLight and EnvironmentMap).
enum DevMatKind : int32_t {
  kMatDark = GBRT_MAT_DARK,
  kMatDiffuse = GBRT_MAT_DIFFUSE,
  kMatMirror = GBRT_MAT_MIRROR,
  kMatPhong = GBRT_MAT_PHONG,
  kMatBlinn = GBRT_MAT_BLINN,
  kMatTransparent = GBRT_MAT_TRANSPARENT,
  kMatTexture = GBRT_MAT_TEXTURE,
};

struct alignas(16) DevMaterial {
  int32_t type;
  float kd[3];
  float ks[3];
  float exponent;
  float ior;
  float rho_d, rho_s;  // lum(kd), lum(ks) for Phong lobe selection
  int32_t tex;         // texture material: texture index (gamma in exponent)
};

struct alignas(16) DevLight {
  int32_t type;       // gbrt_light_type
  int32_t prim;       // primitive id (== light index)
  float origin[3];
  float u[3], v[3];
  float normal[3];    // u x v (unnormalised)
  float normal_len;   // |u x v| (computed through double, like QVector3D::length)
  float nhat[3];      // normalised normal
  float intensity[3]; // BGR; for the env map: its coefficient
};

// The checked build (renderer_gb300/build.py with checked=True: -DGBRT_CHECKED)
// tests the indices the kernels follow (tree nodes, leaf records, instances,
// hit records, lights, materials, queue slots) before using them. A failed
// test sets bit 2 of the call's error word and abandons that access; the
// call then returns GBRT_ERR_NUMERIC. In the normal build the tests compile
// away.
#ifdef GBRT_CHECKED
constexpr bool kChecked = true;
#else
constexpr bool kChecked = false;
#endif
constexpr int kErrStack = 1, kErrIndex = 2;  // bits of the error word
#ifdef __CUDACC__
__device__ __forceinline__ bool in_range(bool ok, int* err) {
  if (kChecked && !ok) {
    atomicOr(err, kErrIndex);
    return false;
  }
  return true;
}
#endif

// Plain-old-data view of a scene on the device, passed by value to kernels.
struct DeviceScene {
  const float4* nodes;
  const float4* recs;
  const int4* meta;
  const float* tri_nrm;  // 12 floats per smooth triangle
  const float4* planes;
  const int2* plane_meta;  // (prim, material)
  const DevMaterial* materials;
  const DevLight* lights;
  const float* env_texels;
  int64_t n_nodes, n_recs;
  int32_t n_planes, n_materials, n_lights;
  int32_t env_light;      // light index / prim id of the environment map, -1 if none
  int32_t env_w, env_h, env_mapping;
  float env_coef[3];
  // Importance sampling of the environment by the physical estimator (null
  // without a map, with a black one or with GBRT_SCENE_ENV_UNIFORM): a
  // piecewise-constant density over the mapping's parameter square of env_h
  // rows x env_w cells. env_marg: the rows' CDF (env_h + 1 floats, 0 ... 1);
  // env_cond: per row the cells' CDF (env_w + 1 floats each); env_dens: per
  // cell its probability x env_w x env_h (the density over the square),
  // computed from the float CDFs so that it is exactly what sampling draws.
  const float* env_marg;
  const float* env_cond;
  const float* env_dens;
  // Textures (null when no material uses one): texels of all textures one
  // after the other (3 floats, BGR), per texture (first texel, W, H, -), and
  // per triangle its three texture coordinates (6 floats, input order; the
  // triangle of primitive id p is p - tri_pid0).
  const float* tex_texels;
  const int4* tex_info;
  const float* tri_uv;
  int32_t n_textures, tri_pid0;
  // CSG: nodes as three float4, (a, op), (b, material), (left, right, -, -)
  // (gbrt_csg_node), and the objects' postfix programs of node indices.
  const float4* csg_nodes;
  const int32_t* csg_prog;
  // Instances (null when none): four float4 each, see above.
  const float4* inst;
  int32_t n_inst;
  // GBRT_SCENE_LIST_ORDER (both null without it): per primitive id its rank
  // in the scene's list, and per record its triangle's index in its mesh
  // (null when the scene has no mesh instances).
  const int32_t* prim_rank;
  const int32_t* rec_sub;
};

// Internal hit encoding of the traversal kernels.
//   rec >= 0       BVH record index
//   rec == -1      nothing hit (the environment, if any, when tmax = +inf)
//   rec <= -2      plane number -2 - rec
struct alignas(16) RawHit {
  float t;
  int32_t rec;
  float u, v;
};

}  // namespace gbrt
