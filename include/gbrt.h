/*
 * gbrt.h — C ABI of the GB300 unidirectional path-tracing hot path.
 *
 * This is the drop-in boundary for the renderer's PerPixelRenderer ->
 * UniDiPathTracingIntegrator path. Every entry point takes plain pointers and
 * sizes; no C++ or torch types cross it, and no C++ exception escapes it.
 *
 * Conventions shared with the renderer being replaced:
 *   - Spectra (material colours, light intensities, film) are stored in BGR
 *     channel order, as cv::Vec3f is in the renderer (src/sceneast.cpp:410-414,
 *     src/mathhelper.cpp:102-105). The scene-file parser swaps RGB->BGR.
 *   - A miss is reported as t = NaN (src/hitrecord.h:62-64, :111-114).
 *   - A hit on the environment map is reported at t = +inf with the map's
 *     primitive id (src/environmentmap.cpp:73-83).
 *   - The film is H x W x 3 float, row-major, row 0 at the top of the image
 *     (src/perpixelrenderer.cpp:62-96, src/camera.cpp:50-58).
 *
 * Primitive ids. The renderer renders IntersectableList(lights..., scene)
 * (src/sceneast.cpp:673-695) and flattens nested lists into BVH leaves
 * (src/intersectable.cpp:6-14, src/intersectablelist.cpp:67-78). gbrt numbers
 * leaves in that spirit with a fixed type order:
 *   [0, n_lights)                       lights (area lights and the env map are
 *                                       hittable; point lights never are)
 *   [+0, +n_tri)                        triangles
 *   [+0, +n_quads)                      quads (one id per quad, like the
 *                                       renderer's Quad object, src/quad.h:32)
 *   [+0, +n_spheres)                    spheres
 *   [+0, +n_planes)                     planes
 *   [+0, +n_csg)                        CSG objects (one id per object)
 *   [+0, +n_instances)                  mesh instances (one id per instance)
 *
 * Threading: calls on one gbrt_ctx are serialised by the caller; distinct
 * contexts are independent. All device memory is owned by the library.
 */
#ifndef GBRT_H
#define GBRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBRT_ABI_VERSION 1

typedef enum gbrt_status {
  GBRT_OK = 0,
  GBRT_ERR_INVALID_ARG = 1,
  GBRT_ERR_OOM = 2,
  GBRT_ERR_CUDA = 3,
  GBRT_ERR_CANCELLED = 4,
  GBRT_ERR_TIMEOUT = 5,
  GBRT_ERR_NUMERIC = 6,
  GBRT_ERR_PARSE = 7,
  GBRT_ERR_IO = 8,
  GBRT_ERR_UNSUPPORTED = 9
} gbrt_status;

/* Material kinds: src/material.h:30-50 and its subclasses. */
typedef enum gbrt_material_type {
  GBRT_MAT_DARK = 0,        /* DarkMatter, src/darkmatter.cpp:32-39          */
  GBRT_MAT_DIFFUSE = 1,     /* DiffuseMaterial, src/diffusematerial.cpp:25-28 */
  GBRT_MAT_MIRROR = 2,      /* MirrorMaterial, src/mirrormaterial.cpp:31-41   */
  GBRT_MAT_PHONG = 3,       /* PhongMaterial, src/phongmaterial.cpp:31-81     */
  GBRT_MAT_BLINN = 4,       /* BlinnMaterial, src/blinnmaterial.cpp:34-84     */
  GBRT_MAT_TRANSPARENT = 5, /* TransparentMaterial, src/transparentmaterial.cpp:34-80 */
  /* TextureMaterial, src/texturematerial.cpp:33-74: a diffuse material whose
   * albedo at texture coordinates (u, v) is pow(kd * T(u, v), exponent), T
   * the bilinear sample of textures[texture] at (frac(u) (W - 1),
   * frac(1 - v) (H - 1)) with the border replicated (cv::getRectSubPix). */
  GBRT_MAT_TEXTURE = 6
} gbrt_material_type;

typedef struct gbrt_material {
  int32_t type;      /* gbrt_material_type                                 */
  float kd[3];       /* diffuse colour (BGR); phong/blinn/diffuse          */
  float ks[3];       /* specular colour (BGR); phong/blinn                 */
  float exponent;    /* phong/blinn exponent                               */
  float ior;         /* transparent: refraction coefficient                */
  float coefficient; /* mirror: coefficient (ignored, as in the renderer)  */
  int32_t texture;   /* texture: index into gbrt_scene_desc.textures       */
} gbrt_material;

/* A texture image, height x width x 3 float BGR, row 0 at the top (the
 * texels of cv::imread(...) converted with scale 1/255, as the renderer
 * loads them, src/texturematerial.cpp:48-60). */
typedef struct gbrt_texture {
  int32_t width, height;
  const float* texels;  /* host pointer, copied by gbrt_scene_create */
} gbrt_texture;

/* Quad(p1,p2,p3,p4): triangles (p1,p2,p4) and (p4,p2,p3), src/quad.h:32. */
typedef struct gbrt_quad {
  float p[4][3];
  int32_t material;
} gbrt_quad;

/* Sphere(center, radius), src/sphere.cpp:29-56. */
typedef struct gbrt_sphere {
  float center[3];
  float radius;
  int32_t material;
} gbrt_sphere;

/* Plane: points x with dot((x,1), plane) = 0, src/plane.cpp:27-40. */
typedef struct gbrt_plane {
  float plane[4];
  int32_t material;
} gbrt_plane;

typedef enum gbrt_light_type {
  GBRT_LIGHT_AREA = 0,   /* AreaLight(origin,u,v,Le), src/arealight.cpp:31-118 */
  GBRT_LIGHT_POINT = 1,  /* PointLight(pos,I), src/pointlight.cpp:29-70        */
  GBRT_LIGHT_ENV = 2,    /* EnvironmentMap, src/environmentmap.cpp:16-108      */
  GBRT_LIGHT_BLACK = 3,  /* BlackLight (failed env map), src/blacklight.cpp:5-24 */
  GBRT_LIGHT_CONE = 4    /* ConeLight(pos,dir,angle,I), src/conelight.cpp:31-60 */
} gbrt_light_type;

typedef struct gbrt_light {
  int32_t type;        /* gbrt_light_type                                  */
  float origin[3];     /* area: corner; point / cone: position             */
  float u[3];          /* area: first edge; cone: axis direction           */
  float v[3];          /* area: second edge; cone: v[0] = opening angle    */
                       /* (radians, measured from the axis)                */
  float intensity[3];  /* BGR; area: Le; point / cone: I; env: coefficient */
} gbrt_light;

typedef enum gbrt_env_mapping {
  GBRT_ENV_ANGULAR = 0, /* angular light probe, src/environmentmap.cpp:57-65 */
  GBRT_ENV_LATLONG = 1  /* equirectangular (extension for lat-long skies)   */
} gbrt_env_mapping;

/* Environment image, height x width x 3 float BGR, row-major. At most one per
 * scene; a light of type GBRT_LIGHT_ENV refers to it. */
typedef struct gbrt_env_map {
  int32_t width, height;
  int32_t mapping;        /* gbrt_env_mapping */
  const float* texels;    /* host pointer, copied by gbrt_scene_create */
} gbrt_env_map;

/* Constructive solid geometry, src/csgobject.cpp:25-44,
 * src/csgoperation.cpp:27-97, src/sphere.cpp:29-56, src/axisalignedbox.cpp:
 * 30-73. A CSG object is a tree of nodes: leaves are spheres (centre a,
 * radius b[0]) and axis-aligned boxes (min a, max b) with a material;
 * operations combine their left and right subtrees' interval lists. A hit is
 * the first interval boundary at or beyond the ray's start; a box's exit
 * boundary carries its entry face's normal, as in the renderer. At most
 * GBRT_CSG_MAX_LEAVES leaves per object. */
typedef enum gbrt_csg_op {
  GBRT_CSG_SPHERE = 0,
  GBRT_CSG_BOX = 1,
  GBRT_CSG_ISECT = 2,  /* left and right, src/csgoperation.cpp:78-81 */
  GBRT_CSG_UNION = 3,  /* left or right */
  GBRT_CSG_DIFF = 4,   /* left and not right */
  GBRT_CSG_XOR = 5     /* left xor right */
} gbrt_csg_op;
#define GBRT_CSG_MAX_LEAVES 8

typedef struct gbrt_csg_node {
  int32_t op;           /* gbrt_csg_op */
  int32_t left, right;  /* operations: child node indices */
  float a[3], b[3];     /* leaves: sphere (centre, radius in b[0]) or box (min, max) */
  int32_t material;     /* leaves */
} gbrt_csg_node;

/* Instanced triangle meshes (a two-level BVH). A mesh is a triangle soup in
 * its own space, built into its own BVH once; an instance places a mesh with
 * an affine object-to-world transform. As IntersectableInstance
 * (src/intersectableinstance.cpp:24-46, src/hitrecord.h:79-84): a ray is
 * moved into the mesh's space by the inverse transform (the direction is not
 * renormalised, so the ray parameter t is the same in both spaces) and the
 * normal back by the inverse transpose. Mesh triangles take the default
 * texture coordinates. Each instance is one primitive in the id space. */
typedef struct gbrt_mesh {
  const float* tri_pos;     /* n_tri x 9 */
  const float* tri_nrm;     /* optional n_tri x 9 (as gbrt_scene_desc.tri_nrm) */
  const int32_t* tri_mat;   /* optional n_tri (NULL: material 0) */
  int64_t n_tri;
} gbrt_mesh;

typedef struct gbrt_instance {
  float transform[12];      /* row-major 3 x 4, object -> world */
  int32_t mesh;             /* index into gbrt_scene_desc.meshes */
  int32_t pad;
} gbrt_instance;

typedef struct gbrt_scene_desc {
  const gbrt_material* materials; int32_t n_materials;
  /* triangle soup: n_tri x 9 positions (p1,p2,p3); optional n_tri x 9 normals
   * (a triangle whose three normals are not all non-zero uses its geometric
   * normal, src/sceneast.cpp:514-521); optional n_tri x 6 texcoords (NULL:
   * (0,0), (0,1), (1,0), the Triangle constructor's default, src/triangle.h:
   * 35-36); material per triangle (NULL: all use material 0). */
  const float* tri_pos; const float* tri_nrm; const float* tri_uv;
  const int32_t* tri_mat; int64_t n_tri;
  const gbrt_quad* quads; int32_t n_quads;
  const gbrt_sphere* spheres; int32_t n_spheres;
  const gbrt_plane* planes; int32_t n_planes;
  const gbrt_light* lights; int32_t n_lights;
  const gbrt_env_map* env;  /* NULL if no environment map */
  int32_t flags;            /* gbrt_scene_flags */
  const gbrt_texture* textures; int32_t n_textures;
  /* CSG objects: csg_roots[i] is the root node (in csg_nodes) of object i */
  const gbrt_csg_node* csg_nodes; int32_t n_csg_nodes;
  const int32_t* csg_roots; int32_t n_csg;
  /* instanced meshes */
  const gbrt_mesh* meshes; int32_t n_meshes;
  const gbrt_instance* instances; int32_t n_instances;
  /* Optional (NULL: primitive-id order): per primitive id, its position in
   * the scene's root list (lights first, then the scene's intersectables as
   * the scene file lists them, src/sceneast.cpp:673-679). Used only with
   * GBRT_SCENE_LIST_ORDER; gbrt_parsed_scene_desc fills it. */
  const int32_t* list_rank;
} gbrt_scene_desc;

typedef enum gbrt_scene_flags {
  /* Triangle inside/outside decisions by the watertight test of Woop, Benthin
   * and Wald (JCGT 2013) instead of the renderer's own float test
   * (src/triangle.cpp:30-56). The renderer's test leaves cracks and overlaps
   * along shared edges; with this flag no ray slips through a closed mesh, at
   * the price of decisions that differ from the renderer's near edges. */
  GBRT_SCENE_WATERTIGHT = 1,
  /* Build the BVH on the GPU (linear BVH over Morton codes, collapsed to the
   * same 4-wide nodes) instead of the host's binned SAH: milliseconds
   * instead of seconds for multi-million-triangle scenes, at some cost in
   * traversal speed. Hits are the same; only exact-t ties may resolve
   * differently. A tree too deep for the traversal stack falls back to the
   * host build. gbrt_scene_info then reports max_depth 0 and SAH cost 0. */
  GBRT_SCENE_GPU_BUILD = 2,
  /* The physical estimator's next-event estimation samples the environment
   * map uniformly over the sphere instead of in proportion to its luminance
   * (importance sampling: a piecewise-constant density over the map's texels
   * weighted by their solid angle, combined with BSDF sampling by the power
   * heuristic). For measuring what importance sampling gains; the
   * renderer's own estimator (GBRT_SEM_REFERENCE) samples it by the cosine
   * either way (src/environmentmap.cpp:40-54). */
  GBRT_SCENE_ENV_UNIFORM = 4,
  /* Exact ties in t between different primitives resolve as the renderer's
   * IntersectableList does (src/intersectablelist.cpp:29-47: each entry is
   * tested with the ray shortened to the best hit so far, inclusive, so the
   * later entry wins), which is what the renderer computes with --no-bvh
   * (src/sceneast.cpp:681-688): the later primitive in list order
   * (gbrt_scene_desc.list_rank) wins, and inside a mesh instance the later
   * mesh triangle. Without the flag an exact tie goes to whichever primitive
   * the traversal reaches first. Closest hits that are not ties are the same
   * either way. */
  GBRT_SCENE_LIST_ORDER = 8
} gbrt_scene_flags;

/* Camera(cop, lookAt, up, fov[radians, full vertical], resolution),
 * src/camera.cpp:34-58. */
typedef struct gbrt_camera {
  float eye[3], look_at[3], up[3];
  float fov;
  int32_t width, height;
} gbrt_camera;

typedef enum gbrt_semantics {
  /* the renderer's estimator with all of its quirks */
  GBRT_SEM_REFERENCE = 0,
  /* Physically based estimator; no counterpart in the renderer. Unbiased
   * Russian roulette (survival 1 - termination_prob from the fourth vertex
   * on), next-event estimation with the light-count factor combined with
   * BSDF-sampled emission by the power heuristic, normalised modified
   * Phong / Blinn lobes sampled with their own pdfs. Same scenes, same
   * options; every light type and material the reference path accepts. */
  GBRT_SEM_PHYSICAL = 1
} gbrt_semantics;

/* Options of PerPixelRenderer (src/perpixelrenderer.cpp:103-112) plus the
 * path-length cap, which the renderer fixes at compile time (MAX_DEPTH 5,
 * src/renderer.h:38). */
typedef struct gbrt_render_params {
  int32_t x_samples;        /* --pt-x-samples (default 4)                  */
  int32_t y_samples;        /* --pt-y-samples (default 4)                  */
  float termination_prob;   /* --pt-termination-prob (default 0.5)         */
  int32_t max_depth;        /* MAX_DEPTH (renderer: 5)                     */
  uint64_t seed;            /* --seed                                      */
  int32_t semantics;        /* gbrt_semantics                              */
  int32_t batch_paths;      /* paths in flight per wavefront; 0 = auto     */
  int32_t flags;            /* gbrt_render_flags                           */
} gbrt_render_params;

typedef enum gbrt_render_flags {
  /* Time every extend / shade / shadow kernel with CUDA events on the
   * render stream (gbrt_stats *_ms fields). */
  GBRT_RENDER_TIME_KERNELS = 1,
  /* Count BVH nodes visited and primitives tested (gbrt_stats counters);
   * slower, for measurement only. */
  GBRT_RENDER_COUNT_TRAVERSAL = 2
} gbrt_render_flags;

typedef struct gbrt_stats {
  uint64_t paths;           /* camera samples traced to termination        */
  uint64_t extension_rays;  /* closest-hit rays (camera + bounce)          */
  uint64_t shadow_rays;     /* any-hit rays                                */
  uint64_t nonfinite;       /* samples whose radiance was NaN/inf (dropped)*/
  double render_ms;         /* device time of the render loop              */
  uint64_t kernel_launches; /* kernels launched by the render loop         */
  /* with GBRT_RENDER_TIME_KERNELS: summed kernel times and launch counts */
  double extend_ms, shade_ms, shadow_ms;
  uint64_t extend_launches, shade_launches, shadow_launches;
  /* with GBRT_RENDER_COUNT_TRAVERSAL: traversal work of all rays */
  uint64_t nodes_closest, prims_closest, nodes_any, prims_any;
} gbrt_stats;

/* Ray(origin, direction, from, to), src/ray.h:36-57. 32 bytes. */
typedef struct gbrt_ray {
  float org[3]; float tmin;
  float dir[3]; float tmax;
} gbrt_ray;

/* HitRecord essentials, src/hitrecord.h:35-60. 16 bytes. */
typedef struct gbrt_hit {
  float t;          /* NaN on a miss, +inf on the environment map         */
  int32_t prim;     /* primitive id (see above); -1 on a miss             */
  float u, v;       /* barycentrics of the hit (triangles/quads)          */
} gbrt_hit;

typedef struct gbrt_ctx gbrt_ctx;
typedef struct gbrt_scene gbrt_scene;

/* ---- library ---------------------------------------------------------- */
int32_t gbrt_abi_version(void);
/* NUL-terminated message of the last failing call on ctx (or a global one
 * when ctx is NULL). Valid until the next call on that context. */
const char* gbrt_last_error(const gbrt_ctx* ctx);

/* ---- context (replaces RenderingManager/Renderer set-up,
 *      src/renderingmanager.cpp:8-59, src/renderer.cpp:131-145) ---------- */
gbrt_status gbrt_ctx_create(int32_t device, gbrt_ctx** out);
gbrt_status gbrt_ctx_destroy(gbrt_ctx* ctx);
/* Per-call device buffers (wavefront state, films) come from a memory pool
 * of the context that keeps freed memory reserved for the next call (about
 * 20 GB after a render of 2^26 paths or more with the default wavefront).
 * This returns the reserved, unused part to the driver (and reports how many
 * bytes the pool still holds; may be NULL). */
gbrt_status gbrt_ctx_trim(gbrt_ctx* ctx, uint64_t* reserved_bytes);

/* Host-side fault injection, for tests of the failure paths. The renderer
 * has no counterpart; it stands in for the conditions the renderer meets with
 * assert (src/perpixelrenderer.cpp:90-91) or not at all. Every fault is made
 * on the host or by a bounded wait: none faults, traps or hangs the GPU, and
 * the context stays usable afterwards. Faults stay set until
 * GBRT_FAULT_NONE clears them all.
 *   GBRT_FAULT_ALLOC       arg = n: the device allocations of this context
 *                          succeed n more times, then one fails as out of
 *                          memory (the call returns GBRT_ERR_OOM); one-shot.
 *   GBRT_FAULT_NAN         arg = n > 0: the radiance of every camera sample
 *                          whose path index is a multiple of n is replaced by
 *                          NaN before accumulation (counted in
 *                          gbrt_stats.nonfinite and dropped); 0 turns it off.
 *   GBRT_FAULT_SMALL_STACK arg != 0: renders trace with a 4-entry traversal
 *                          stack; a ray that needs more sets the error word and
 *                          the call returns GBRT_ERR_NUMERIC.
 *   GBRT_FAULT_GUIDE_WAIT  arg = ns in (0, 1e9]: the guide's kernels issue no
 *                          tensor-core products and give up waiting for them
 *                          after arg ns (the call returns GBRT_ERR_TIMEOUT,
 *                          the kernels' tensor memory is freed); 0 turns it off.
 */
typedef enum gbrt_fault {
  GBRT_FAULT_NONE = 0,
  GBRT_FAULT_ALLOC = 1,
  GBRT_FAULT_NAN = 2,
  GBRT_FAULT_SMALL_STACK = 3,
  GBRT_FAULT_GUIDE_WAIT = 4
} gbrt_fault;
gbrt_status gbrt_debug_fault(gbrt_ctx* ctx, int32_t kind, int64_t arg);

/* ---- scene (replaces scene_builder::getScene + Intersectable::createBVH,
 *      src/sceneast.cpp:673-695, src/intersectable.cpp:11-14,
 *      src/bvh.cpp:67-94). Deep-copies desc to the device and builds the
 *      BVH. ------------------------------------------------------------- */
gbrt_status gbrt_scene_create(gbrt_ctx* ctx, const gbrt_scene_desc* desc,
                              gbrt_scene** out);
/* A scene must be destroyed before the context it was created on. */
gbrt_status gbrt_scene_destroy(gbrt_scene* scene);
/* BVH statistics: nodes, leaves, max depth, SAH cost, build milliseconds. */
gbrt_status gbrt_scene_info(const gbrt_scene* scene, int64_t* n_nodes,
                            int64_t* n_leaves, int32_t* max_depth,
                            double* sah_cost, double* build_ms);
/* Box of the scene's bounded primitives (planes excluded): lo.xyz, hi.xyz.
 * (No counterpart in the renderer; the guide normalises positions by it.) */
gbrt_status gbrt_scene_bounds(const gbrt_scene* scene, float bounds[6]);

/* ---- ray queries (batched Intersectable::intersect, src/intersectable.h:40;
 *      BVHNode::intersect, src/bvh.cpp:135-149) ------------------------- */
/* Host pointers; copies in and out inside the call. */
gbrt_status gbrt_trace_closest(gbrt_scene* scene, const gbrt_ray* rays,
                               int64_t n, gbrt_hit* hits);
/* Any-hit occlusion: occluded[i] = 1 if some primitive other than
 * ignore_prim[i] (may be NULL) is hit in [tmin, tmax]. The environment map
 * never occludes. Host pointers. (src/arealight.cpp:41-46,
 * src/pointlight.cpp:55-60, src/environmentmap.cpp:44-50) */
gbrt_status gbrt_trace_any(gbrt_scene* scene, const gbrt_ray* rays,
                           const int32_t* ignore_prim, int64_t n,
                           uint8_t* occluded);
/* Device-pointer variants, enqueued on the context's stream (stream may be
 * NULL for the context stream, else a cudaStream_t). Asynchronous. */
gbrt_status gbrt_trace_closest_device(gbrt_scene* scene, const gbrt_ray* d_rays,
                                      int64_t n, gbrt_hit* d_hits, void* stream);
gbrt_status gbrt_trace_any_device(gbrt_scene* scene, const gbrt_ray* d_rays,
                                  const int32_t* d_ignore_prim, int64_t n,
                                  uint8_t* d_occluded, void* stream);

/* ---- render (PerPixelRenderer::render + UniDiPathTracingIntegrator,
 *      src/perpixelrenderer.cpp:43-101, src/unidipathtracingintegrator.cpp:34-107,
 *      src/renderer.cpp:47-106) ----------------------------------------- */
/* film_bgr: H x W x 3 float host buffer, overwritten with the per-pixel
 * mean. opt_sum / opt_sumsq: optional H x W x 3 double host buffers that
 * receive the per-pixel sum and sum of squares of the per-sample radiance
 * (for variance / z-tests). stop_flag: optional host flag polled between
 * wavefront batches (the renderer's doStop, src/renderer.h:71); a set flag
 * ends the call with GBRT_ERR_CANCELLED. stats may be NULL. */
gbrt_status gbrt_render(gbrt_scene* scene, const gbrt_camera* camera,
                        const gbrt_render_params* params, float* film_bgr,
                        double* opt_sum, double* opt_sumsq,
                        const volatile int32_t* stop_flag, gbrt_stats* stats);
/* Device-resident variant: d_film_bgr (float) and the optional d_sum /
 * d_sumsq (double) are device pointers of H x W x 3. Synchronous. */
gbrt_status gbrt_render_device(gbrt_scene* scene, const gbrt_camera* camera,
                               const gbrt_render_params* params,
                               float* d_film_bgr, double* d_sum,
                               double* d_sumsq, gbrt_stats* stats);
/* No counterpart in the renderer. The same render as gbrt_render_device,
 * for callers that cannot call cudaMalloc during a render: an application
 * whose device memory is owned by its own pool or held to a fixed budget, or a
 * frame loop that cannot take the device-wide synchronisation cudaMalloc and
 * cudaFree may imply. It allocates nothing: the wavefront state lives in one
 * fixed 20 MiB array in device memory (a batch of at most
 * GBRT_NOALLOC_MAX_BATCH paths), which every GPU that loads this library
 * holds until the process exits. The caller passes every buffer that scales
 * with the image: d_film_bgr (float) and d_sum (double, required here) and
 * the optional d_sumsq, each H x W x 3 on the device. params->batch_paths = 0
 * means GBRT_NOALLOC_MAX_BATCH; a larger value is rejected with
 * GBRT_ERR_INVALID_ARG. The first call on a context looks up the array's
 * device address (a context created after cudaDeviceReset looks it up again).
 * That first call, like the first launch of any kernel, may also make the
 * CUDA driver load this library's kernels and enlarge its per-thread local
 * memory reservation (the traversal stacks live in local memory, up to 190
 * entries a thread): callers on a fixed memory budget should make one
 * warm-up call at start-up, and the first call must come before any stream
 * capture. All calls in the process share the one array and leave their
 * state in it (each call clears what must start at zero), so calls that
 * overlap on the GPU race: issue them one at a time. GBRT_RENDER_TIME_KERNELS
 * is ignored (stats get host-timed render_ms only). Synchronous. */
#define GBRT_NOALLOC_MAX_BATCH 65536
gbrt_status gbrt_render_device_noalloc(gbrt_scene* scene,
                                       const gbrt_camera* camera,
                                       const gbrt_render_params* params,
                                       float* d_film_bgr, double* d_sum,
                                       double* d_sumsq, gbrt_stats* stats);

/* Resumable accumulation in passes (a checkpoint of a long render, e.g. a
 * 65,536-spp reference, is the FP64 sums plus the number of passes done; the
 * renderer accumulates one image per process and has none). Renders passes
 * first_pass .. first_pass + n_passes - 1, pass k with the seed derived from
 * (params->seed, k) and params' samples per pixel, adding into d_sum (and
 * d_sumsq when given), which are cleared first only when first_pass is 0;
 * d_film (device, H x W x 3 BGR) gets the mean of all passes 0 ..
 * first_pass + n_passes - 1. Rendering passes [0, a) and then, from the
 * saved sums, [a, b) gives the sums and film of one call over [0, b): the
 * same paths, the same per-pixel order of the FP64 additions, and only the
 * order in which a vertex's shadow rays add into its path's radiance (float
 * atomics) may differ. stats add up over the call's passes. Synchronous. */
gbrt_status gbrt_render_passes(gbrt_scene* scene, const gbrt_camera* camera,
                               const gbrt_render_params* params,
                               int32_t first_pass, int32_t n_passes,
                               float* d_film_bgr, double* d_sum,
                               double* d_sumsq, gbrt_stats* stats);

/* ---- output (Tonemapper::map, src/tonemapper.cpp:31-56; the --save-exr,
 *      --save-img and --save-mat writers, src/main.cpp:223-265) ---------- */
/* rgb: width x height x 3 bytes, RGB order: clamp(255 * c^(1/gamma)) per
 * channel of the BGR film, truncated. Host buffers. */
gbrt_status gbrt_tonemap(const float* film_bgr, int32_t width, int32_t height,
                         float gamma, uint8_t* rgb);
/* Device buffers, enqueued on stream (NULL: the context stream). */
gbrt_status gbrt_tonemap_device(gbrt_ctx* ctx, const float* d_film_bgr,
                                int32_t width, int32_t height, float gamma,
                                uint8_t* d_rgb, void* stream);
/* Writes a host film by file extension: .exr (OpenEXR, uncompressed float
 * B,G,R), .pfm, .hdr (RGBE), .m (MATLAB function), or .png/.ppm/.bmp
 * (8-bit, tonemapped with gamma). */
gbrt_status gbrt_write_image(const char* path, const float* film_bgr,
                             int32_t width, int32_t height, float gamma);

/* ---- batches of renders (no counterpart in the renderer, which renders one
 *      image per process). The jobs run concurrently on several CUDA
 *      streams, each as the same wavefront as gbrt_render, so that many
 *      small images keep the GPU busy; the host waits once, at the end. ---- */
typedef struct gbrt_batch_job {
  gbrt_scene* scene;            /* created on the same context */
  gbrt_camera camera;
  gbrt_render_params params;    /* batch_paths 0: the call's batch_paths */
  float* film;                  /* host, H x W x 3 BGR */
} gbrt_batch_job;

typedef struct gbrt_batch_stats {
  uint64_t paths, extension_rays, shadow_rays, nonfinite;
  double wall_ms;               /* host wall time of the call */
  int32_t streams;
  int32_t pad;
  int64_t batch_paths;          /* wavefront size used for jobs without their own */
  double device_ms;             /* device time from the first job's start to the
                                   last job's end (films not yet copied out) */
  uint64_t kernel_launches;
} gbrt_batch_stats;

/* streams / batch_paths 0: the values gbrt_batch_autotune chose on this
 * context (4 and 2^22 before any tuning). job_ms (optional, n doubles): each
 * job's device time from its first to its last kernel. */
gbrt_status gbrt_render_batch(gbrt_ctx* ctx, const gbrt_batch_job* jobs,
                              int32_t n, int32_t streams, int64_t batch_paths,
                              double* job_ms, gbrt_batch_stats* stats);
/* Renders up to 8 of the jobs at one sample per pixel with 1, 2, 4 and 8
 * streams and wavefronts of 2^22 and 2^24 paths, keeps the fastest pair on
 * the context (for later calls with 0s) and returns it. Films are not
 * written. */
gbrt_status gbrt_batch_autotune(gbrt_ctx* ctx, const gbrt_batch_job* jobs,
                                int32_t n, int32_t* streams,
                                int64_t* batch_paths);

/* The single-launch batch (no counterpart in the renderer). The jobs' paths
 * are numbered one after the other and every wavefront holds the paths of as
 * many jobs as it covers, so that each launch of the extend, shade and shadow
 * kernels serves several images and scenes at once (each slot records its
 * job; the kernels read the job's scene and parameters from device tables).
 * One wavefront (set-up, camera rays, max_depth x (extend, shade, shadow),
 * accumulation) is captured as a CUDA graph and replayed until every path is
 * done; `pipelines` such graphs run at once on streams of the context
 * (pipeline k takes wavefronts k, k + pipelines, ...), so that one
 * wavefront's last, nearly empty bounces overlap another's first ones. Jobs
 * are numbered smallest first (pixels x spp x max_depth), so that small
 * images finish in the first wavefronts. All
 * jobs share one estimator (params.semantics) and one triangle test
 * (GBRT_SCENE_WATERTIGHT); at most 65,535 jobs; params.batch_paths is
 * ignored. Every path draws the numbers it draws in gbrt_render, so a job's
 * film equals its gbrt_render film up to the summation order of the FP64
 * pixel sums. */
typedef struct gbrt_batch_schedule {
  int64_t wavefront_paths;  /* paths per wavefront */
  int32_t pipelines;        /* wavefront pipelines in flight at once, 1..8 */
  int32_t trace_block;      /* threads per block of extend and shadow: 64 or 128 */
  int32_t shade_block;      /* threads per block of shade: 128 or 256 */
  int32_t pad;
} gbrt_batch_schedule;
/* schedule NULL, or a field 0: the value gbrt_batch_autotune_fused chose on
 * this context (2^24 paths, 2 pipelines, 128 and 256 threads before any
 * tuning). job_ms (optional): per job, device time from the batch's start to
 * the end of the wavefront that finishes it. stats->streams is the number of
 * pipelines; kernel_launches counts the kernels of the replayed graphs and
 * the final film kernel. */
gbrt_status gbrt_render_batch_fused(gbrt_ctx* ctx, const gbrt_batch_job* jobs,
                                    int32_t n,
                                    const gbrt_batch_schedule* schedule,
                                    double* job_ms, gbrt_batch_stats* stats);
/* Renders every job at up to 2 x 2 samples per pixel for wavefronts of 2^20, 2^22 and
 * 2^24 paths, 1, 2 and 4 pipelines (at most 2^25 paths in flight) and each
 * pair of tile sizes, keeps the fastest schedule (device time) on the context
 * and returns it. Films are not written. */
gbrt_status gbrt_batch_autotune_fused(gbrt_ctx* ctx, const gbrt_batch_job* jobs,
                                      int32_t n, gbrt_batch_schedule* schedule);

/* ---- neural path guiding. No counterpart in the renderer, whose
 *      integrators sample the BSDF only (src/unidipathtracingintegrator.cpp:
 *      34-46); used with the physical estimator. ---------------------------
 * The guide is an MLP 208 -> 64 -> 64 -> 64 -> 40 (ReLU, no biases) on a
 * frequency encoding of the position (normalised by bounds) and normal and a
 * one-blob encoding of the outgoing direction; its output is a mixture of 8
 * von Mises-Fisher lobes. Products run in BF16 on the tensor cores with FP32
 * accumulation; FP32 master weights and Adam state live on the device. */
typedef struct gbrt_guide gbrt_guide;
/* Parameters: row-major [out][in] matrices W1 64x208, W2 64x64, W3 64x64,
 * W4 40x64, concatenated. */
#define GBRT_GUIDE_PARAMS 24064
/* One network input: point, normal facing the viewer, outgoing direction. */
#define GBRT_GUIDE_INPUT 9
/* One mixture: lobe weights [8], then (mean x, y, z, kappa) for each lobe. */
#define GBRT_GUIDE_OUTPUT 40
/* One training sample: point, normal, outgoing direction, sampled incident
 * direction, weight = target / pdf (loss = -mean(weight * log q(direction))). */
#define GBRT_GUIDE_SAMPLE 13

gbrt_status gbrt_guide_create(gbrt_ctx* ctx, const float bounds[6],
                              uint64_t seed, gbrt_guide** out);
gbrt_status gbrt_guide_destroy(gbrt_guide* guide);
gbrt_status gbrt_guide_get_weights(gbrt_guide* guide, float* weights,
                                   size_t n);
/* Checkpoint and resume of training (no counterpart in the renderer): the
 * FP32 master parameters, Adam's first and second moments (GBRT_GUIDE_PARAMS
 * floats each, host buffers) and its step count. set_state restores all of
 * them, so that training continues exactly where the saved guide stopped
 * (up to the order of the float additions of the gradient), and marks the
 * guide usable by renders. */
gbrt_status gbrt_guide_get_state(gbrt_guide* guide, float* params,
                                 float* adam_m, float* adam_v, int64_t* step);
gbrt_status gbrt_guide_set_state(gbrt_guide* guide, const float* params,
                                 const float* adam_m, const float* adam_v,
                                 int64_t step);
/* Also resets the optimizer state and marks the guide usable by renders. */
gbrt_status gbrt_guide_set_weights(gbrt_guide* guide, const float* weights,
                                   size_t n);
/* Host arrays: inputs n x GBRT_GUIDE_INPUT -> mixtures n x GBRT_GUIDE_OUTPUT. */
gbrt_status gbrt_guide_eval(gbrt_guide* guide, const float* inputs, size_t n,
                            float* mixtures);
/* Gradient of the loss over n host samples (n x GBRT_GUIDE_SAMPLE) into grad
 * (GBRT_GUIDE_PARAMS floats); the weights are not changed. */
gbrt_status gbrt_guide_gradient(gbrt_guide* guide, const float* samples,
                                size_t n, float* grad, float* loss);
/* One Adam step (beta 0.9 / 0.999) on n host samples. */
gbrt_status gbrt_guide_train_step(gbrt_guide* guide, const float* samples,
                                  size_t n, float learning_rate, float* loss);

typedef struct gbrt_guide_params {
  float guide_fraction;   /* probability of sampling the guide at a
                             non-specular vertex (one-sample MIS), e.g. 0.5 */
  int32_t passes;         /* passes of x_samples * y_samples per pixel (of
                             late_pass_samples after training, when set);
                             0 = until time_budget_ms is spent */
  int32_t train_passes;   /* the first train_passes passes record samples and
                             are each followed by steps_per_pass Adam steps */
  int32_t steps_per_pass;
  int32_t batch_samples;  /* training samples per step, e.g. 2^18 */
  float learning_rate;    /* e.g. 1e-2 */
  float time_budget_ms;   /* > 0 with passes = 0: equal-time rendering */
  int32_t guide_depth;    /* guide (and train on) path vertices i < guide_depth
                             only (vertex 0 is the camera ray's hit); 0 = all */
  int32_t flags;          /* gbrt_guide_flags */
  int32_t warmup_steps;   /* while training, passes sample the BSDF only until
                             this many Adam steps are done (0: guide from the
                             pass after the first step) */
  int32_t late_pass_samples; /* samples per pixel of every pass after the last
                             training pass (of every pass when the render does
                             not train), as late_pass_samples x 1 jittered
                             strata; 0 = x_samples * y_samples like the
                             training passes. Larger passes keep the GPU full
                             once the guide no longer changes. */
} gbrt_guide_params;

typedef enum gbrt_guide_flags {
  /* While a guide trains, passes are combined with weights inversely proportional
   * to their relative squared deviation from the mean of the earlier passes
   * (the first, unguided pass only seeds that mean), so that the noisy
   * passes of an untrained network weigh little. This flag averages all
   * passes with equal weights instead. Renders that do not train a guide
   * always average equally. */
  GBRT_GUIDE_EQUAL_WEIGHTS = 1,
  /* Training samples weighted by their share of their pixel's value relative
   * to sqrt(pixel^2 + 0.01) instead of by their radiance alone. */
  GBRT_GUIDE_PIXEL_RELATIVE = 2,
  /* The guide learns the product of the BSDF, the incident radiance and the
   * cosine (the radiance each sampled direction reflects towards wo) instead
   * of the incident radiance times the cosine: the two differ at glossy
   * vertices, where the product follows the lobe. */
  GBRT_GUIDE_PRODUCT = 4,
  /* The Adam steps after a training pass run on a second stream of the
   * context while the next pass renders: pass p samples the weights left by
   * the steps after pass p - 2 (one pass later than without the flag), so
   * that training and rendering overlap on the GPU. The sample buffers and
   * the weight snapshots are double-buffered; the call returns after all of
   * its steps, with the guide's weights those of the last step. */
  GBRT_GUIDE_ASYNC_TRAINING = 8
} gbrt_guide_flags;

typedef struct gbrt_guide_stats {
  int32_t passes;
  int32_t train_steps;
  uint64_t paths;
  uint64_t train_samples;
  uint64_t extension_rays;
  uint64_t shadow_rays;
  uint64_t nonfinite;
  double total_ms;        /* device time of the whole call, training included */
  double train_ms;
  float last_loss;
  int32_t pad;
  /* With GBRT_RENDER_TIME_KERNELS: device time of the network's inference
   * (input preparation included) and its launches; always: the rows (path
   * vertices) the network evaluated. */
  double infer_ms;
  uint64_t infer_launches;
  uint64_t infer_rows;
} gbrt_guide_stats;

/* Renders with the physical estimator (params->semantics must be
 * GBRT_SEM_PHYSICAL) in passes, the film (host, H x W x 3 BGR) being the
 * mean over the passes. A non-specular vertex samples the guide with
 * probability guide_fraction once the guide is trained or given weights, and
 * the BSDF otherwise; both densities enter the path weight and the MIS
 * weights of emission and next-event estimation, so the estimator stays
 * unbiased whatever the network predicts. guide = NULL (or guide_fraction 0)
 * renders the same passes with BSDF sampling only. */
gbrt_status gbrt_render_guided(gbrt_scene* scene, const gbrt_camera* camera,
                               const gbrt_render_params* params,
                               gbrt_guide* guide, const gbrt_guide_params* gp,
                               float* film_bgr, gbrt_guide_stats* stats);

/* ---- Markov-chain renderers over the primary sample space: the renderer's
 *      MetropolisRenderer (src/metropolisrenderer.cpp:56-201) and
 *      EnergyRedistributionRenderer (src/energyredistributionrenderer.cpp:
 *      38-135), with MetropolisSample's mutations
 *      (src/metropolissample.cpp:33-121). Reference semantics only. A sample
 *      is a vector of 3 + 5 max_depth numbers in [0, 1]: camera position
 *      over the image (0, 1), path length (2), direction sample i (3 + 2i,
 *      4 + 2i), light sample k (3 + 2D + 3k, +1) and light choice (+2).
 *      The chains run in parallel, one per path of a wavefront, and each
 *      iteration traces every chain's proposal with the same extend / shade
 *      / shadow kernels as gbrt_render. ---- */
typedef struct gbrt_mlt_params {
  int32_t mutations;        /* --met-mutations: mutations per pixel (16)      */
  int32_t bootstrap;        /* --met-bootstrap: bootstrap samples (10000)     */
  float large_step_prob;    /* --met-large-step-prob (0.1)                    */
  float termination_prob;   /* --met-termination-prob (0.5)                   */
  int64_t chains;           /* chains run in parallel (the renderer: its
                               OpenMP threads); 0 = mutations x pixels / 16
                               within [4096, 2^20]; at most mutations x
                               pixels                                         */
} gbrt_mlt_params;

typedef struct gbrt_erpt_params {
  int32_t mutations;        /* --erpt-mutations: mutations per chain (100)    */
  int32_t x_samples;        /* --erpt-x-samples (2)                           */
  int32_t y_samples;        /* --erpt-y-samples (2)                           */
  int32_t pad;
  int64_t batch_chains;     /* chains per wavefront; 0 = 2^22                 */
} gbrt_erpt_params;

typedef struct gbrt_chain_stats {
  uint64_t paths;           /* paths traced (bootstrap / initial + proposals) */
  uint64_t extension_rays, shadow_rays, nonfinite;
  uint64_t chains;          /* Markov chains run                              */
  uint64_t mutations;       /* proposals made                                 */
  uint64_t accepted;        /* proposals accepted                             */
  double normaliser;        /* MLT: b, the mean bootstrap luminance;
                               ERPT: ed, the energy of one deposit            */
  double render_ms;         /* device time                                    */
  uint64_t kernel_launches;
} gbrt_chain_stats;

/* MetropolisRenderer::render. params supplies seed, max_depth (MAX_DEPTH)
 * and semantics (GBRT_SEM_REFERENCE); the film (host, H x W x 3 BGR) is
 * overwritten. Each chain starts from a bootstrap sample drawn in proportion
 * to its luminance (systematic resampling over the chains; with one chain,
 * the renderer's own choice) and makes mutations x pixels / chains
 * mutations, depositing the current and the proposed sample with weights
 * 1 - a and a. */
gbrt_status gbrt_render_mlt(gbrt_scene* scene, const gbrt_camera* camera,
                            const gbrt_render_params* params,
                            const gbrt_mlt_params* mp, float* film_bgr,
                            gbrt_chain_stats* stats);
/* EnergyRedistributionRenderer::render: ed from one path per pixel corner
 * (termination probability 0.1), then per pixel x_samples x y_samples
 * jittered initial samples, each starting (int)(u + |c| / (mutations ed))
 * chains of `mutations` small steps that deposit |c| ed / (|c| chains)
 * per step. The film is overwritten. */
gbrt_status gbrt_render_erpt(gbrt_scene* scene, const gbrt_camera* camera,
                             const gbrt_render_params* params,
                             const gbrt_erpt_params* ep, float* film_bgr,
                             gbrt_chain_stats* stats);

/* ---- scene files (SceneGrammar::parse + resolveVars + buildScene,
 *      src/sceneparser.cpp:36-156, src/sceneast.cpp:673-747,
 *      src/objreader.cpp:142-366) --------------------------------------- */
typedef struct gbrt_parsed_scene gbrt_parsed_scene;
/* Parses a scene file (the renderer's scene language) with its OBJ/MTL files
 * and its environment map (Radiance .hdr or .pfm). Pure host code. */
gbrt_status gbrt_parse_scene_file(const char* path, gbrt_parsed_scene** out,
                                  char* err, int32_t err_len);
gbrt_status gbrt_parse_scene_string(const char* text, const char* base_dir,
                                    gbrt_parsed_scene** out, char* err,
                                    int32_t err_len);
/* Borrowed views, valid until gbrt_parsed_scene_free. has_camera is 0 when
 * the file defines no variable named "camera". */
gbrt_status gbrt_parsed_scene_desc(const gbrt_parsed_scene* ps,
                                   gbrt_scene_desc* desc, gbrt_camera* camera,
                                   int32_t* has_camera);
void gbrt_parsed_scene_free(gbrt_parsed_scene* ps);

/* Image reader for environment and texture images: Radiance RGBE (.hdr),
 * PFM, PPM (samples 0..maxval), PNG and sequential JPEG (both recognised by
 * their signatures; 8-bit samples 0..255 as cv::imread(IMREAD_COLOR) gives
 * them). Returns
 * H x W x 3 float BGR in a buffer the caller frees with gbrt_free. (Replaces
 * cv::imread in src/environmentmap.cpp:20-33 and
 * src/texturematerial.cpp:48-60.) */
gbrt_status gbrt_read_hdr(const char* path, float** texels_bgr,
                          int32_t* width, int32_t* height);
void gbrt_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* GBRT_H */
