"""ctypes mirror of include/gbrt.h (the C ABI of the GB300 path tracer).

The structures here must match the header field for field; tests check the
sizes against the C compiler's view of the same header.
"""
import ctypes as C

F3 = C.c_float * 3


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("kd", F3), ("ks", F3), ("exponent", C.c_float),
                ("ior", C.c_float), ("coefficient", C.c_float), ("texture", C.c_int32)]


class Texture(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("texels", C.POINTER(C.c_float))]


class Quad(C.Structure):
    _fields_ = [("p", F3 * 4), ("material", C.c_int32)]


class Sphere(C.Structure):
    _fields_ = [("center", F3), ("radius", C.c_float), ("material", C.c_int32)]


class Plane(C.Structure):
    _fields_ = [("plane", C.c_float * 4), ("material", C.c_int32)]


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("origin", F3), ("u", F3), ("v", F3), ("intensity", F3)]


class EnvMap(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("mapping", C.c_int32),
                ("texels", C.POINTER(C.c_float))]


class CsgNode(C.Structure):
    _fields_ = [("op", C.c_int32), ("left", C.c_int32), ("right", C.c_int32), ("a", F3), ("b", F3),
                ("material", C.c_int32)]


class Mesh(C.Structure):
    _fields_ = [("tri_pos", C.POINTER(C.c_float)), ("tri_nrm", C.POINTER(C.c_float)),
                ("tri_mat", C.POINTER(C.c_int32)), ("n_tri", C.c_int64)]


class Instance(C.Structure):
    _fields_ = [("transform", C.c_float * 12), ("mesh", C.c_int32), ("pad", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("materials", C.POINTER(Material)), ("n_materials", C.c_int32),
                ("tri_pos", C.POINTER(C.c_float)), ("tri_nrm", C.POINTER(C.c_float)),
                ("tri_uv", C.POINTER(C.c_float)), ("tri_mat", C.POINTER(C.c_int32)),
                ("n_tri", C.c_int64),
                ("quads", C.POINTER(Quad)), ("n_quads", C.c_int32),
                ("spheres", C.POINTER(Sphere)), ("n_spheres", C.c_int32),
                ("planes", C.POINTER(Plane)), ("n_planes", C.c_int32),
                ("lights", C.POINTER(Light)), ("n_lights", C.c_int32),
                ("env", C.POINTER(EnvMap)), ("flags", C.c_int32),
                ("textures", C.POINTER(Texture)), ("n_textures", C.c_int32),
                ("csg_nodes", C.POINTER(CsgNode)), ("n_csg_nodes", C.c_int32),
                ("csg_roots", C.POINTER(C.c_int32)), ("n_csg", C.c_int32),
                ("meshes", C.POINTER(Mesh)), ("n_meshes", C.c_int32),
                ("instances", C.POINTER(Instance)), ("n_instances", C.c_int32),
                ("list_rank", C.POINTER(C.c_int32))]


class Camera(C.Structure):
    _fields_ = [("eye", F3), ("look_at", F3), ("up", F3), ("fov", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("x_samples", C.c_int32), ("y_samples", C.c_int32),
                ("termination_prob", C.c_float), ("max_depth", C.c_int32),
                ("seed", C.c_uint64), ("semantics", C.c_int32), ("batch_paths", C.c_int32),
                ("flags", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64),
                ("shadow_rays", C.c_uint64), ("nonfinite", C.c_uint64),
                ("render_ms", C.c_double), ("kernel_launches", C.c_uint64),
                ("extend_ms", C.c_double), ("shade_ms", C.c_double), ("shadow_ms", C.c_double),
                ("extend_launches", C.c_uint64), ("shade_launches", C.c_uint64),
                ("shadow_launches", C.c_uint64),
                ("nodes_closest", C.c_uint64), ("prims_closest", C.c_uint64),
                ("nodes_any", C.c_uint64), ("prims_any", C.c_uint64)]


class BatchJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", Camera), ("params", RenderParams), ("film", C.c_void_p)]


class BatchSchedule(C.Structure):
    _fields_ = [("wavefront_paths", C.c_int64), ("pipelines", C.c_int32), ("trace_block", C.c_int32),
                ("shade_block", C.c_int32), ("pad", C.c_int32)]


class BatchStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nonfinite", C.c_uint64), ("wall_ms", C.c_double), ("streams", C.c_int32), ("pad", C.c_int32),
                ("batch_paths", C.c_int64), ("device_ms", C.c_double),
                ("kernel_launches", C.c_uint64)]


class MltParams(C.Structure):
    _fields_ = [("mutations", C.c_int32), ("bootstrap", C.c_int32), ("large_step_prob", C.c_float),
                ("termination_prob", C.c_float), ("chains", C.c_int64)]


class ErptParams(C.Structure):
    _fields_ = [("mutations", C.c_int32), ("x_samples", C.c_int32), ("y_samples", C.c_int32), ("pad", C.c_int32),
                ("batch_chains", C.c_int64)]


class ChainStats(C.Structure):
    _fields_ = [("paths", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nonfinite", C.c_uint64), ("chains", C.c_uint64), ("mutations", C.c_uint64),
                ("accepted", C.c_uint64), ("normaliser", C.c_double), ("render_ms", C.c_double),
                ("kernel_launches", C.c_uint64)]


class GuideParams(C.Structure):
    _fields_ = [("guide_fraction", C.c_float), ("passes", C.c_int32), ("train_passes", C.c_int32),
                ("steps_per_pass", C.c_int32), ("batch_samples", C.c_int32), ("learning_rate", C.c_float),
                ("time_budget_ms", C.c_float), ("guide_depth", C.c_int32), ("flags", C.c_int32),
                ("warmup_steps", C.c_int32), ("late_pass_samples", C.c_int32)]


class GuideStats(C.Structure):
    _fields_ = [("passes", C.c_int32), ("train_steps", C.c_int32), ("paths", C.c_uint64),
                ("train_samples", C.c_uint64), ("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64),
                ("nonfinite", C.c_uint64), ("total_ms", C.c_double), ("train_ms", C.c_double),
                ("last_loss", C.c_float), ("pad", C.c_int32), ("infer_ms", C.c_double),
                ("infer_launches", C.c_uint64), ("infer_rows", C.c_uint64)]


class Ray(C.Structure):
    _fields_ = [("org", F3), ("tmin", C.c_float), ("dir", F3), ("tmax", C.c_float)]


class Hit(C.Structure):
    _fields_ = [("t", C.c_float), ("prim", C.c_int32), ("u", C.c_float), ("v", C.c_float)]


# gbrt_status
OK, ERR_INVALID_ARG, ERR_OOM, ERR_CUDA, ERR_CANCELLED, ERR_TIMEOUT, ERR_NUMERIC, ERR_PARSE, \
    ERR_IO, ERR_UNSUPPORTED = range(10)
STATUS_NAMES = {0: "OK", 1: "INVALID_ARG", 2: "OOM", 3: "CUDA", 4: "CANCELLED", 5: "TIMEOUT",
                6: "NUMERIC", 7: "PARSE", 8: "IO", 9: "UNSUPPORTED"}

# gbrt_material_type
MAT_DARK, MAT_DIFFUSE, MAT_MIRROR, MAT_PHONG, MAT_BLINN, MAT_TRANSPARENT, MAT_TEXTURE = range(7)
# gbrt_light_type
LIGHT_AREA, LIGHT_POINT, LIGHT_ENV, LIGHT_BLACK, LIGHT_CONE = range(5)
# gbrt_env_mapping
ENV_ANGULAR, ENV_LATLONG = range(2)
# gbrt_semantics
SEM_REFERENCE, SEM_PHYSICAL = range(2)
# gbrt_scene_flags / gbrt_render_flags
SCENE_WATERTIGHT, SCENE_GPU_BUILD, SCENE_ENV_UNIFORM, SCENE_LIST_ORDER = 1, 2, 4, 8
RENDER_TIME_KERNELS, RENDER_COUNT_TRAVERSAL = 1, 2
NOALLOC_MAX_BATCH = 65536
# gbrt_fault (host-side fault injection for the failure-path tests)
FAULT_NONE, FAULT_ALLOC, FAULT_NAN, FAULT_SMALL_STACK, FAULT_GUIDE_WAIT = 0, 1, 2, 3, 4
GUIDE_PARAMS, GUIDE_INPUT, GUIDE_OUTPUT, GUIDE_SAMPLE = 24064, 9, 40, 13
CSG_SPHERE, CSG_BOX, CSG_ISECT, CSG_UNION, CSG_DIFF, CSG_XOR = range(6)
CSG_MAX_LEAVES = 8
GUIDE_EQUAL_WEIGHTS, GUIDE_PIXEL_RELATIVE, GUIDE_PRODUCT, GUIDE_ASYNC_TRAINING = 1, 2, 4, 8

P = C.c_void_p

# (name, restype, argtypes) of every exported entry point declared in gbrt.h.
SIGNATURES = [
    ("gbrt_abi_version", C.c_int32, []),
    ("gbrt_last_error", C.c_char_p, [P]),
    ("gbrt_ctx_create", C.c_int, [C.c_int32, C.POINTER(P)]),
    ("gbrt_ctx_destroy", C.c_int, [P]),
    ("gbrt_scene_create", C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(P)]),
    ("gbrt_scene_destroy", C.c_int, [P]),
    ("gbrt_scene_info", C.c_int, [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("gbrt_scene_bounds", C.c_int, [P, C.POINTER(C.c_float)]),
    ("gbrt_trace_closest", C.c_int, [P, P, C.c_int64, P]),
    ("gbrt_trace_any", C.c_int, [P, P, P, C.c_int64, P]),
    ("gbrt_trace_closest_device", C.c_int, [P, P, C.c_int64, P, P]),
    ("gbrt_trace_any_device", C.c_int, [P, P, P, C.c_int64, P, P]),
    ("gbrt_render", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), P, P, P, P,
                              C.POINTER(Stats)]),
    ("gbrt_render_device", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), P, P, P,
                                     C.POINTER(Stats)]),
    ("gbrt_render_device_noalloc", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), P, P, P,
                                             C.POINTER(Stats)]),
    ("gbrt_tonemap", C.c_int, [P, C.c_int32, C.c_int32, C.c_float, P]),
    ("gbrt_tonemap_device", C.c_int, [P, P, C.c_int32, C.c_int32, C.c_float, P, P]),
    ("gbrt_write_image", C.c_int, [C.c_char_p, P, C.c_int32, C.c_int32, C.c_float]),
    ("gbrt_render_batch", C.c_int, [P, C.POINTER(BatchJob), C.c_int32, C.c_int32, C.c_int64,
                                    C.POINTER(C.c_double), C.POINTER(BatchStats)]),
    ("gbrt_batch_autotune", C.c_int, [P, C.POINTER(BatchJob), C.c_int32, C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int64)]),
    ("gbrt_render_batch_fused", C.c_int, [P, C.POINTER(BatchJob), C.c_int32, C.POINTER(BatchSchedule),
                                          C.POINTER(C.c_double), C.POINTER(BatchStats)]),
    ("gbrt_batch_autotune_fused", C.c_int, [P, C.POINTER(BatchJob), C.c_int32, C.POINTER(BatchSchedule)]),
    ("gbrt_render_passes", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), C.c_int32, C.c_int32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Stats)]),
    ("gbrt_guide_get_state", C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    ("gbrt_guide_set_state", C.c_int, [P, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]),
    ("gbrt_ctx_trim", C.c_int, [P, C.POINTER(C.c_uint64)]),
    ("gbrt_debug_fault", C.c_int, [P, C.c_int32, C.c_int64]),
    ("gbrt_render_mlt", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), C.POINTER(MltParams), P,
                                  C.POINTER(ChainStats)]),
    ("gbrt_render_erpt", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), C.POINTER(ErptParams), P,
                                   C.POINTER(ChainStats)]),
    ("gbrt_guide_create", C.c_int, [P, C.POINTER(C.c_float), C.c_uint64, C.POINTER(P)]),
    ("gbrt_guide_destroy", C.c_int, [P]),
    ("gbrt_guide_get_weights", C.c_int, [P, P, C.c_size_t]),
    ("gbrt_guide_set_weights", C.c_int, [P, P, C.c_size_t]),
    ("gbrt_guide_eval", C.c_int, [P, P, C.c_size_t, P]),
    ("gbrt_guide_gradient", C.c_int, [P, P, C.c_size_t, P, C.POINTER(C.c_float)]),
    ("gbrt_guide_train_step", C.c_int, [P, P, C.c_size_t, C.c_float, C.POINTER(C.c_float)]),
    ("gbrt_render_guided", C.c_int, [P, C.POINTER(Camera), C.POINTER(RenderParams), P, C.POINTER(GuideParams),
                                     P, C.POINTER(GuideStats)]),
    ("gbrt_parse_scene_file", C.c_int, [C.c_char_p, C.POINTER(P), C.c_char_p, C.c_int32]),
    ("gbrt_parse_scene_string", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(P), C.c_char_p, C.c_int32]),
    ("gbrt_parsed_scene_desc", C.c_int, [P, C.POINTER(SceneDesc), C.POINTER(Camera),
                                         C.POINTER(C.c_int32)]),
    ("gbrt_parsed_scene_free", None, [P]),
    ("gbrt_read_hdr", C.c_int, [C.c_char_p, C.POINTER(C.POINTER(C.c_float)), C.POINTER(C.c_int32),
                                C.POINTER(C.c_int32)]),
    ("gbrt_free", None, [P]),
]
