"""Scene files in the renderer's scene language (src/sceneparser.cpp:36-125).

load_scene(path)          parse with the library's parser -> SceneData
load_scene_string(text)   same, from a string
write_scene(data, path)   write SceneData in the scene language (meshes as OBJ)
write_obj(path, tri_pos, tri_nrm=None)
"""
import ctypes as C
import os

import numpy as np

from . import _abi, check, lib
from .scene import SceneData


def _from_parsed(ps):
    d = _abi.SceneDesc()
    cam = _abi.Camera()
    has = C.c_int32()
    check(lib().gbrt_parsed_scene_desc(ps, C.byref(d), C.byref(cam), C.byref(has)))
    s = SceneData()
    for i in range(d.n_materials):
        m = d.materials[i]
        s.materials.append(dict(type=m.type, kd=tuple(m.kd), ks=tuple(m.ks), exponent=m.exponent, ior=m.ior,
                                coefficient=m.coefficient, texture=m.texture))
    for i in range(d.n_textures):
        t = d.textures[i]
        s.textures.append(np.ctypeslib.as_array(t.texels, shape=(t.height, t.width, 3)).copy())
    for i in range(d.n_csg_nodes):
        g = d.csg_nodes[i]
        s.csg_nodes.append((g.op, g.left, g.right, tuple(g.a), tuple(g.b), g.material))
    s.csg_roots = [d.csg_roots[i] for i in range(d.n_csg)]
    if d.n_tri:
        s.tri_pos = np.ctypeslib.as_array(d.tri_pos, shape=(d.n_tri, 9)).copy()
        if d.tri_nrm:
            s.tri_nrm = np.ctypeslib.as_array(d.tri_nrm, shape=(d.n_tri, 9)).copy()
        if d.tri_uv:
            s.tri_uv = np.ctypeslib.as_array(d.tri_uv, shape=(d.n_tri, 6)).copy()
        s.tri_mat = np.ctypeslib.as_array(d.tri_mat, shape=(d.n_tri,)).copy()
    for i in range(d.n_meshes):
        m = d.meshes[i]
        s.add_mesh(np.ctypeslib.as_array(m.tri_pos, shape=(m.n_tri, 9)).copy(),
                   np.ctypeslib.as_array(m.tri_nrm, shape=(m.n_tri, 9)).copy() if m.tri_nrm else None,
                   np.ctypeslib.as_array(m.tri_mat, shape=(m.n_tri,)).copy())
    for i in range(d.n_instances):
        g = d.instances[i]
        s.add_instance(np.array(list(g.transform), np.float32).reshape(3, 4), g.mesh)
    for i in range(d.n_quads):
        q = d.quads[i]
        s.quads.append(tuple(tuple(q.p[k]) for k in range(4)) + (q.material,))
    for i in range(d.n_spheres):
        q = d.spheres[i]
        s.spheres.append((tuple(q.center), q.radius, q.material))
    for i in range(d.n_planes):
        q = d.planes[i]
        s.planes.append((tuple(q.plane), q.material))
    for i in range(d.n_lights):
        L = d.lights[i]
        s.lights.append(dict(type=L.type, origin=tuple(L.origin), u=tuple(L.u), v=tuple(L.v),
                             intensity=tuple(L.intensity)))
    if d.list_rank:
        s.list_rank = np.ctypeslib.as_array(d.list_rank, shape=(s.n_prims(),)).copy()
    if d.env:
        e = d.env.contents
        s.env = np.ctypeslib.as_array(e.texels, shape=(e.height, e.width, 3)).copy()
        s.env_mapping = e.mapping
    if has.value:
        s.camera = dict(eye=tuple(cam.eye), look_at=tuple(cam.look_at), up=tuple(cam.up), fov=cam.fov,
                        width=cam.width, height=cam.height)
    return s


def _parse(fn, *args):
    ps = C.c_void_p()
    err = C.create_string_buffer(1024)
    st = fn(*args, C.byref(ps), err, len(err))
    if st != _abi.OK:
        from . import GbrtError
        raise GbrtError(st, err.value.decode())
    try:
        return _from_parsed(ps)
    finally:
        lib().gbrt_parsed_scene_free(ps)


def load_scene(path):
    return _parse(lib().gbrt_parse_scene_file, os.fsencode(path))


def load_scene_string(text, base_dir=""):
    return _parse(lib().gbrt_parse_scene_string, text.encode(), os.fsencode(base_dir))


def read_hdr(path):
    """Radiance .hdr (or .pfm) -> (H, W, 3) float32 BGR."""
    p = C.POINTER(C.c_float)()
    w, h = C.c_int32(), C.c_int32()
    check(lib().gbrt_read_hdr(os.fsencode(path), C.byref(p), C.byref(w), C.byref(h)))
    try:
        return np.ctypeslib.as_array(p, shape=(h.value, w.value, 3)).copy()
    finally:
        lib().gbrt_free(p)


def _v(x):
    return "[" + " ".join(repr(float(c)) for c in x) + "]"


def _rgb(bgr):
    return _v((bgr[2], bgr[1], bgr[0]))


def _material(m):
    t = m["type"]
    if t == _abi.MAT_DIFFUSE:
        return "diffuse(%s)" % _rgb(m["kd"])
    if t == _abi.MAT_PHONG:
        return "phong(%s, %s, %r)" % (_rgb(m["kd"]), _rgb(m["ks"]), float(m["exponent"]))
    if t == _abi.MAT_BLINN:
        return "blinn(%s, %s, %r)" % (_rgb(m["kd"]), _rgb(m["ks"]), float(m["exponent"]))
    if t == _abi.MAT_MIRROR:
        return "mirror(%r)" % float(m.get("coefficient", 1.0))
    if t == _abi.MAT_TRANSPARENT:
        return "refractive(%r)" % float(m["ior"])
    return "diffuse([0 0 0])"


def write_obj(path, tri_pos, tri_nrm=None):
    """Triangle soup as OBJ (one vertex per corner), vn lines when normals are given."""
    P = np.asarray(tri_pos, np.float32).reshape(-1, 3)
    n = len(P)
    with open(path, "w") as f:
        np.savetxt(f, P, fmt="v %.9g %.9g %.9g")
        if tri_nrm is not None:
            np.savetxt(f, np.asarray(tri_nrm, np.float32).reshape(-1, 3), fmt="vn %.9g %.9g %.9g")
            idx = np.arange(1, n + 1).reshape(-1, 3)
            np.savetxt(f, np.repeat(idx, 2, axis=1), fmt="f %d//%d %d//%d %d//%d")
        else:
            np.savetxt(f, np.arange(1, n + 1).reshape(-1, 3), fmt="f %d %d %d")


def write_scene(s: SceneData, path, env_file=None):
    """Writes s in the scene language. Meshes go to <path>.obj (one obj() per
    material); the environment image, if any, must already exist as env_file."""
    lines = []
    for i, m in enumerate(s.materials):
        lines.append("m%d = %s;" % (i, _material(m)))
    items = []
    base = os.path.splitext(path)[0]
    if s.n_tri():
        mats = np.zeros(s.n_tri(), np.int32) if s.tri_mat is None else s.tri_mat
        for m in np.unique(mats):
            sel = mats == m
            objp = "%s_m%d.obj" % (base, m)
            write_obj(objp, s.tri_pos[sel], None if s.tri_nrm is None else s.tri_nrm[sel])
            items.append('obj("%s", m%d)' % (os.path.basename(objp), m))
    for q in s.quads:
        items.append("quad(%s, %s, %s, %s, m%d)" % (_v(q[0]), _v(q[1]), _v(q[2]), _v(q[3]), q[4]))
    for c, r, m in s.spheres:
        items.append("sphere(%s, %r, m%d)" % (_v(c), float(r), m))
    for p, m in s.planes:
        items.append("plane(%s, m%d)" % (_v(p), m))
    lines.append("intersectable = intersectables {\n  " + "\n  ".join(items) + "\n};")
    ls = []
    for L in s.lights:
        if L["type"] == _abi.LIGHT_AREA:
            ls.append("arealight(%s, %s, %s, %s)" % (_v(L["origin"]), _v(L["u"]), _v(L["v"]), _rgb(L["intensity"])))
        elif L["type"] == _abi.LIGHT_POINT:
            ls.append("pointlight(%s, %s)" % (_v(L["origin"]), _rgb(L["intensity"])))
        elif L["type"] == _abi.LIGHT_ENV:
            mapping = ', "latlong"' if s.env_mapping == _abi.ENV_LATLONG else ""
            ls.append('environmentmap("%s", %s%s)' % (env_file or "missing.hdr", _rgb(L["intensity"]), mapping))
    lines.append("lights = lights {\n  " + "\n  ".join(ls) + "\n};")
    if s.camera:
        c = s.camera
        lines.append("camera = camera(%s, %s, %s, %r, %d, %d);" % (_v(c["eye"]), _v(c["look_at"]), _v(c["up"]),
                                                                 float(c["fov"]), c["width"], c["height"]))
    with open(path, "w") as f:
        f.write("// written by renderer_gb300.scenefile\n" + "\n".join(lines) + "\n")
    return path


def write_hdr(path, bgr):
    """Radiance RGBE writer (flat, non-RLE rows) for H x W x 3 BGR floats."""
    img = np.asarray(bgr, np.float64)[..., ::-1]
    H, W, _ = img.shape
    m = img.max(-1)
    e = np.where(m > 1e-32, np.floor(np.log2(np.maximum(m, 1e-32))) + 1, 0)
    scale = np.where(m > 1e-32, 256.0 / np.exp2(e), 0)
    rgbe = np.zeros((H, W, 4), np.uint8)
    rgbe[..., :3] = np.clip(np.floor(img * scale[..., None]), 0, 255)
    rgbe[..., 3] = np.where(m > 1e-32, e + 128, 0)
    with open(path, "wb") as f:
        f.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y %d +X %d\n" % (H, W))
        f.write(rgbe.tobytes())
