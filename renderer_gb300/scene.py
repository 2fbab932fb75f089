"""Scene description held in numpy arrays, and its gbrt_scene_desc view.

A SceneData mirrors what the renderer's scene builder produces
(src/sceneast.cpp:673-695): materials, geometry (triangles, quads, spheres,
planes), the ordered light list and at most one environment image. Spectra are
BGR, as in the renderer's cv::Vec3f.
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _abi


def _f3(v):
    return _abi.F3(*[float(x) for x in v])


@dataclass
class SceneData:
    materials: List[dict] = field(default_factory=list)
    tri_pos: Optional[np.ndarray] = None   # (N, 9) float32
    tri_nrm: Optional[np.ndarray] = None   # (N, 9) float32 or None
    tri_uv: Optional[np.ndarray] = None    # (N, 6) float32 or None
    tri_mat: Optional[np.ndarray] = None   # (N,) int32 or None (all material 0)
    quads: List[tuple] = field(default_factory=list)     # (p1, p2, p3, p4, material)
    spheres: List[tuple] = field(default_factory=list)   # (center, radius, material)
    planes: List[tuple] = field(default_factory=list)    # (plane4, material)
    lights: List[dict] = field(default_factory=list)     # {"type", "origin", "u", "v", "intensity"}
    env: Optional[np.ndarray] = None       # (H, W, 3) float32 BGR
    env_mapping: int = _abi.ENV_ANGULAR
    camera: Optional[dict] = None          # {"eye", "look_at", "up", "fov", "width", "height"}
    flags: int = 0                         # gbrt_scene_flags
    textures: List[np.ndarray] = field(default_factory=list)  # (H, W, 3) float32 BGR each
    csg_nodes: List[tuple] = field(default_factory=list)  # (op, left, right, a3, b3, material)
    csg_roots: List[int] = field(default_factory=list)
    meshes: List[dict] = field(default_factory=list)     # {"pos" (N, 9), "nrm" (N, 9) or None, "mat" (N,) or None}
    instances: List[tuple] = field(default_factory=list)  # (3x4 object->world transform, mesh index)
    list_rank: Optional[np.ndarray] = None  # (n_prims,) int32: position in the root list, or None

    # ------------------------------------------------------------ building
    def add_material(self, type, kd=(0, 0, 0), ks=(0, 0, 0), exponent=0.0, ior=1.0, coefficient=1.0, texture=-1):
        self.materials.append(dict(type=type, kd=tuple(kd), ks=tuple(ks), exponent=float(exponent),
                                   ior=float(ior), coefficient=float(coefficient), texture=int(texture)))
        return len(self.materials) - 1

    def add_texture(self, texels):
        """A (H, W, 3) BGR texture; returns its index."""
        self.textures.append(np.ascontiguousarray(texels, np.float32))
        return len(self.textures) - 1

    def n_tri(self):
        return 0 if self.tri_pos is None else int(self.tri_pos.shape[0])

    def n_prims(self):
        return len(self.lights) + self.n_tri() + len(self.quads) + len(self.spheres) + len(self.planes) + \
            len(self.csg_roots) + len(self.instances)

    def csg_leaf(self, op, a, b, material):
        """A sphere (a = centre, b = (r, 0, 0)) or box (a = min, b = max) node."""
        self.csg_nodes.append((op, -1, -1, tuple(a), tuple(b), int(material)))
        return len(self.csg_nodes) - 1

    def csg_op(self, op, left, right):
        self.csg_nodes.append((op, int(left), int(right), (0, 0, 0), (0, 0, 0), -1))
        return len(self.csg_nodes) - 1

    def add_mesh(self, pos, nrm=None, mat=None):
        """A triangle mesh for instancing; returns its index."""
        self.meshes.append(dict(pos=np.ascontiguousarray(pos, np.float32).reshape(-1, 9),
                                nrm=None if nrm is None else np.ascontiguousarray(nrm, np.float32).reshape(-1, 9),
                                mat=None if mat is None else np.ascontiguousarray(mat, np.int32).reshape(-1)))
        return len(self.meshes) - 1

    def add_instance(self, transform, mesh):
        """Places mesh with a 3x4 (or 4x4) object-to-world transform."""
        t = np.asarray(transform, np.float64)[:3, :4]
        self.instances.append((t.astype(np.float32), int(mesh)))
        return len(self.instances) - 1

    def add_csg(self, root):
        self.csg_roots.append(int(root))
        return len(self.csg_roots) - 1

    def prim_offsets(self):
        """First primitive id of each type, in the order of include/gbrt.h."""
        o = {"lights": 0}
        o["tri"] = len(self.lights)
        o["quads"] = o["tri"] + self.n_tri()
        o["spheres"] = o["quads"] + len(self.quads)
        o["planes"] = o["spheres"] + len(self.spheres)
        o["csg"] = o["planes"] + len(self.planes)
        o["instances"] = o["csg"] + len(self.csg_roots)
        return o

    # ------------------------------------------------------------ C view
    def to_desc(self):
        """Returns (gbrt_scene_desc, keepalive). keepalive must outlive every use."""
        keep = []
        d = _abi.SceneDesc()
        if self.materials:
            arr = (_abi.Material * len(self.materials))()
            for i, m in enumerate(self.materials):
                arr[i] = _abi.Material(m["type"], _f3(m["kd"]), _f3(m["ks"]), m["exponent"], m["ior"],
                                       m["coefficient"], m.get("texture", -1))
            keep.append(arr)
            d.materials = arr
            d.n_materials = len(self.materials)
        if self.n_tri():
            pos = np.ascontiguousarray(self.tri_pos, dtype=np.float32)
            keep.append(pos)
            d.tri_pos = pos.ctypes.data_as(C.POINTER(C.c_float))
            if self.tri_nrm is not None:
                nrm = np.ascontiguousarray(self.tri_nrm, dtype=np.float32)
                keep.append(nrm)
                d.tri_nrm = nrm.ctypes.data_as(C.POINTER(C.c_float))
            if self.tri_uv is not None:
                uv = np.ascontiguousarray(self.tri_uv, dtype=np.float32)
                keep.append(uv)
                d.tri_uv = uv.ctypes.data_as(C.POINTER(C.c_float))
            if self.tri_mat is not None:
                mat = np.ascontiguousarray(self.tri_mat, dtype=np.int32)
                keep.append(mat)
                d.tri_mat = mat.ctypes.data_as(C.POINTER(C.c_int32))
            d.n_tri = self.n_tri()
        if self.quads:
            arr = (_abi.Quad * len(self.quads))()
            for i, q in enumerate(self.quads):
                arr[i].p = (_abi.F3 * 4)(*[_f3(p) for p in q[:4]])
                arr[i].material = int(q[4])
            keep.append(arr)
            d.quads = arr
            d.n_quads = len(self.quads)
        if self.spheres:
            arr = (_abi.Sphere * len(self.spheres))()
            for i, s in enumerate(self.spheres):
                arr[i] = _abi.Sphere(_f3(s[0]), float(s[1]), int(s[2]))
            keep.append(arr)
            d.spheres = arr
            d.n_spheres = len(self.spheres)
        if self.planes:
            arr = (_abi.Plane * len(self.planes))()
            for i, p in enumerate(self.planes):
                arr[i] = _abi.Plane((C.c_float * 4)(*[float(x) for x in p[0]]), int(p[1]))
            keep.append(arr)
            d.planes = arr
            d.n_planes = len(self.planes)
        if self.lights:
            arr = (_abi.Light * len(self.lights))()
            for i, L in enumerate(self.lights):
                arr[i] = _abi.Light(L["type"], _f3(L.get("origin", (0, 0, 0))), _f3(L.get("u", (0, 0, 0))),
                                    _f3(L.get("v", (0, 0, 0))), _f3(L.get("intensity", (0, 0, 0))))
            keep.append(arr)
            d.lights = arr
            d.n_lights = len(self.lights)
        if self.env is not None:
            tex = np.ascontiguousarray(self.env, dtype=np.float32)
            keep.append(tex)
            e = _abi.EnvMap(tex.shape[1], tex.shape[0], self.env_mapping,
                            tex.ctypes.data_as(C.POINTER(C.c_float)))
            keep.append(e)
            d.env = C.pointer(e)
        d.flags = int(self.flags)
        if self.textures:
            arr = (_abi.Texture * len(self.textures))()
            for i, t in enumerate(self.textures):
                t = np.ascontiguousarray(t, np.float32)
                keep.append(t)
                arr[i] = _abi.Texture(t.shape[1], t.shape[0], t.ctypes.data_as(C.POINTER(C.c_float)))
            keep.append(arr)
            d.textures = arr
            d.n_textures = len(self.textures)
        if self.csg_roots:
            arr = (_abi.CsgNode * len(self.csg_nodes))()
            for i, (op, l, r, a, b, m) in enumerate(self.csg_nodes):
                arr[i] = _abi.CsgNode(op, l, r, _f3(a), _f3(b), m)
            roots = (C.c_int32 * len(self.csg_roots))(*self.csg_roots)
            keep += [arr, roots]
            d.csg_nodes = arr
            d.n_csg_nodes = len(self.csg_nodes)
            d.csg_roots = roots
            d.n_csg = len(self.csg_roots)
        if self.instances:
            marr = (_abi.Mesh * len(self.meshes))()
            for i, m in enumerate(self.meshes):
                keep.append(m["pos"])
                marr[i].tri_pos = m["pos"].ctypes.data_as(C.POINTER(C.c_float))
                if m["nrm"] is not None:
                    keep.append(m["nrm"])
                    marr[i].tri_nrm = m["nrm"].ctypes.data_as(C.POINTER(C.c_float))
                if m["mat"] is not None:
                    keep.append(m["mat"])
                    marr[i].tri_mat = m["mat"].ctypes.data_as(C.POINTER(C.c_int32))
                marr[i].n_tri = len(m["pos"])
            iarr = (_abi.Instance * len(self.instances))()
            for i, (t, mi) in enumerate(self.instances):
                iarr[i].transform = (C.c_float * 12)(*[float(x) for x in np.asarray(t).reshape(-1)])
                iarr[i].mesh = mi
            keep += [marr, iarr]
            d.meshes = marr
            d.n_meshes = len(self.meshes)
            d.instances = iarr
            d.n_instances = len(self.instances)
        if self.list_rank is not None:
            rank = np.ascontiguousarray(self.list_rank, np.int32).reshape(-1)
            if len(rank) != self.n_prims():
                raise ValueError("list_rank needs one entry per primitive")
            keep.append(rank)
            d.list_rank = rank.ctypes.data_as(C.POINTER(C.c_int32))
        return d, keep

    def camera_struct(self, width=None, height=None):
        c = self.camera
        return _abi.Camera(_f3(c["eye"]), _f3(c["look_at"]), _f3(c["up"]), float(c["fov"]),
                           int(width or c["width"]), int(height or c["height"]))


def render_params(x_samples=4, y_samples=4, termination_prob=0.5, max_depth=5, seed=0,
                  semantics=_abi.SEM_REFERENCE, batch_paths=0, flags=0):
    """gbrt_render_params with PerPixelRenderer's defaults (src/perpixelrenderer.cpp:103-112)
    and the renderer's MAX_DEPTH of 5 (src/renderer.h:38)."""
    return _abi.RenderParams(int(x_samples), int(y_samples), float(termination_prob), int(max_depth),
                             int(seed), int(semantics), int(batch_paths), int(flags))
