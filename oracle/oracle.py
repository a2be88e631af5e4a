"""ctypes wrapper of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py use this module as the checker; the product never imports it.
The C restatement it wraps follows shamazmazum/voxvision src/voxtrees/search.c,
geom.c, tree.c and src/voxrnd/renderer.c (file:line cited in oracle.c) and is
pinned to the reference's own compiled sources through tests/golden/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
LIB_FC_PATH = os.path.join(HERE, "_build", "liboracle_fc.so")   # the same with FP contraction on
REF_DIR = os.path.join(HERE, "_ref")

_lib = None
_lib_fc = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "oracle.h"))):
        subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    return LIB_PATH


def render_best_contracted(tree_ptr, state: dict, w: int, h: int, texture: np.ndarray, nthreads=None):
    """render_best by the restatement compiled with floating-point contraction
    on (liboracle_fc.so): what a build with the compiler's default
    contraction draws, for the CPU baseline's comparison only."""
    global _lib_fc
    if _lib_fc is None:
        build()
        if not os.path.exists(LIB_FC_PATH):
            subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
        L = C.CDLL(LIB_FC_PATH)
        L.orc_render_best.argtypes = [C.c_void_p, C.POINTER(OrcCamera), C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_int]
        L.orc_render_best.restype = C.c_int
        _lib_fc = L
    tex = np.ascontiguousarray(texture, dtype=np.uint8)
    out = np.zeros(w * h, np.uint32)
    cnt = np.zeros(3, np.uint64)
    rc = _lib_fc.orc_render_best(tree_ptr, C.byref(camera(state)), w, h, _p(tex), _p(out), _p(cnt),
                                 nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("bad geometry: width must be a multiple of 16 and height of 4")
    return out.reshape(h, w), cnt


class OrcCamera(C.Structure):
    _fields_ = [("kind", C.c_int32), ("position", C.c_float * 3), ("rotation", C.c_float * 4),
                ("mul", C.c_float), ("xsub", C.c_float), ("ysub", C.c_float),
                ("sinphi", C.c_float), ("cosphi", C.c_float), ("k", C.c_float),
                ("rays", C.c_void_p), ("rays_w", C.c_int32)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        vp, sz, fp = C.c_void_p, C.c_size_t, C.c_void_p
        L.orc_set_voxel.argtypes = [C.c_float] * 3
        L.orc_make_tree.argtypes = [fp, sz]; L.orc_make_tree.restype = vp
        L.orc_destroy_tree.argtypes = [vp]
        L.orc_count_nodes.argtypes = [vp]; L.orc_count_nodes.restype = sz
        L.orc_count_stored_dots.argtypes = [vp]; L.orc_count_stored_dots.restype = sz
        L.orc_preorder.argtypes = [vp, vp]; L.orc_preorder.restype = sz
        L.orc_ray_batch.argtypes = [vp, vp, sz, fp, fp, vp, vp, fp, vp, C.c_int]
        L.orc_ball_batch.argtypes = [vp, sz, fp, fp, vp, vp, C.c_int]
        L.orc_screen2world.argtypes = [C.POINTER(OrcCamera), C.c_int, C.c_int, fp]
        L.orc_camera_simple.argtypes = [C.POINTER(OrcCamera), fp, fp, C.c_int, C.c_int, C.c_float]
        L.orc_render_best.argtypes = [vp, C.POINTER(OrcCamera), C.c_int, C.c_int, vp, vp, vp, C.c_int]
        L.orc_render_best.restype = C.c_int
        L.orc_render_quality.argtypes = [vp, C.POINTER(OrcCamera), C.c_int, C.c_int, C.c_uint, vp, vp,
                                         vp, C.c_int]
        L.orc_render_quality.restype = C.c_int
        L.orc_ray_counts_per_ray.argtypes = [vp, sz, fp, fp, vp, C.c_int]
        L.orc_lights_new.restype = vp
        L.orc_lights_free.argtypes = [vp]
        L.orc_lights_ambient.argtypes = [vp, fp]; L.orc_lights_ambient.restype = C.c_int
        L.orc_lights_insert.argtypes = [vp, fp, C.c_float, fp]; L.orc_lights_insert.restype = C.c_int
        L.orc_lights_delete.argtypes = [vp, fp, C.c_float]; L.orc_lights_delete.restype = C.c_int
        L.orc_lights_count.argtypes = [vp]; L.orc_lights_count.restype = C.c_int
        L.orc_lights_get.argtypes = [vp, fp, fp]; L.orc_lights_get.restype = C.c_int
        L.orc_lights_verify.argtypes = [vp]; L.orc_lights_verify.restype = C.c_int
        L.orc_render_lit.argtypes = [vp, C.POINTER(OrcCamera), C.c_int, C.c_int, C.c_uint, vp, vp, vp, C.c_int]
        L.orc_render_lit.restype = C.c_int
        L.orc_dump.argtypes = [vp] * 8; L.orc_dump.restype = sz
        L.orc_from_dump.argtypes = [sz] + [vp] * 7; L.orc_from_dump.restype = vp
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def nthreads_default() -> int:
    return max(1, len(os.sched_getaffinity(0)))


def set_voxel(v=(1.0, 1.0, 1.0)):
    lib().orc_set_voxel(*[float(x) for x in v])


class OracleTree:
    """A reference-layout host tree built (or rebuilt) by the oracle."""

    def __init__(self, ptr):
        self.ptr = ptr

    @classmethod
    def from_voxels(cls, voxels: np.ndarray) -> "OracleTree":
        s = np.ascontiguousarray(voxels, dtype=np.float32).copy()   # build is destructive
        return cls(lib().orc_make_tree(_p(s), s.shape[0]))

    @classmethod
    def from_dump(cls, d: dict) -> "OracleTree":
        n = int(d["flags"].shape[0])
        arrs = [np.ascontiguousarray(d[k]) for k in
                ("flags", "dots_num", "boxes", "centers", "child_mask", "dot_offset", "dots")]
        return cls(lib().orc_from_dump(n, *[_p(a) for a in arrs]))

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.orc_destroy_tree(self.ptr)
            self.ptr = None

    def node_count(self) -> int:
        return int(lib().orc_count_nodes(self.ptr))

    def preorder(self) -> np.ndarray:
        n = self.node_count()
        out = np.zeros(max(n, 1), dtype=np.uint64)
        lib().orc_preorder(self.ptr, _p(out))
        return out[:n]

    def dump(self) -> dict:
        return dump_tree(self.ptr)

    def rays(self, origins, dirs, root=None, nthreads=None):
        return ray_batch(self.ptr, origins, dirs, root=root, nthreads=nthreads)

    def balls(self, centres, radii, nthreads=None):
        return ball_batch(self.ptr, centres, radii, nthreads=nthreads)


def dump_tree(ptr) -> dict:
    L = lib()
    n = int(L.orc_count_nodes(ptr))
    nd = int(L.orc_count_stored_dots(ptr))
    d = dict(flags=np.zeros(n, np.uint32), dots_num=np.zeros(n, np.uint32),
             boxes=np.zeros((n, 6), np.float32), centers=np.zeros((n, 3), np.float32),
             child_mask=np.zeros(n, np.uint8), dot_offset=np.zeros(n, np.uint64),
             dots=np.zeros((max(nd, 1), 3), np.float32))
    if n:
        L.orc_dump(ptr, *[_p(d[k]) for k in ("flags", "dots_num", "boxes", "centers",
                                             "child_mask", "dot_offset", "dots")])
    d["dots"] = d["dots"][:nd]
    return d


def ray_batch(tree_ptr, origins, dirs, root=None, nthreads=None):
    o = np.ascontiguousarray(origins, dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    n = o.shape[0]
    leaf = np.empty(n, np.uint32)
    slot = np.empty(n, np.uint8)
    pts = np.zeros((n, 3), np.float32)
    cnt = np.zeros(3, np.uint64)
    lib().orc_ray_batch(tree_ptr, root if root is not None else tree_ptr, n, _p(o), _p(d),
                        _p(leaf), _p(slot), _p(pts), _p(cnt), nthreads or nthreads_default())
    return leaf, slot, pts, cnt


def ball_batch(tree_ptr, centres, radii, nthreads=None):
    c = np.ascontiguousarray(centres, dtype=np.float32)
    r = np.ascontiguousarray(radii, dtype=np.float32)
    hit = np.empty(c.shape[0], np.uint8)
    cnt = np.zeros(3, np.uint64)
    lib().orc_ball_batch(tree_ptr, c.shape[0], _p(c), _p(r), _p(hit), _p(cnt),
                         nthreads or nthreads_default())
    return hit, cnt


def camera(state: dict) -> OrcCamera:
    cam = OrcCamera()
    cam.kind = int(state.get("kind", 0))
    cam.position[:] = [float(x) for x in state["position"]]
    cam.rotation[:] = [float(x) for x in state.get("rotation", (1, 0, 0, 0))]
    for k in ("mul", "xsub", "ysub", "sinphi", "cosphi", "k"):
        setattr(cam, k, float(state.get(k, 0.0)))
    if cam.kind == 2:   # directions of every pixel, shape (h, w, 3)
        rays = np.ascontiguousarray(state["rays"], dtype=np.float32)
        cam._rays = rays
        cam.rays = rays.ctypes.data
        cam.rays_w = rays.shape[1]
    return cam


def camera_simple(position, target, w: int, h: int, fov: float = 1.0) -> dict:
    """The state of a simple-camera set up for a w x h window at `position`
    looking at `target` (the oracle's restatement of simple-camera.c's
    set-up), as a camera-state dict for render_best and friends."""
    cam = OrcCamera()
    pos = np.ascontiguousarray(np.asarray(position, np.float32).reshape(3))
    tgt = np.ascontiguousarray(np.asarray(target, np.float32).reshape(3))
    lib().orc_camera_simple(C.byref(cam), _p(pos), _p(tgt), int(w), int(h), float(fov))
    return dict(kind=0, position=np.array(cam.position[:], np.float32),
                rotation=np.array(cam.rotation[:], np.float32), mul=np.float32(cam.mul),
                xsub=np.float32(cam.xsub), ysub=np.float32(cam.ysub), fov=np.float32(fov))


def screen2world(state: dict, sx: int, sy: int) -> np.ndarray:
    out = np.zeros(3, np.float32)
    lib().orc_screen2world(C.byref(camera(state)), sx, sy, _p(out))
    return out


def render_best(tree_ptr, state: dict, w: int, h: int, texture: np.ndarray, nthreads=None):
    tex = np.ascontiguousarray(texture, dtype=np.uint8)
    out = np.zeros(w * h, np.uint32)
    cnt = np.zeros(3, np.uint64)
    rc = lib().orc_render_best(tree_ptr, C.byref(camera(state)), w, h, _p(tex), _p(out), _p(cnt),
                               nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("bad geometry: width must be a multiple of 16 and height of 4")
    return out.reshape(h, w), cnt


def render_quality(tree_ptr, state: dict, w: int, h: int, quality: int, texture: np.ndarray,
                   nthreads=None):
    tex = np.ascontiguousarray(texture, dtype=np.uint8)
    out = np.zeros(w * h, np.uint32)
    cnt = np.zeros(3, np.uint64)
    rc = lib().orc_render_quality(tree_ptr, C.byref(camera(state)), w, h, quality, _p(tex), _p(out),
                                  _p(cnt), nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("bad geometry: width must be a multiple of 16 and height of 4")
    return out.reshape(h, w), cnt


def ray_counts_per_ray(root_ptr, origins, dirs, nthreads=None):
    o = np.ascontiguousarray(origins, dtype=np.float32)
    d = np.ascontiguousarray(dirs, dtype=np.float32)
    out = np.zeros((o.shape[0], 3), np.uint32)
    lib().orc_ray_counts_per_ray(root_ptr, o.shape[0], _p(o), _p(d), _p(out), nthreads or nthreads_default())
    return out


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


class OracleLights:
    """The oracle's light manager (lights.c / mtree.c restated)."""

    def __init__(self):
        self.ptr = lib().orc_lights_new()

    def __del__(self):
        if getattr(self, "ptr", None):
            lib().orc_lights_free(self.ptr)
            self.ptr = None

    def ambient(self, color) -> bool:
        return bool(lib().orc_lights_ambient(self.ptr, _p(_f3(color))))

    def insert(self, center, radius, color) -> bool:
        return bool(lib().orc_lights_insert(self.ptr, _p(_f3(center)), float(radius), _p(_f3(color))))

    def delete(self, center, radius) -> bool:
        return bool(lib().orc_lights_delete(self.ptr, _p(_f3(center)), float(radius)))

    def count(self) -> int:
        return int(lib().orc_lights_count(self.ptr))

    def light(self, p):
        """(light rgb, number of spheres containing p)."""
        out = np.zeros(3, np.float32)
        n = lib().orc_lights_get(self.ptr, _p(_f3(p)), _p(out))
        return out, int(n)

    def verify(self) -> int:
        return int(lib().orc_lights_verify(self.ptr))


def render_lit(tree_ptr, state: dict, w: int, h: int, quality: int, texture: np.ndarray, lights, nthreads=None):
    tex = np.ascontiguousarray(texture, dtype=np.uint8)
    out = np.zeros(w * h, np.uint32)
    rc = lib().orc_render_lit(tree_ptr, C.byref(camera(state)), w, h, quality, _p(tex),
                              lights.ptr if lights is not None else None, _p(out), nthreads or nthreads_default())
    if rc != 0:
        raise ValueError("bad geometry: width must be a multiple of 16 and height of 4")
    return out.reshape(h, w)
