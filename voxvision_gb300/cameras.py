"""Python handle on the library's built-in camera classes (include/voxrnd.h).

The camera objects live in the C library and are driven through their
vtables exactly as a C caller would (camera.h:17-117); `state()` reads the
fields screen2world uses, for vox_cuda_camera.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import CAMERA_DOOM, CAMERA_SIMPLE, CameraStruct, lib

_vp = C.c_void_p
S2W = C.CFUNCTYPE(None, _vp, _vp, C.c_int, C.c_int)
SETDOT = C.CFUNCTYPE(None, _vp, C.c_char_p, _vp)
SETNUM = C.CFUNCTYPE(None, _vp, C.c_char_p, C.c_float)
DOTM = C.CFUNCTYPE(None, _vp, _vp)
WS = C.CFUNCTYPE(None, _vp, C.c_int, C.c_int)
CONS = C.CFUNCTYPE(_vp, _vp)
DESTROY = C.CFUNCTYPE(None, _vp)


class _Simple(C.Structure):       # simple-camera.c:10-17
    _fields_ = [("iface", _vp), ("xsub", C.c_float), ("ysub", C.c_float), ("position", C.c_float * 3),
                ("rotation", C.c_float * 4), ("mul", C.c_float), ("fov", C.c_float)]


class _Doom(C.Structure):         # doom-camera.c:8-15
    _fields_ = [("iface", _vp), ("xsub", C.c_float), ("ysub", C.c_float), ("position", C.c_float * 3),
                ("phi", C.c_float), ("sinphi", C.c_float), ("cosphi", C.c_float), ("k", C.c_float),
                ("mul", C.c_float), ("fov", C.c_float)]


class HostCamera:
    NAMES = {CAMERA_SIMPLE: b"simple-camera", CAMERA_DOOM: b"doom-camera"}

    def __init__(self, kind: int = CAMERA_SIMPLE):
        self.kind = kind
        meth = lib().vox_camera_methods(self.NAMES[kind])
        if not meth:
            raise ValueError("unknown camera class")
        tbl = C.cast(meth, C.POINTER(_vp * 10)).contents
        self.obj = CONS(tbl[8])(None)
        it = C.cast(C.cast(self.obj, C.POINTER(_vp))[0], C.POINTER(_vp * 10)).contents
        self._set_num = SETNUM(it[0]); self._set_dot = SETDOT(it[1]); self._s2w = S2W(it[2])
        self._rotate = DOTM(it[3]); self._move = DOTM(it[4]); self._look_at = DOTM(it[5])
        self._get_pos = DOTM(it[6]); self._set_ws = WS(it[7]); self._destroy = DESTROY(it[9])

    def close(self):
        if self.obj:
            self._destroy(self.obj)
            self.obj = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _f3(v):
        return np.ascontiguousarray(np.asarray(v, np.float32).reshape(3))

    def set_fov(self, fov: float):
        self._set_num(self.obj, b"fov", C.c_float(fov))

    def set_position(self, p):
        a = self._f3(p)
        self._set_dot(self.obj, b"position", a.ctypes.data_as(_vp))

    def set_rotation(self, r):
        a = self._f3(r)
        self._set_dot(self.obj, b"rotation", a.ctypes.data_as(_vp))

    def look_at(self, p):
        a = self._f3(p)
        self._look_at(self.obj, a.ctypes.data_as(_vp))

    def rotate(self, d):
        a = self._f3(d)
        self._rotate(self.obj, a.ctypes.data_as(_vp))

    def move(self, d):
        a = self._f3(d)
        self._move(self.obj, a.ctypes.data_as(_vp))

    def set_window_size(self, w: int, h: int):
        self._set_ws(self.obj, w, h)

    def screen2world(self, sx: int, sy: int) -> np.ndarray:
        out = np.zeros(3, np.float32)
        self._s2w(self.obj, out.ctypes.data_as(_vp), sx, sy)
        return out

    def position(self) -> np.ndarray:
        out = np.zeros(3, np.float32)
        self._get_pos(self.obj, out.ctypes.data_as(_vp))
        return out

    def state(self) -> dict:
        st = C.cast(self.obj, C.POINTER(_Simple if self.kind == CAMERA_SIMPLE else _Doom)).contents
        s = dict(kind=self.kind, position=np.array(st.position[:], np.float32), mul=np.float32(st.mul),
                 xsub=np.float32(st.xsub), ysub=np.float32(st.ysub), fov=np.float32(st.fov))
        if self.kind == CAMERA_SIMPLE:
            s["rotation"] = np.array(st.rotation[:], np.float32)
        else:
            s.update(sinphi=np.float32(st.sinphi), cosphi=np.float32(st.cosphi), k=np.float32(st.k),
                     phi=np.float32(st.phi))
        return s

    def gpu_struct(self) -> CameraStruct:
        from . import camera_struct
        return camera_struct(self.state())


def orbit_camera(frame: int, nframes: int, w: int, h: int, centre, radius: float,
                 elevation_deg: float = 20.0, fov: float = 1.0, kind: int = CAMERA_SIMPLE) -> HostCamera:
    """A camera on a circular orbit around `centre`, looking at it."""
    from .workloads import orbit_pose
    cam = HostCamera(kind)
    cam.set_fov(fov)
    cam.set_window_size(w, h)
    cam.set_position(orbit_pose(frame, nframes, centre, radius, elevation_deg))
    cam.look_at(np.asarray(centre, np.float32))
    return cam
