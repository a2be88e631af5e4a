"""voxvision_gb300: the voxtrees ray/ball search path of shamazmazum/voxvision
on GB300 (sm_103a), behind the reference's C API.

Python here is a thin host layer over the C ABI of libvoxtrees_cuda.so
(include/voxtrees_cuda.h, include/voxtrees.h): tests and the benchmark call
the library exactly as a C program would.  numpy arrays are host buffers;
torch tensors (or raw integers) are device pointers for the *_device entry
points.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (CAMERA_DOOM, CAMERA_SIMPLE, VOX_CUDA_MISS, VOX_CUDA_SLOT_DENSE, BatchConfig, CameraStruct,
                   FrameJob, RawTest, RenderConfig, ReplayRequest, ReplayResult, ServerConfig, ServerStats,
                   TreeInfo, VoxCudaError, available, check, lib)

__all__ = ["HostTree", "DeviceTree", "FrameBatch", "BatchConfig", "Server", "ServerConfig", "Camera", "camera_struct", "VoxCudaError", "available", "lib",
           "VOX_CUDA_MISS", "VOX_CUDA_SLOT_DENSE", "CAMERA_SIMPLE", "CAMERA_DOOM", "set_voxel_size",
           "frame_rect", "render_config", "set_render_config", "LightManager", "DeviceLights"]


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _dptr(x):
    """Device pointer of a torch tensor, an int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return C.c_void_p(x)
    return C.c_void_p(x.data_ptr())


def set_voxel_size(v=(1.0, 1.0, 1.0)):
    lib().vox_set_voxel_size(*[float(a) for a in v])


class HostTree:
    """A host octree built by the library's vox_make_tree (tree.c:249-338 order)."""

    def __init__(self, ptr: int | None, owned: bool = True):
        self.ptr = ptr
        self.owned = owned

    @classmethod
    def from_voxels(cls, voxels: np.ndarray) -> "HostTree":
        s = np.ascontiguousarray(voxels, dtype=np.float32).copy()   # the build reorders its input
        if s.ndim != 2 or s.shape[1] != 3:
            raise ValueError("voxels must be (n, 3)")
        return cls(lib().vox_make_tree(_p(s), s.shape[0]))

    def voxels(self) -> int:
        return int(lib().vox_voxels_in_tree(self.ptr)) if self.ptr else 0

    def close(self):
        if self.ptr and self.owned:
            lib().vox_destroy_tree(self.ptr)
        self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def measure_tree(host_ptr) -> dict:
    """vox_cuda_tree_measure: flatten and check on the host, report sizes."""
    i = TreeInfo()
    check(lib().vox_cuda_tree_measure(host_ptr, C.byref(i)), "vox_cuda_tree_measure")
    return {k: int(getattr(i, k)) for k, _ in TreeInfo._fields_}


def _raw_test(samplesize: int, lo: int | None, hi: int | None, test=None):
    """A vox_cuda_raw_test: the range [lo, hi] of solid samples, or a
    predicate tabulated over every sample value (samplesize 1 or 2)."""
    if test is not None:
        if samplesize > 2:
            raise ValueError("a predicate is tabulated only for 1- and 2-byte samples")
        vals = np.arange(1 << (8 * samplesize), dtype=np.uint64)
        bits = np.fromiter((1 if test(int(v)) else 0 for v in vals), np.uint8, vals.size)
        mask = np.packbits(bits, bitorder="little")
        return RawTest(0, 0, mask.ctypes.data), mask
    lo = 0 if lo is None else int(lo)
    hi = (1 << (8 * samplesize)) - 1 if hi is None else int(hi)
    return RawTest(lo, hi, None), None


class DeviceTree:
    """A device tree: uploaded from a host tree (vox_cuda_tree_upload), or built
    on the GPU from voxels or a raw volume (DeviceTree.build*, from_raw)."""

    def __init__(self, host_ptr=None, *, handle=None):
        if handle is not None:
            self.h = handle
            return
        h = C.c_void_p()
        check(lib().vox_cuda_tree_upload(host_ptr, C.byref(h)), "vox_cuda_tree_upload")
        self.h = h

    @classmethod
    def build(cls, voxels: np.ndarray) -> "DeviceTree":
        """vox_cuda_tree_build: vox_make_tree's tree of `voxels` ((n, 3) float32,
        host), built on the GPU."""
        s = np.ascontiguousarray(voxels, dtype=np.float32)
        if s.ndim != 2 or s.shape[1] != 3:
            raise ValueError("voxels must be (n, 3)")
        h = C.c_void_p()
        check(lib().vox_cuda_tree_build(_p(s), s.shape[0], C.byref(h)), "vox_cuda_tree_build")
        return cls(handle=h)

    @classmethod
    def build_device(cls, voxels, n: int | None = None) -> "DeviceTree":
        """vox_cuda_tree_build_device: voxels already on the device (a torch
        tensor of (n, 3) float32 or a device pointer with n)."""
        if n is None:
            n = int(voxels.shape[0])
        h = C.c_void_p()
        check(lib().vox_cuda_tree_build_device(_dptr(voxels), n, C.byref(h)), "vox_cuda_tree_build_device")
        return cls(handle=h)

    @classmethod
    def from_raw(cls, samples, dim, samplesize: int = 1, lo: int | None = None, hi: int | None = None,
                 test=None) -> "DeviceTree":
        """vox_cuda_tree_build_raw: a dim[0] x dim[1] x dim[2] volume of
        little-endian samples (bytes or a numpy array), solid where
        lo <= sample <= hi or where test(sample) is true."""
        buf = np.ascontiguousarray(np.frombuffer(samples, np.uint8) if isinstance(samples, (bytes, bytearray))
                                   else np.asarray(samples)).view(np.uint8)
        d = (C.c_uint * 3)(*[int(x) for x in dim])
        rt, keep = _raw_test(samplesize, lo, hi, test)
        h = C.c_void_p()
        check(lib().vox_cuda_tree_build_raw(_p(buf), C.byref(d), samplesize, C.byref(rt), C.byref(h)),
              "vox_cuda_tree_build_raw")
        del keep
        return cls(handle=h)

    @classmethod
    def read_raw(cls, path: str, dim, samplesize: int = 1, lo: int | None = None, hi: int | None = None,
                 test=None) -> "DeviceTree":
        """vox_cuda_read_raw_data (vox_read_raw_data with the test on the GPU)."""
        d = (C.c_uint * 3)(*[int(x) for x in dim])
        rt, keep = _raw_test(samplesize, lo, hi, test)
        h = C.c_void_p()
        err = C.c_char_p()
        rc = lib().vox_cuda_read_raw_data(path.encode(), C.byref(d), samplesize, C.byref(rt), C.byref(h),
                                         C.byref(err))
        del keep
        if rc:
            raise VoxCudaError(rc, f"vox_cuda_read_raw_data: {err.value.decode() if err.value else rc}")
        return cls(handle=h)

    def image(self):
        """The device image: (units as an (n, 4) uint32 array, pre-order id ->
        record offset)."""
        nu, ni = C.c_size_t(), C.c_size_t()
        check(lib().vox_cuda_tree_image(self.h, None, 0, None, 0, C.byref(nu), C.byref(ni)), "vox_cuda_tree_image")
        units = np.zeros((nu.value, 4), np.uint32)
        ids = np.zeros(ni.value, np.uint32)
        check(lib().vox_cuda_tree_image(self.h, _p(units), nu.value, _p(ids), ni.value, None, None),
              "vox_cuda_tree_image")
        return units, ids

    def info(self) -> dict:
        i = TreeInfo()
        check(lib().vox_cuda_tree_get_info(self.h, C.byref(i)), "vox_cuda_tree_get_info")
        return {k: int(getattr(i, k)) for k, _ in TreeInfo._fields_}

    def node(self, preorder_id: int):
        return lib().vox_cuda_tree_node(self.h, preorder_id)

    def node_id(self, host_node_ptr) -> int:
        v = C.c_uint32()
        check(lib().vox_cuda_tree_node_id(self.h, host_node_ptr, C.byref(v)), "vox_cuda_tree_node_id")
        return int(v.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().vox_cuda_tree_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---------------------------------------------------------- host buffers
    def rays(self, origins, dirs, roots=None, stream=None):
        o = np.ascontiguousarray(origins, dtype=np.float32)
        d = np.ascontiguousarray(dirs, dtype=np.float32)
        n = o.shape[0]
        leaf = np.empty(n, np.uint32)
        slot = np.empty(n, np.uint8)
        pts = np.zeros((n, 3), np.float32)
        r = None if roots is None else np.ascontiguousarray(roots, dtype=np.uint32)
        check(lib().vox_cuda_ray_batch(self.h, _p(o), _p(d), None if r is None else _p(r), n,
                                       _p(leaf), _p(slot), _p(pts), stream),
              "vox_cuda_ray_batch")
        return leaf, slot, pts

    def balls(self, centres, radii, stream=None):
        c = np.ascontiguousarray(centres, dtype=np.float32)
        r = np.ascontiguousarray(radii, dtype=np.float32)
        hit = np.empty(c.shape[0], np.uint8)
        check(lib().vox_cuda_ball_batch(self.h, _p(c), _p(r), c.shape[0], _p(hit), stream),
              "vox_cuda_ball_batch")
        return hit

    def render(self, camera: CameraStruct, w: int, h: int, texture: np.ndarray, stream=None):
        tex = np.ascontiguousarray(texture, dtype=np.uint8)
        out = np.empty((h, w), np.uint32)
        check(lib().vox_cuda_render(self.h, C.byref(camera), w, h, _p(tex), _p(out), stream),
              "vox_cuda_render")
        return out

    def render_frames(self, cameras, w: int, h: int, texture: np.ndarray, frames=None, stream=None):
        """vox_cuda_render_frames: one BEST frame per camera into host
        buffers (numpy arrays, or pinned torch tensors drawn in place)."""
        cams = (CameraStruct * len(cameras))(*cameras)
        tex = np.ascontiguousarray(texture, dtype=np.uint8)
        if frames is None:
            frames = [np.empty((h, w), np.uint32) for _ in cameras]
        ptrs = (C.c_void_p * len(frames))(*[f.ctypes.data if isinstance(f, np.ndarray) else f.data_ptr()
                                             for f in frames])
        check(lib().vox_cuda_render_frames(self.h, C.byref(cams), len(cameras), w, h, _p(tex), ptrs, stream),
              "vox_cuda_render_frames")
        return frames

    def render_quality(self, camera: CameraStruct, w: int, h: int, quality: int, texture: np.ndarray,
                       stream=None):
        tex = np.ascontiguousarray(texture, dtype=np.uint8)
        out = np.empty((h, w), np.uint32)
        check(lib().vox_cuda_render_quality(self.h, C.byref(camera), w, h, quality, _p(tex), _p(out),
                                            stream), "vox_cuda_render_quality")
        return out

    # -------------------------------------------------------- device buffers
    def render_lit(self, camera: CameraStruct, w: int, h: int, quality: int, texture: np.ndarray,
                   lights: "DeviceLights | None", stream=None):
        """vox_cuda_render_lit with host buffers: (h, w) uint32 ARGB."""
        tex = np.ascontiguousarray(texture, dtype=np.uint8)
        out = np.empty(w * h, np.uint32)
        check(lib().vox_cuda_render_lit(self.h, C.byref(camera), w, h, quality, _p(tex),
                                        lights.h if lights is not None else None, _p(out), stream),
              "vox_cuda_render_lit")
        return out.reshape(h, w)

    def rays_device(self, origins, dirs, leaf, slot=None, points=None, roots=None, n=None, stream=None):
        n = int(origins.shape[0]) if n is None else n
        check(lib().vox_cuda_ray_batch_device(self.h, _dptr(origins), _dptr(dirs), _dptr(roots), n,
                                              _dptr(leaf), _dptr(slot), _dptr(points), stream),
              "vox_cuda_ray_batch_device")

    def balls_device(self, centres, radii, hit, n=None, stream=None):
        n = int(centres.shape[0]) if n is None else n
        check(lib().vox_cuda_ball_batch_device(self.h, _dptr(centres), _dptr(radii), n, _dptr(hit),
                                               stream), "vox_cuda_ball_batch_device")

    def render_device(self, camera: CameraStruct, w: int, h: int, texture, argb, stream=None):
        check(lib().vox_cuda_render_device(self.h, C.byref(camera), w, h, _dptr(texture), _dptr(argb),
                                           stream), "vox_cuda_render_device")

    def render_quality_device(self, camera: CameraStruct, w: int, h: int, quality: int, texture, argb,
                              stream=None):
        """vox_cuda_render_quality_device: a frame of any quality into device memory."""
        check(lib().vox_cuda_render_quality_device(self.h, C.byref(camera), w, h, quality, _dptr(texture),
                                                   _dptr(argb), stream), "vox_cuda_render_quality_device")

    def render_rays_device(self, origin, dirs, w: int, h: int, quality: int, texture, argb,
                           lights: "DeviceLights | None" = None, stream=None):
        """vox_cuda_render_rays_device: a frame from each pixel's direction
        (`dirs`, device, (h, w, 3) float32) and the camera's position."""
        o = np.ascontiguousarray(np.asarray(origin, np.float32).reshape(3))
        check(lib().vox_cuda_render_rays_device(self.h, _p(o), _dptr(dirs), w, h, quality, _dptr(texture),
                                                lights.h if lights is not None else None, _dptr(argb), stream),
              "vox_cuda_render_rays_device")

    def render_counts_device(self, camera: CameraStruct, w: int, h: int, counts, stream=None):
        check(lib().vox_cuda_render_counts_device(self.h, C.byref(camera), w, h, _dptr(counts), stream),
              "vox_cuda_render_counts_device")

    def ray_counts_device(self, origins, dirs, counts, n=None, stream=None):
        n = int(origins.shape[0]) if n is None else n
        check(lib().vox_cuda_ray_counts_device(self.h, _dptr(origins), _dptr(dirs), n, _dptr(counts),
                                               stream), "vox_cuda_ray_counts_device")

    def ball_counts_device(self, centres, radii, counts, n=None, stream=None):
        n = int(centres.shape[0]) if n is None else n
        check(lib().vox_cuda_ball_counts_device(self.h, _dptr(centres), _dptr(radii), n, _dptr(counts),
                                                stream), "vox_cuda_ball_counts_device")


def camera_struct(state: dict) -> CameraStruct:
    """vox_cuda_camera from a dict of camera state (position, rotation, mul,
    xsub, ysub; sinphi, cosphi, k for the doom camera)."""
    cam = CameraStruct()
    cam.kind = int(state.get("kind", CAMERA_SIMPLE))
    cam.position[:] = [float(x) for x in state["position"]]
    cam.rotation[:] = [float(x) for x in state.get("rotation", (1.0, 0.0, 0.0, 0.0))]
    for k in ("mul", "xsub", "ysub", "sinphi", "cosphi", "k"):
        setattr(cam, k, float(state.get(k, 0.0)))
    return cam


Camera = CameraStruct


def _f3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(3))


class LightManager:
    """The library's light manager (include/voxrnd.h, lights.h of the reference)."""

    def __init__(self):
        self.ptr = lib().vox_make_light_manager()
        if not self.ptr:
            raise MemoryError("vox_make_light_manager")

    def close(self):
        if self.ptr:
            lib().vox_destroy_light_manager(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ambient(self, color) -> bool:
        return bool(lib().vox_set_ambient_light(self.ptr, _p(_f3(color))))

    def insert(self, center, radius, color) -> bool:
        return bool(lib().vox_insert_shadowless_light(self.ptr, _p(_f3(center)), float(radius), _p(_f3(color))))

    def delete(self, center, radius) -> bool:
        return bool(lib().vox_delete_shadowless_light(self.ptr, _p(_f3(center)), float(radius)))

    def clear(self):
        lib().vox_delete_shadowless_lights(self.ptr)

    def count(self) -> int:
        return int(lib().vox_shadowless_lights_number(self.ptr))

    def upload(self) -> "DeviceLights":
        return DeviceLights(self)


class DeviceLights:
    """vox_cuda_lights: a snapshot of a LightManager on the device."""

    def __init__(self, manager: LightManager):
        h = C.c_void_p()
        check(lib().vox_cuda_lights_upload(manager.ptr, C.byref(h)), "vox_cuda_lights_upload")
        self.h = h

    def close(self):
        if self.h:
            lib().vox_cuda_lights_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def frame_rect(bbox, cam: CameraStruct, w: int, h: int):
    """vox_cuda_frame_rect: (x0, y0, x1, y1) of the w x h frame outside which
    no ray of `cam` can enter the box bbox = (min xyz, max xyz)."""
    b = np.ascontiguousarray(bbox, dtype=np.float32)
    r = np.zeros(4, np.uint32)
    check(lib().vox_cuda_frame_rect(_p(b), C.byref(cam), w, h, _p(r)), "vox_cuda_frame_rect")
    return tuple(int(x) for x in r)


def render_config() -> dict:
    """The process-wide BEST frame kernel settings (vox_cuda_render_get_config)."""
    c = RenderConfig()
    check(lib().vox_cuda_render_get_config(C.byref(c)), "vox_cuda_render_get_config")
    return {"cull": c.cull, "overlap": c.overlap}


def set_render_config(cull: int = 1, overlap: int = 1):
    """vox_cuda_render_set_config: cull to the tree's screen rectangle,
    overlap consecutive frames' kernels (both 0 or 1)."""
    c = RenderConfig(cull, overlap)
    check(lib().vox_cuda_render_set_config(C.byref(c)), "vox_cuda_render_set_config")


class FrameBatch:
    """vox_cuda_batch: many frames in one persistent kernel replayed from a
    CUDA graph.  jobs: iterable of (DeviceTree, CameraStruct, w, h,
    texture_device_ptr_or_tensor, argb_device_ptr_or_tensor)."""

    def __init__(self, jobs, config: BatchConfig | None = None):
        jobs = list(jobs)
        arr = (FrameJob * len(jobs))()
        for i, (tree, cam, w, h, tex, argb) in enumerate(jobs):
            arr[i].tree = tree.h.value
            arr[i].camera = cam
            arr[i].w, arr[i].h = w, h
            arr[i].texture = _dptr(tex).value
            arr[i].argb = _dptr(argb).value
        self._keep = jobs
        h = C.c_void_p()
        check(lib().vox_cuda_batch_create(arr, len(jobs), C.byref(config) if config else None, C.byref(h)),
              "vox_cuda_batch_create")
        self.h = h

    def launch(self, stream=None):
        check(lib().vox_cuda_batch_launch(self.h, stream), "vox_cuda_batch_launch")

    def set_camera(self, job: int, cam: CameraStruct):
        check(lib().vox_cuda_batch_set_camera(self.h, job, C.byref(cam)), "vox_cuda_batch_set_camera")

    def config(self) -> dict:
        c = BatchConfig()
        check(lib().vox_cuda_batch_get_config(self.h, C.byref(c)), "vox_cuda_batch_get_config")
        return c.as_dict()

    def set_config(self, cfg: BatchConfig):
        check(lib().vox_cuda_batch_set_config(self.h, C.byref(cfg)), "vox_cuda_batch_set_config")

    def autotune(self, stream=None, reps: int = 3):
        c = BatchConfig()
        ms = C.c_float()
        check(lib().vox_cuda_batch_autotune(self.h, stream, reps, C.byref(c), C.byref(ms)),
              "vox_cuda_batch_autotune")
        return c.as_dict(), float(ms.value)

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().vox_cuda_batch_free(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_bytes(ptr: int, nbytes: int):
    """A torch uint8 tensor viewing `nbytes` of device memory at `ptr` (no
    copy), through the CUDA array interface."""
    import torch

    class _View:
        __cuda_array_interface__ = {"shape": (nbytes,), "typestr": "|u1", "data": (ptr, False), "version": 2}

    return torch.as_tensor(_View(), device="cuda")


class Server:
    """vox_cuda_server: frame and ball requests from many threads, admitted by
    a device-memory budget and batched continuously onto the GPU."""

    def __init__(self, texture: np.ndarray, config: ServerConfig | None = None):
        self._tex = np.ascontiguousarray(texture, dtype=np.uint8)
        h = C.c_void_p()
        check(lib().vox_cuda_server_create(C.byref(config) if config else None, _p(self._tex), C.byref(h)),
              "vox_cuda_server_create")
        self.h = h
        self._trees = []

    def add_tree(self, tree: "DeviceTree") -> int:
        tid = C.c_uint32()
        check(lib().vox_cuda_server_add_tree(self.h, tree.h, C.byref(tid)), "vox_cuda_server_add_tree")
        self._trees.append(tree)
        return int(tid.value)

    def submit_frame(self, tree_id: int, cam: CameraStruct, w: int, h: int) -> int:
        t = C.c_uint64()
        check(lib().vox_cuda_server_submit_frame(self.h, tree_id, C.byref(cam), w, h, C.byref(t)),
              "vox_cuda_server_submit_frame")
        return int(t.value)

    def submit_balls(self, tree_id: int, centres: np.ndarray, radii: np.ndarray) -> int:
        c = np.ascontiguousarray(centres, dtype=np.float32)
        r = np.ascontiguousarray(radii, dtype=np.float32)
        t = C.c_uint64()
        check(lib().vox_cuda_server_submit_balls(self.h, tree_id, _p(c), _p(r), r.shape[0], C.byref(t)),
              "vox_cuda_server_submit_balls")
        return int(t.value)

    def wait(self, ticket: int, timeout_ms: int = 60000) -> int:
        return int(lib().vox_cuda_server_wait(self.h, ticket, timeout_ms))

    def result(self, ticket: int, copy: bool = True, on_device: bool = False):
        """(array of the result, (t_submit, t_launch, t_done) ns).  With
        on_device (a frame of a server whose frames stay on the device) the
        result is copied out of device memory."""
        data = C.c_void_p()
        nbytes = C.c_size_t()
        times = (C.c_uint64 * 3)()
        check(lib().vox_cuda_server_result(self.h, ticket, C.byref(data), C.byref(nbytes), times),
              "vox_cuda_server_result")
        arr = None
        if copy and on_device:
            arr = device_bytes(data.value, nbytes.value).cpu().numpy()
        elif copy:
            arr = np.ctypeslib.as_array((C.c_uint8 * nbytes.value).from_address(data.value)).copy()
        return arr, tuple(int(x) for x in times)

    def release(self, ticket: int):
        check(lib().vox_cuda_server_release(self.h, ticket), "vox_cuda_server_release")

    def inject(self, what: int):
        """vox_cuda_server_inject: a host-side fault for the next launch
        (1: its requests fail, 2: the worker fails)."""
        check(lib().vox_cuda_server_inject(self.h, what), "vox_cuda_server_inject")

    def replay(self, requests, collectors: int = 8):
        """vox_cuda_server_replay over a trace: a list of ("frame", tree_id,
        camera, w, h, arrival_s) and ("balls", tree_id, centres, radii,
        arrival_s) tuples, arrivals ascending.  Returns an (n, 4) int64 array
        of status, submit, launch and done times (ns)."""
        n = len(requests)
        arr = (ReplayRequest * max(n, 1))()
        keep = []
        for i, q in enumerate(requests):
            r = arr[i]
            if q[0] == "frame":
                _, tid, cam, w, h, at = q
                r.kind, r.tree_id, r.camera, r.w, r.h, r.arrival_s = 0, tid, cam, w, h, at
            else:
                _, tid, c, rad, at = q
                c = np.ascontiguousarray(c, dtype=np.float32)
                rad = np.ascontiguousarray(rad, dtype=np.float32)
                keep += [c, rad]
                r.kind, r.tree_id, r.n, r.arrival_s = 1, tid, rad.shape[0], at
                r.centres, r.radii = c.ctypes.data, rad.ctypes.data
        out = (ReplayResult * max(n, 1))()
        check(lib().vox_cuda_server_replay(self.h, arr, n, collectors, out), "vox_cuda_server_replay")
        return np.array([(o.status, o.submit_ns, o.launch_ns, o.done_ns) for o in out[:n]], dtype=np.int64)

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().vox_cuda_server_get_stats(self.h, C.byref(s)), "vox_cuda_server_get_stats")
        return {k: int(getattr(s, k)) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            lib().vox_cuda_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
