"""ctypes binding of libvoxtrees_cuda.so (the C ABI in include/voxtrees_cuda.h,
include/voxtrees.h and include/voxrnd.h).

The library is built in-tree by voxvision_gb300.build; importing this module
never builds and never falls back to anything: a missing library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# VOXTREES_CUDA_LIB selects another build of the library (the checked one).
LIB_PATH = os.environ.get("VOXTREES_CUDA_LIB") or os.path.join(HERE, "libvoxtrees_cuda.so")

VOX_CUDA_MISS = 0xFFFFFFFF
VOX_CUDA_SLOT_DENSE = 0xFF
CAMERA_SIMPLE = 0
CAMERA_DOOM = 1

ERRORS = {
    0: "ok", -1: "EINVAL", -2: "ENOMEM", -3: "ECUDA", -4: "EDEPTH", -5: "ESTACK",
    -6: "ETOOBIG", -7: "EGEOMETRY", -8: "EBUDGET", -9: "ETIMEOUT", -10: "ENODEV", -11: "ECAPACITY",
}


class VoxCudaError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, code)} ({code})")


class CameraStruct(C.Structure):
    """vox_cuda_camera (include/voxtrees_cuda.h)."""
    _fields_ = [("kind", C.c_int32), ("position", C.c_float * 3), ("rotation", C.c_float * 4),
                ("mul", C.c_float), ("xsub", C.c_float), ("ysub", C.c_float),
                ("sinphi", C.c_float), ("cosphi", C.c_float), ("k", C.c_float)]


class TreeInfo(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in
                ("nodes", "inner", "leaves", "dense_leaves", "dots", "depth", "device_bytes")]


class RawTest(C.Structure):
    """vox_cuda_raw_test (include/voxtrees_cuda.h)."""
    _fields_ = [("lo", C.c_uint32), ("hi", C.c_uint32), ("mask", C.c_void_p)]


class FrameJob(C.Structure):
    """vox_cuda_frame_job (include/voxtrees_cuda.h)."""
    _fields_ = [("tree", C.c_void_p), ("camera", CameraStruct), ("w", C.c_uint32), ("h", C.c_uint32),
                ("texture", C.c_void_p), ("argb", C.c_void_p)]


class BatchConfig(C.Structure):
    """vox_cuda_batch_config (include/voxtrees_cuda.h)."""
    _fields_ = [("tile_w", C.c_uint32), ("tile_h", C.c_uint32), ("tiles_per_grab", C.c_uint32),
                ("blocks_per_sm", C.c_uint32), ("stack_class", C.c_uint32)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


class ServerConfig(C.Structure):
    """vox_cuda_server_config (include/voxtrees_cuda.h)."""
    _fields_ = [("budget_bytes", C.c_uint64), ("host_budget_bytes", C.c_uint64), ("max_inflight", C.c_uint32),
                ("max_batch", C.c_uint32),
                ("streams", C.c_uint32), ("max_launches", C.c_uint32), ("frames_on_device", C.c_uint32)]


class RenderConfig(C.Structure):
    """vox_cuda_render_config (include/voxtrees_cuda.h)."""
    _fields_ = [("cull", C.c_uint32), ("overlap", C.c_uint32)]


class ReplayRequest(C.Structure):
    """vox_cuda_replay_request (include/voxtrees_cuda.h)."""
    _fields_ = [("kind", C.c_uint32), ("tree_id", C.c_uint32), ("camera", CameraStruct), ("w", C.c_uint32),
                ("h", C.c_uint32), ("centres", C.c_void_p), ("radii", C.c_void_p), ("n", C.c_uint32),
                ("arrival_s", C.c_double)]


class ReplayResult(C.Structure):
    """vox_cuda_replay_result (include/voxtrees_cuda.h)."""
    _fields_ = [("status", C.c_int32), ("submit_ns", C.c_uint64), ("launch_ns", C.c_uint64),
                ("done_ns", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "rejected", "launches", "bytes_in_use",
                                          "peak_bytes", "pending", "inflight", "host_bytes_in_use",
                                          "host_peak_bytes", "worker_busy_ns", "build_ns", "host_pin_ns",
                                          "host_pins", "device_alloc_ns", "frame_bytes_out", "host_slabs",
                                          "frame_bytes_full")]


_lib = None

# name -> (restype, argtypes)
_vp, _sz, _u32, _f = C.c_void_p, C.c_size_t, C.c_uint32, C.c_float
SIGNATURES = {
    "vox_cuda_strerror": (C.c_char_p, [C.c_int]),
    "vox_cuda_version": (C.c_char_p, []),
    "vox_cuda_launch_count": (C.c_uint64, []),
    "vox_cuda_tree_upload": (C.c_int, [_vp, C.POINTER(_vp)]),
    "vox_cuda_tree_free": (C.c_int, [_vp]),
    "vox_cuda_tree_refresh": (C.c_int, [_vp, _vp]),
    "vox_cuda_render_frames": (C.c_int, [_vp, _vp, _u32, _u32, _u32, _vp, _vp, _vp]),
    "vox_cuda_tree_build": (C.c_int, [_vp, _sz, C.POINTER(_vp)]),
    "vox_cuda_make_tree_gpu_min": (_sz, [_sz]),
    "vox_make_tree_host": (_vp, [_vp, _sz]),
    "vox_cuda_tree_build_device": (C.c_int, [_vp, _sz, C.POINTER(_vp)]),
    "vox_cuda_tree_build_raw": (C.c_int, [_vp, C.POINTER(C.c_uint * 3), C.c_uint, C.POINTER(RawTest),
                                          C.POINTER(_vp)]),
    "vox_cuda_read_raw_data": (C.c_int, [C.c_char_p, C.POINTER(C.c_uint * 3), C.c_uint, C.POINTER(RawTest),
                                         C.POINTER(_vp), C.POINTER(C.c_char_p)]),
    "vox_cuda_tree_image": (C.c_int, [_vp, _vp, _sz, _vp, _sz, C.POINTER(_sz), C.POINTER(_sz)]),
    "vox_cuda_tree_measure": (C.c_int, [_vp, C.POINTER(TreeInfo)]),
    "vox_cuda_tree_get_info": (C.c_int, [_vp, C.POINTER(TreeInfo)]),
    "vox_cuda_tree_node": (_vp, [_vp, _u32]),
    "vox_cuda_tree_node_id": (C.c_int, [_vp, _vp, C.POINTER(_u32)]),
    "vox_cuda_ray_batch": (C.c_int, [_vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp]),
    "vox_cuda_ray_batch_device": (C.c_int, [_vp, _vp, _vp, _vp, _sz, _vp, _vp, _vp, _vp]),
    "vox_cuda_ball_batch": (C.c_int, [_vp, _vp, _vp, _sz, _vp, _vp]),
    "vox_cuda_ball_batch_device": (C.c_int, [_vp, _vp, _vp, _sz, _vp, _vp]),
    "vox_cuda_render": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, _vp, _vp, _vp]),
    "vox_cuda_render_device": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, _vp, _vp, _vp]),
    "vox_cuda_render_quality": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, C.c_uint, _vp, _vp,
                                          _vp]),
    "vox_cuda_render_quality_device": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, C.c_uint, _vp,
                                                 _vp, _vp]),
    "vox_cuda_frame_rect": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, _vp]),
    "vox_cuda_render_set_config": (C.c_int, [C.POINTER(RenderConfig)]),
    "vox_cuda_render_get_config": (C.c_int, [C.POINTER(RenderConfig)]),
    "vox_cuda_lights_upload": (C.c_int, [_vp, C.POINTER(_vp)]),
    "vox_cuda_lights_free": (C.c_int, [_vp]),
    "vox_cuda_render_lit": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, C.c_uint, _vp, _vp, _vp, _vp]),
    "vox_cuda_render_lit_device": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, C.c_uint, _vp, _vp, _vp,
                                             _vp]),
    "vox_cuda_build_checked": (C.c_int, []),
    "vox_cuda_server_inject": (C.c_int, [_vp, C.c_int]),
    "vox_cuda_tree_flatten_host": (C.c_int, [_vp, _vp, C.c_size_t, _vp, C.c_size_t, C.POINTER(C.c_size_t),
                                             C.POINTER(C.c_size_t)]),
    "vox_cuda_image_check": (C.c_int, [_vp, C.c_size_t, C.c_size_t]),
    "vox_cuda_measure_l2_read": (C.c_int, [C.c_size_t, _u32, C.POINTER(C.c_float)]),
    "vox_cuda_tree_upload_layout": (C.c_int, [_vp, C.c_int, _vp, C.POINTER(_vp)]),
    "vox_cuda_tree_refresh_layout": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "vox_cuda_tree_flatten_host_layout": (C.c_int, [_vp, C.c_int, _vp, _vp, C.c_size_t, _vp, C.c_size_t,
                                                    C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "vox_cuda_render_rays_device": (C.c_int, [_vp, _vp, _vp, _u32, _u32, C.c_uint, _vp, _vp, _vp, _vp]),
    "vox_cuda_batch_create": (C.c_int, [C.POINTER(FrameJob), _u32, C.POINTER(BatchConfig), C.POINTER(_vp)]),
    "vox_cuda_batch_set_camera": (C.c_int, [_vp, _u32, C.POINTER(CameraStruct)]),
    "vox_cuda_batch_launch": (C.c_int, [_vp, _vp]),
    "vox_cuda_batch_get_config": (C.c_int, [_vp, C.POINTER(BatchConfig)]),
    "vox_cuda_batch_set_config": (C.c_int, [_vp, C.POINTER(BatchConfig)]),
    "vox_cuda_batch_autotune": (C.c_int, [_vp, _vp, _u32, C.POINTER(BatchConfig), C.POINTER(C.c_float)]),
    "vox_cuda_batch_free": (C.c_int, [_vp]),
    "vox_cuda_render_frames_noalloc": (C.c_int, [C.POINTER(FrameJob), _u32, _vp]),
    "vox_cuda_server_create": (C.c_int, [C.POINTER(ServerConfig), _vp, C.POINTER(_vp)]),
    "vox_cuda_server_add_tree": (C.c_int, [_vp, _vp, C.POINTER(_u32)]),
    "vox_cuda_server_submit_frame": (C.c_int, [_vp, _u32, C.POINTER(CameraStruct), _u32, _u32,
                                               C.POINTER(C.c_uint64)]),
    "vox_cuda_server_submit_balls": (C.c_int, [_vp, _u32, _vp, _vp, _u32, C.POINTER(C.c_uint64)]),
    "vox_cuda_server_wait": (C.c_int, [_vp, C.c_uint64, _u32]),
    "vox_cuda_server_result": (C.c_int, [_vp, C.c_uint64, C.POINTER(_vp), C.POINTER(_sz), C.POINTER(C.c_uint64)]),
    "vox_cuda_server_release": (C.c_int, [_vp, C.c_uint64]),
    "vox_cuda_server_get_stats": (C.c_int, [_vp, C.POINTER(ServerStats)]),
    "vox_cuda_server_destroy": (C.c_int, [_vp]),
    "vox_cuda_server_replay": (C.c_int, [_vp, C.POINTER(ReplayRequest), _u32, _u32, C.POINTER(ReplayResult)]),
    "vox_cuda_render_counts_device": (C.c_int, [_vp, C.POINTER(CameraStruct), _u32, _u32, _vp, _vp]),
    "vox_cuda_ray_counts_device": (C.c_int, [_vp, _vp, _vp, _sz, _vp, _vp]),
    "vox_cuda_ball_counts_device": (C.c_int, [_vp, _vp, _vp, _sz, _vp, _vp]),
    # voxtrees.h
    "vox_make_tree": (_vp, [_vp, _sz]),
    "vox_insert_voxel": (C.c_int, [C.POINTER(_vp), _vp]),
    "vox_insert_voxel_coord": (C.c_int, [C.POINTER(_vp), _f, _f, _f]),
    "vox_delete_voxel": (C.c_int, [C.POINTER(_vp), _vp]),
    "vox_delete_voxel_coord": (C.c_int, [C.POINTER(_vp), _f, _f, _f]),
    "vox_rebuild_tree": (_vp, [_vp]),
    "vox_destroy_tree": (None, [_vp]),
    "vox_voxels_in_tree": (_sz, [_vp]),
    "vox_bounding_box": (None, [_vp, _vp]),
    "vox_make_dense_leaf": (_vp, [_vp]),
    "vox_set_voxel_size": (None, [_f, _f, _f]),
    "vox_ray_tree_intersection": (_vp, [_vp, _vp, _vp, _vp]),
    "vox_tree_ball_collidep": (C.c_int, [_vp, _vp, _f]),
    "vox_cuda_forget_tree": (None, [_vp]),
    # voxrnd.h (cameras)
    "vox_camera_methods": (_vp, [C.c_char_p]),
    "vox_init_camera": (None, [_vp]),
    "vox_use_camera_methods": (None, [_vp, _vp]),
    # voxrnd.h (renderer)
    "vox_make_context_headless": (_vp, [C.c_uint, C.c_uint]),
    "vox_destroy_context": (None, [_vp]),
    "vox_context_set_scene": (None, [_vp, _vp]),
    "vox_context_set_camera": (None, [_vp, _vp]),
    "vox_context_set_quality": (C.c_int, [_vp, C.c_uint]),
    "vox_context_set_texture": (None, [_vp, _vp]),
    "vox_render": (None, [_vp]),
    "vox_redraw": (None, [_vp]),
    "vox_context_pixels": (_vp, [_vp]),
    "vox_context_status": (C.c_int, [_vp]),
    "vox_make_light_manager": (_vp, []),
    "vox_destroy_light_manager": (None, [_vp]),
    "vox_set_ambient_light": (C.c_int, [_vp, _vp]),
    "vox_insert_shadowless_light": (C.c_int, [_vp, _vp, _f, _vp]),
    "vox_delete_shadowless_light": (C.c_int, [_vp, _vp, _f]),
    "vox_delete_shadowless_lights": (None, [_vp]),
    "vox_shadowless_lights_number": (C.c_int, [_vp]),
    "vox_context_set_light_manager": (None, [_vp, _vp]),
    "vox_make_cd": (_vp, []),
    "vox_cd_attach_camera": (None, [_vp, _vp, _f]),
    "vox_cd_attach_context": (None, [_vp, _vp]),
    "vox_cd_collide": (None, [_vp]),
    "vox_cd_gravity": (None, [_vp, _vp]),
}


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run voxvision_gb300.build.build() first "
                               "(there is no fallback implementation)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, what: str):
    if rc != 0:
        raise VoxCudaError(rc, what)
