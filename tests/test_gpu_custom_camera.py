"""GPU parity of frames through camera classes the library does not know.

vox_render asks such a camera for every pixel's direction through its own
screen2world, as the reference's tasks do (renderer.c:251,260,292), and draws
the frame from that ray buffer on the GPU (vox_cuda_render_rays_device).  The
oracle reads the same directions (its camera kind 2).  Frames equal the
oracle's pixel for pixel in every quality, lit and unlit; a built-in simple
camera seen through a foreign iface draws the frame its own class draws; and
the device entry point takes ray buffers in device memory directly.
"""
import ctypes as C
import math
import threading

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

QUALITIES = (0, 1, 2, 2 | 4, 2 | 8)
W, H = 192, 128


@pytest.fixture(scope="module")
def scene():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as vg
    from voxvision_gb300 import workloads as wl
    vg.set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    ht = vg.HostTree.from_voxels(wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20)))
    dt = vg.DeviceTree(ht.ptr)
    return vg, wl, ht, dt


class ForeignCamera:
    """A camera object whose iface is a copy of its built-in class's with
    screen2world replaced by `fn(x, y) -> 3 floats`, a Python callback: to the
    library a class it does not know.  Counts the calls."""

    def __init__(self, base, fn):
        from voxvision_gb300.cameras import S2W
        self.base = base
        self._slot = C.cast(base.obj, C.POINTER(C.c_void_p))
        self._orig = self._slot[0]
        self._tbl = (C.c_void_p * 10)(*C.cast(self._orig, C.POINTER(C.c_void_p * 10)).contents)
        self.calls = 0
        lock = threading.Lock()

        def s2w(_cam, ray, x, y):
            r = fn(x, y)
            out = C.cast(ray, C.POINTER(C.c_float * 3)).contents
            out[0], out[1], out[2] = float(r[0]), float(r[1]), float(r[2])
            with lock:
                self.calls += 1

        self._cb = S2W(s2w)
        self._tbl[2] = C.cast(self._cb, C.c_void_p).value
        self._slot[0] = C.addressof(self._tbl)

    def close(self):
        self._slot[0] = self._orig


def _camera(kind=0, w=W, h=H, pos=(150.0, -90.0, 100.0)):
    from voxvision_gb300.cameras import HostCamera
    cam = HostCamera(kind)
    cam.set_window_size(w, h)
    cam.set_position(pos)
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    return cam


def panorama(pos, target, w=W, h=H, span=2.4):
    """A cylindrical projection (no built-in class draws one): yaw across the
    width, height along the cylinder's axis; (h, w, 3) float32."""
    p, c = np.asarray(pos, np.float64), np.asarray(target, np.float64)
    f = (c - p) / np.linalg.norm(c - p)
    r = np.cross(f, (0.0, 0.0, 1.0))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    yaw = (np.arange(w) - w / 2 + 0.5) * (span / w)
    lift = (h / 2 - np.arange(h)) * (span / w)
    d = (np.sin(yaw)[None, :, None] * r + np.cos(yaw)[None, :, None] * f + lift[:, None, None] * u)
    return np.ascontiguousarray(d, np.float32)


def _context(L, cam, ht, tex):
    ctx = L.vox_make_context_headless(W, H)
    assert ctx
    L.vox_context_set_camera(ctx, cam.obj)
    L.vox_context_set_scene(ctx, ht.ptr)
    L.vox_context_set_texture(ctx, tex.ctypes.data_as(C.c_void_p))
    return ctx


def _frame(L, ctx):
    L.vox_render(ctx)
    assert L.vox_context_status(ctx) == 0
    L.vox_redraw(ctx)
    px = np.ctypeslib.as_array(C.cast(L.vox_context_pixels(ctx), C.POINTER(C.c_uint32)), (W * H,))
    return px.reshape(H, W).copy()


def test_simple_camera_behind_a_foreign_iface_draws_its_own_frame(scene):
    """The host asks the camera for every direction; the frame is the one the
    built-in class draws (its directions computed on the device)."""
    vg, wl, ht, dt = scene
    L = vg.lib()
    cam = _camera(0)
    tex = wl.texture32(7)
    fc = ForeignCamera(cam, cam.screen2world)
    ctx = _context(L, cam, ht, tex)
    try:
        for q in QUALITIES:
            assert L.vox_context_set_quality(ctx, q) == 1
            before = fc.calls
            img = _frame(L, ctx)
            assert fc.calls - before == W * H
            assert np.array_equal(img, orc.render_quality(ht.ptr, cam.state(), W, H, q, tex)[0])
            assert np.array_equal(img, dt.render_quality(cam.gpu_struct(), W, H, q, tex))
    finally:
        L.vox_destroy_context(ctx)
        fc.close()


@pytest.mark.parametrize("kind", [0, 1])
def test_foreign_projection_equals_oracle_in_every_quality(scene, kind):
    """A cylindrical panorama on top of a simple or doom camera object (its
    position and window handling kept): every quality as the oracle draws it
    from the same directions."""
    vg, wl, ht, dt = scene
    L = vg.lib()
    pos = (120.0, -70.0, 90.0)
    cam = _camera(kind, pos=pos)
    table = panorama(pos, (32.0, 32.0, 32.0))
    tex = wl.texture32(3)
    fc = ForeignCamera(cam, lambda x, y: table[y, x])
    ctx = _context(L, cam, ht, tex)
    state = dict(kind=2, position=cam.position(), rays=table)
    try:
        hits = 0
        for q in QUALITIES:
            assert L.vox_context_set_quality(ctx, q) == 1
            img = _frame(L, ctx)
            ref, _ = orc.render_quality(ht.ptr, state, W, H, q, tex)
            assert np.array_equal(img, ref)
            hits += int((img != 0).sum())
        assert hits > W * H // 10   # the panorama sees the scene
    finally:
        L.vox_destroy_context(ctx)
        fc.close()


def test_foreign_projection_lit(scene):
    """With a light manager: colours as the oracle's lit get_color, also after
    a light is removed."""
    vg, wl, ht, dt = scene
    L = vg.lib()
    rng = np.random.default_rng(11)
    M, O = vg.LightManager(), orc.OracleLights()
    assert M.ambient((0.15, 0.1, 0.2)) and O.ambient((0.15, 0.1, 0.2))
    live = []
    for _ in range(60):
        c = rng.uniform(-10, 74, 3).astype(np.float32)
        r = float(rng.uniform(3, 30))
        col = rng.uniform(0, 1, 3).astype(np.float32)
        a = M.insert(c, r, col)
        assert a == O.insert(c, r, col)
        if a:
            live.append((c, r))
    pos = (110.0, 100.0, 70.0)
    cam = _camera(0, pos=pos)
    table = panorama(pos, (32.0, 32.0, 32.0), span=1.8)
    tex = wl.texture32(5)
    fc = ForeignCamera(cam, lambda x, y: table[y, x])
    ctx = _context(L, cam, ht, tex)
    L.vox_context_set_light_manager(ctx, M.ptr)
    state = dict(kind=2, position=cam.position(), rays=table)
    try:
        for q in (0, 2 | 8):
            assert L.vox_context_set_quality(ctx, q) == 1
            assert np.array_equal(_frame(L, ctx), orc.render_lit(ht.ptr, state, W, H, q, tex, O))
            c, r = live.pop()
            assert M.delete(c, r) and O.delete(c, r)
            assert np.array_equal(_frame(L, ctx), orc.render_lit(ht.ptr, state, W, H, q, tex, O))
    finally:
        L.vox_context_set_light_manager(ctx, None)
        L.vox_destroy_context(ctx)
        fc.close()


def test_render_rays_device(scene):
    """vox_cuda_render_rays_device on device buffers: the oracle's frame for
    every quality; a simple camera's own directions give its BEST frame; bad
    arguments are refused."""
    vg, wl, ht, dt = scene
    pos = (40.0, -60.0, 120.0)
    table = panorama(pos, (30.0, 34.0, 28.0), w=256, h=96, span=math.pi)
    tex = wl.texture32(9)
    d_dirs = torch.from_numpy(table).cuda()
    d_tex = torch.from_numpy(tex).cuda()
    d_argb = torch.full((96, 256), 0x5A5A5A5A, dtype=torch.int32, device="cuda")
    state = dict(kind=2, position=np.array(pos, np.float32), rays=table)
    for q in QUALITIES:
        dt.render_rays_device(pos, d_dirs, 256, 96, q, d_tex, d_argb)
        torch.cuda.synchronize()
        img = d_argb.cpu().numpy().view(np.uint32)
        assert np.array_equal(img, orc.render_quality(ht.ptr, state, 256, 96, q, tex)[0])

    cam = _camera(1, w=256, h=96)
    own = np.array([[cam.screen2world(x, y) for x in range(256)] for y in range(96)], np.float32)
    dt.render_rays_device(cam.position(), torch.from_numpy(own).cuda(), 256, 96, 0, d_tex, d_argb)
    torch.cuda.synchronize()
    assert np.array_equal(d_argb.cpu().numpy().view(np.uint32), dt.render(cam.gpu_struct(), 256, 96, tex))

    with pytest.raises(vg.VoxCudaError) as e:
        dt.render_rays_device(pos, None, 256, 96, 0, d_tex, d_argb)
    assert e.value.code == -1
    with pytest.raises(vg.VoxCudaError) as e:
        dt.render_rays_device(pos, d_dirs, 250, 96, 0, d_tex, d_argb)
    assert e.value.code == -7
    with pytest.raises(vg.VoxCudaError) as e:
        dt.render_rays_device(pos, d_dirs, 256, 96, 3, d_tex, d_argb)
    assert e.value.code == -1


def test_render_rays_empty_tree(scene):
    vg, wl, ht, dt = scene
    empty = vg.DeviceTree(None)
    d_dirs = torch.ones((32, 64, 3), dtype=torch.float32, device="cuda")
    d_tex = torch.zeros(32768, dtype=torch.uint8, device="cuda")
    d_argb = torch.full((32, 64), 7, dtype=torch.int32, device="cuda")
    for q in QUALITIES:
        empty.render_rays_device((0, 0, 0), d_dirs, 64, 32, q, d_tex, d_argb)
        torch.cuda.synchronize()
        assert (d_argb == 0).all()
