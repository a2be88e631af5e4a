"""GPU parity of lit frames: the library's light manager uploaded to the
device colours every hit as the oracle's restatement of get_color with a
light manager does (renderer.c:40-49, lights.c:91-116, mtree.c:463-493),
pixel for pixel, in every quality mode; after lights are removed or the
ambient light changes; and through the drop-in render context."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


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


def _lights(vg, n, seed, rmax=30.0, cmax=1.0):
    """The same insertion sequence into the library's manager and the oracle's."""
    rng = np.random.default_rng(seed)
    M, O = vg.LightManager(), orc.OracleLights()
    # a dim ambient light: with the default (1, 1, 1) every channel saturates
    assert M.ambient((0.15, 0.1, 0.2)) and O.ambient((0.15, 0.1, 0.2))
    live = []
    for _ in range(n):
        c = rng.uniform(-10, 74, 3).astype(np.float32)
        r = float(rng.uniform(3, rmax))
        col = rng.uniform(0, cmax, 3).astype(np.float32)
        a, b = M.insert(c, r, col), O.insert(c, r, col)
        assert a == b
        if a:
            live.append((c, r))
    return M, O, live


def _camera(vg, kind=0, w=336, h=200, pos=(150.0, -90.0, 100.0)):
    from voxvision_gb300.cameras import HostCamera
    cam = HostCamera(kind)
    cam.set_window_size(w, h)
    cam.set_position(pos)
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    return cam


@pytest.mark.parametrize("quality", [0, 1, 2, 2 | 4, 2 | 8])
def test_lit_frames_equal_oracle_in_every_quality(scene, quality):
    vg, wl, ht, dt = scene
    M, O, _ = _lights(vg, 150, 5, rmax=15.0, cmax=0.6)
    dl = M.upload()
    tex = wl.texture32(7)
    for kind in (0, 1):
        cam = _camera(vg, kind)
        img = dt.render_lit(cam.gpu_struct(), 336, 200, quality, tex, dl)
        ref = orc.render_lit(ht.ptr, cam.state(), 336, 200, quality, tex, O)
        assert (img != 0).any()
        assert np.array_equal(img, ref), f"{(img != ref).sum()} pixels differ"
    # the lights are really applied: hit pixels differ from grey texels, and
    # some of them from the ambient light alone
    grey = dt.render_lit(cam.gpu_struct(), 336, 200, quality, tex, None)
    A = vg.LightManager()
    assert A.ambient((0.15, 0.1, 0.2))
    ambient = dt.render_lit(cam.gpu_struct(), 336, 200, quality, tex, A.upload())
    hit = img != 0
    assert (grey[hit] != img[hit]).mean() > 0.5
    assert (ambient[hit] != img[hit]).mean() > 0.05


def test_lights_follow_changes_after_upload(scene):
    vg, wl, ht, dt = scene
    M, O, live = _lights(vg, 400, 6, rmax=20.0)
    tex = wl.texture32(7)
    cam = _camera(vg, 0, 256, 192, (-60.0, 140.0, 80.0))
    for step in range(3):
        for c, r in live[step::3][:60]:
            assert M.delete(c, r) and O.delete(c, r)
        amb = (0.1 * step, 0.3, 0.05 * step)
        assert M.ambient(amb) and O.ambient(amb)
        dl = M.upload()
        img = dt.render_lit(cam.gpu_struct(), 256, 192, 0, tex, dl)
        ref = orc.render_lit(ht.ptr, cam.state(), 256, 192, 0, tex, O)
        assert np.array_equal(img, ref), f"step {step}: {(img != ref).sum()} pixels differ"
        dl.close()


def test_ambient_only_and_saturating_lights(scene):
    vg, wl, ht, dt = scene
    tex = wl.texture32(7)
    cam = _camera(vg, 1)
    M, O = vg.LightManager(), orc.OracleLights()
    assert M.ambient((0.25, 0.5, 1.0)) and O.ambient((0.25, 0.5, 1.0))
    img = dt.render_lit(cam.gpu_struct(), 336, 200, 0, tex, M.upload())
    assert np.array_equal(img, orc.render_lit(ht.ptr, cam.state(), 336, 200, 0, tex, O))
    for i in range(40):                               # many bright overlapping lights: sums above 1
        c = (20.0 + i, 30.0 - i * 0.5, 25.0 + (i % 7))
        assert M.insert(c, 60.0, (1.0, 0.9, 0.8)) and O.insert(c, 60.0, (1.0, 0.9, 0.8))
    img = dt.render_lit(cam.gpu_struct(), 336, 200, 2, tex, M.upload())
    ref = orc.render_lit(ht.ptr, cam.state(), 336, 200, 2, tex, O)
    assert np.array_equal(img, ref)


def test_render_context_with_light_manager(scene):
    """vox_context_set_light_manager: vox_render colours with the manager and
    follows its changes at the next frame."""
    vg, wl, ht, dt = scene
    L = vg.lib()
    M, O, live = _lights(vg, 200, 8)
    ctx = L.vox_make_context_headless(320, 240)
    cam = _camera(vg, 0, 320, 240)
    L.vox_context_set_camera(ctx, cam.obj)
    L.vox_context_set_scene(ctx, ht.ptr)
    tex = wl.texture32(7)
    L.vox_context_set_texture(ctx, tex.ctypes.data_as(C.c_void_p))
    L.vox_context_set_light_manager(ctx, M.ptr)
    for q in (0, 2):
        assert L.vox_context_set_quality(ctx, q) == 1
        for rnd in range(2):
            L.vox_render(ctx)
            L.vox_redraw(ctx)
            assert L.vox_context_status(ctx) == 0
            px = np.ctypeslib.as_array(C.cast(L.vox_context_pixels(ctx), C.POINTER(C.c_uint32)), (240 * 320,))
            ref = orc.render_lit(ht.ptr, cam.state(), 320, 240, q, tex, O)
            assert np.array_equal(px.reshape(240, 320), ref)
            c, r = live.pop()
            assert M.delete(c, r) and O.delete(c, r)   # seen by the next vox_render
    L.vox_context_set_light_manager(ctx, None)
    L.vox_render(ctx)
    L.vox_redraw(ctx)
    px = np.ctypeslib.as_array(C.cast(L.vox_context_pixels(ctx), C.POINTER(C.c_uint32)), (240 * 320,))
    assert np.array_equal(px.reshape(240, 320), orc.render_quality(ht.ptr, cam.state(), 320, 240, 2, tex)[0])
    L.vox_destroy_context(ctx)
