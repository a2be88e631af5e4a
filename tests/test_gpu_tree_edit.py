"""Edited trees on the GPU: after vox_insert_voxel / vox_delete_voxel,
vox_cuda_tree_refresh makes the device copy draw the edited tree exactly as
the oracle does (also when the tree grows past its old device allocation),
and the drop-in single-query search sees edits made through the library
without vox_cuda_forget_tree."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as vg
    vg.set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    return vg


def _frame(vg, dt, root, cam, tex):
    img = dt.render(cam.gpu_struct(), 320, 240, tex)
    ref, _ = orc.render_best(root.value, cam.state(), 320, 240, tex)
    return img, ref


def test_refresh_after_edits(lib):
    vg = lib
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    L = vg.lib()
    vox = np.ascontiguousarray(wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20))).copy()
    root = C.c_void_p(L.vox_make_tree(vox.ctypes.data_as(C.c_void_p), vox.shape[0]))
    dt = vg.DeviceTree(root.value)
    cam = HostCamera(0)
    cam.set_window_size(320, 240)
    cam.set_position((150.0, -90.0, 100.0))
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    tex = wl.texture32(7)
    img, ref = _frame(vg, dt, root, cam, tex)
    assert np.array_equal(img, ref)
    rng = np.random.default_rng(12)
    for batch in range(3):
        n_ins = (200, 3000, 100)[batch]                # the second batch grows the tree past its old pool
        for _ in range(n_ins):
            a = rng.integers(-8, 72, 3).astype(np.float32)
            L.vox_insert_voxel(C.byref(root), a.ctypes.data_as(C.c_void_p))
        for _ in range(400):
            a = vox[int(rng.integers(len(vox)))].copy()
            L.vox_delete_voxel(C.byref(root), a.ctypes.data_as(C.c_void_p))
        vg.check(L.vox_cuda_tree_refresh(dt.h, root), "vox_cuda_tree_refresh")
        img, ref = _frame(vg, dt, root, cam, tex)
        assert np.array_equal(img, ref), f"batch {batch}: {(img != ref).sum()} pixels differ"
        # rays through the batch entry point report the edited tree's leaves
        o = np.tile(np.float32([150, -90, 100]), (500, 1))
        d = (rng.uniform(-1, 1, (500, 3)) + np.float32([-0.7, 0.8, -0.45])).astype(np.float32)
        leaf, _, pts = dt.rays(o, d)
        rl, _, rp, _ = orc.ray_batch(root.value, o, d)
        assert np.array_equal(leaf, rl)
    dt.close()
    L.vox_destroy_tree(root)


def test_dropin_search_sees_library_edits(lib):
    vg = lib
    L = vg.lib()
    root = C.c_void_p(None)
    for x in range(10):
        L.vox_insert_voxel_coord(C.byref(root), float(x), 0.0, 0.0)
    o = np.float32([-5, 0.5, 0.5]); d = np.float32([1, 0, 0]); res = np.zeros(3, np.float32)
    hit = L.vox_ray_tree_intersection(root, o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                                      res.ctypes.data_as(C.c_void_p))
    assert hit and res[0] == 0.0
    L.vox_delete_voxel_coord(C.byref(root), 0.0, 0.0, 0.0)      # drops the cached device copy
    hit = L.vox_ray_tree_intersection(root, o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                                      res.ctypes.data_as(C.c_void_p))
    assert hit and res[0] == 1.0
    L.vox_insert_voxel_coord(C.byref(root), -3.0, 0.0, 0.0)
    c = np.float32([-2.5, 0.5, 0.5])
    assert L.vox_tree_ball_collidep(root, c.ctypes.data_as(C.c_void_p), C.c_float(0.6)) == 1
    L.vox_destroy_tree(root)
