"""Host-side tree construction (vox_make_tree) and the built-in cameras,
against the reference's outputs (no GPU needed)."""
import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import dumps_equal, load, tree_dump
from voxvision_gb300 import HostTree, set_voxel_size
from voxvision_gb300 import workloads as wl
from voxvision_gb300.cameras import HostCamera

BUILT = ["ball12", "overflow", "voxsize", "dense", "holes", "cloud48"]


@pytest.mark.parametrize("case", BUILT)
def test_make_tree_matches_reference(case):
    g = load(case)
    set_voxel_size(tuple(g["voxel"]))
    t = HostTree.from_voxels(g["voxels"])
    ok, key = dumps_equal(orc.dump_tree(t.ptr), tree_dump(g))
    set_voxel_size((1, 1, 1))
    assert ok, f"tree differs from the reference's in {key}"


def test_make_tree_render64_volume():
    g = load("render64")
    set_voxel_size((1, 1, 1))
    t = HostTree.from_voxels(g["voxels"].astype(np.float32))
    ok, key = dumps_equal(orc.dump_tree(t.ptr), tree_dump(g))
    assert ok, key


@pytest.mark.parametrize("n,seed,solid", [(256, 2, 0.08)] + list(wl.BATCH_TREES))
def test_make_tree_matches_oracle_on_noise_volumes(n, seed, solid):
    """The benchmark's trees: the 256^3 orbit volume and the four trees of the
    mixed-camera batch (64^3 .. 512^3, 13.9 M voxels), node for node."""
    set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    vox = wl.voxels_from_mask(wl.noise_volume(n, seed, solid))
    a = HostTree.from_voxels(vox)
    b = orc.OracleTree.from_voxels(vox)
    ok, key = dumps_equal(orc.dump_tree(a.ptr), b.dump())
    assert ok, key


def test_empty_and_single():
    set_voxel_size((1, 1, 1))
    assert HostTree.from_voxels(np.zeros((0, 3), np.float32)).ptr is None
    t = HostTree.from_voxels(np.array([[1, 2, 3]], np.float32))
    d = orc.dump_tree(t.ptr)
    assert d["flags"].tolist() == [2] and d["dots_num"].tolist() == [1]


def _camera_from_golden(g, i):
    kind = int(g[f"c{i}_kind"])
    w, h = (int(x) for x in g[f"c{i}_wh"])
    cam = HostCamera(kind)
    cam.set_fov(float(g[f"c{i}_fov"]))
    cam.set_window_size(w, h)
    cam.set_position(g[f"c{i}_setpos"])
    if not np.isnan(g[f"c{i}_setrot"]).any():
        cam.set_rotation(g[f"c{i}_setrot"])
    if not np.isnan(g[f"c{i}_lookat"]).any():
        cam.look_at(g[f"c{i}_lookat"])
    return cam


def test_cameras_match_reference_plugins():
    """Same set-up calls -> same camera state as the reference's plugins (to
    libm rounding of sinf/cosf/atan2f), and bit-identical screen2world rays
    whenever the state is bit-identical."""
    g = load("cameras")
    for i in range(int(g["ncams"])):
        cam = _camera_from_golden(g, i)
        st = cam.state()
        for k in ("position", "rotation", "mul", "xsub", "ysub", "sinphi", "cosphi", "k"):
            if f"c{i}_{k}" in g:
                np.testing.assert_allclose(np.asarray(st[k], np.float64), g[f"c{i}_{k}"], rtol=2e-6,
                                           atol=2e-7, err_msg=f"camera {i} {k}")
        exact = all(np.array_equal(np.asarray(st[k], np.float32).view(np.uint32),
                                   np.asarray(g[f"c{i}_{k}"], np.float32).view(np.uint32))
                    for k in ("position", "rotation", "mul", "xsub", "ysub", "sinphi", "cosphi", "k")
                    if f"c{i}_{k}" in g)
        for (x, y), ray in zip(g[f"c{i}_pixels"], g[f"c{i}_rays"]):
            r = cam.screen2world(int(x), int(y))
            if exact:
                assert np.array_equal(r.view(np.uint32), ray.view(np.uint32)), (i, x, y)
            else:
                np.testing.assert_allclose(r, ray, rtol=1e-5, atol=1e-6)


def test_camera_reference_expectations():
    """tests.c:661-709: a fresh camera looks along +y; after a rotation of pi/2
    about z it looks along -x; moving along the view axis moves to (-1, 0, 0)."""
    for kind in (0, 1):
        cam = HostCamera(kind)
        cam.set_position((0, 0, 0))
        cam.set_window_size(100, 100)
        np.testing.assert_allclose(cam.screen2world(50, 50), [0, 1, 0], atol=1e-5)
        cam.set_rotation((0, 0, np.pi / 2))
        np.testing.assert_allclose(cam.screen2world(50, 50), [-1, 0, 0], atol=1e-5)
        cam.rotate((0, np.pi / 2, 0))
        np.testing.assert_allclose(cam.screen2world(50, 50), [-1, 0, 0], atol=1e-5)
        cam.move((0, 1, 0))
        np.testing.assert_allclose(cam.position(), [-1, 0, 0], atol=1e-5)


def test_camera_look_at_reference_expectations():
    """tests.c:712-733: after look_at, the centre ray of either class passes
    through the target (the reference's hit_dot at approx_check 0.5)."""
    for kind in (0, 1):
        cam = HostCamera(kind)
        cam.set_window_size(100, 100)
        pos, target = np.array([-100, 20, -20], np.float32), np.zeros(3, np.float32)
        cam.set_position(pos)
        cam.look_at(target)
        d = cam.screen2world(50, 50)
        t = np.float32((target[0] - pos[0]) / d[0])
        assert t >= 0
        hit = np.array([target[0], d[1] * t + pos[1], d[2] * t + pos[2]], np.float32)
        assert np.max(np.abs(hit - target)) <= 0.5


def test_camera_look_at_then_move():
    """tests.c:735-759: looking at the default direction and moving by (1, 0, 0)
    lands at (1, 0, 0), twice in a row."""
    cam = HostCamera(0)
    for _ in range(2):
        cam.set_position((0, 0, 0))
        cam.look_at(np.array([0, 1, 0], np.float32))
        cam.move((1, 0, 0))
        np.testing.assert_allclose(cam.position(), [1, 0, 0], atol=1e-5)


def test_camera_copy_construction():
    """tests.c:761-776: construct_camera(camera) copies the camera's state."""
    import ctypes as C
    from voxvision_gb300 import lib
    from voxvision_gb300.cameras import CONS, DOTM, DESTROY
    cam = HostCamera(0)
    cam.set_position((10, 110, 1110))
    cam.set_window_size(100, 100)
    tbl = C.cast(lib().vox_camera_methods(b"simple-camera"), C.POINTER(C.c_void_p * 10)).contents
    copy = CONS(tbl[8])(cam.obj)
    assert copy
    pos = np.zeros(3, np.float32)
    DOTM(tbl[6])(copy, pos.ctypes.data_as(C.c_void_p))
    np.testing.assert_allclose(pos, [10, 110, 1110], atol=1e-5)
    DESTROY(tbl[9])(copy)


@pytest.mark.parametrize("case", BUILT + ["g676d50c"])
def test_flattened_image_is_sound(case):
    """vox_cuda_tree_measure flattens the tree on the host, walks the device
    image it would upload (every offset in range, every node reached once)
    and reports the reference tree's node census."""
    from tests.helpers import load as _load
    from voxvision_gb300 import measure_tree
    g = _load(case)
    set_voxel_size(tuple(g["voxel"]))
    orc.set_voxel(tuple(g["voxel"]))
    if "voxels" in g:
        t = HostTree.from_voxels(g["voxels"])
    else:
        t = orc.OracleTree.from_dump(tree_dump(g))
    info = measure_tree(t.ptr)
    d = tree_dump(g)
    f = d["flags"]
    assert info["nodes"] == len(f)
    assert info["inner"] == int(((f & 3) == 0).sum())
    assert info["dense_leaves"] == int(((f & 2) != 0).sum())
    assert info["leaves"] == int(((f & 1) != 0).sum())
    assert info["dots"] == len(d["dots"])
    set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))


def test_flattened_image_large_volume():
    from voxvision_gb300 import measure_tree
    set_voxel_size((1, 1, 1))
    vox = wl.voxels_from_mask(wl.noise_volume(256, 2, 0.08))
    t = HostTree.from_voxels(vox)
    info = measure_tree(t.ptr)
    assert info["depth"] >= 6 and info["nodes"] > 100000
    assert info["device_bytes"] < 64 << 20
