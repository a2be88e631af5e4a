"""vox_make_tree built on the GPU (sets of at least vox_cuda_make_tree_gpu_min
voxels): the host tree is the host build's node for node, the caller's set is
left in the same order, and the device copy kept for the first upload equals
a fresh flatten of the tree -- unless an edit or a new voxel size made it
stale, in which case it is not used."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import dumps_equal, load

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def vg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as m
    m.set_voxel_size((1, 1, 1))
    L = m.lib()
    old = L.vox_cuda_make_tree_gpu_min(0)   # every build on the GPU in this module
    yield m
    L.vox_cuda_make_tree_gpu_min(old)
    m.set_voxel_size((1, 1, 1))


def _both(vg, vox, voxel=(1, 1, 1)):
    """(host-build root, its set after the build), (GPU-build root, its set)."""
    L = vg.lib()
    vg.set_voxel_size(voxel)
    a = np.ascontiguousarray(vox, np.float32).copy()
    b = a.copy()
    ra = L.vox_make_tree_host(a.ctypes.data_as(C.c_void_p), a.shape[0])
    rb = L.vox_make_tree(b.ctypes.data_as(C.c_void_p), b.shape[0])
    return (ra, a), (rb, b)


def _image(vg, root):
    dt = vg.DeviceTree(root)
    img = dt.image()
    nodes = [dt.node(i) for i in range(0, dt.info()["nodes"], 997)]
    dt.close()
    return img, nodes


SETS = {
    "noise64": lambda wl: wl.voxels_from_mask(wl.noise_volume(64, 3, 0.10)),
    "noise256": lambda wl: wl.voxels_from_mask(wl.noise_volume(256, 2, 0.08)),
    "random_dups": lambda wl: np.random.default_rng(9).integers(0, 50, (60000, 3)).astype(np.float32),
    "offgrid": lambda wl: (np.random.default_rng(5).integers(-90, 90, (200000, 3)) * 0.37
                           + np.random.default_rng(6).random((200000, 3)) * 0.01).astype(np.float32),
}


@pytest.mark.parametrize("name", list(SETS))
def test_gpu_make_tree_equals_host_build(vg, name):
    from voxvision_gb300 import workloads as wl
    voxel = (0.37, 1.9, 2.5) if name == "offgrid" else (1, 1, 1)
    (ra, a), (rb, b) = _both(vg, SETS[name](wl), voxel)
    try:
        ok, key = dumps_equal(orc.dump_tree(ra), orc.dump_tree(rb))
        assert ok, f"GPU-built host tree differs from the host build in {key}"
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "the set is left in another order"
        (ia, _), (ib, nb) = _image(vg, ra), _image(vg, rb)      # rb's first upload takes the kept copy
        assert np.array_equal(ia[0], ib[0]) and np.array_equal(ia[1], ib[1])
        (ic, nc) = _image(vg, rb)                                # a second upload flattens afresh
        assert np.array_equal(ib[0], ic[0]) and nb == nc
    finally:
        vg.lib().vox_destroy_tree(ra)
        vg.lib().vox_destroy_tree(rb)
        vg.set_voxel_size((1, 1, 1))


@pytest.mark.parametrize("case", ["ball12", "overflow", "voxsize", "dense", "holes", "cloud48"])
def test_gpu_make_tree_matches_reference_golden(vg, case):
    from tests.helpers import tree_dump
    g = load(case)
    voxel = tuple(float(x) for x in g["voxel"])
    (ra, a), (rb, b) = _both(vg, g["voxels"], voxel)
    try:
        ok, key = dumps_equal(orc.dump_tree(rb), tree_dump(g))
        assert ok, f"differs from the reference's tree in {key}"
    finally:
        vg.lib().vox_destroy_tree(ra)
        vg.lib().vox_destroy_tree(rb)
        vg.set_voxel_size((1, 1, 1))


def test_kept_copy_is_not_used_after_an_edit_or_a_new_voxel_size(vg):
    from voxvision_gb300 import workloads as wl
    L = vg.lib()
    vox = wl.voxels_from_mask(wl.noise_volume(64, 7, 0.15))
    # an edit drops the kept copy: the upload shows the edited tree
    (ra, _), (rb, _) = _both(vg, vox)
    root = C.c_void_p(rb)
    v = np.array([70.0, 70.0, 70.0], np.float32)
    assert L.vox_insert_voxel(C.byref(root), v.ctypes.data_as(C.c_void_p)) == 1
    ra_box = C.c_void_p(ra)
    assert L.vox_insert_voxel(C.byref(ra_box), v.ctypes.data_as(C.c_void_p)) == 1
    (ia, _), (ib, _) = _image(vg, ra_box.value), _image(vg, root.value)
    assert np.array_equal(ia[0], ib[0]) and np.array_equal(ia[1], ib[1])
    L.vox_destroy_tree(ra_box.value)
    L.vox_destroy_tree(root.value)
    # another voxel size at upload: the copy made for the old one is not used
    (ra, _), (rb, _) = _both(vg, vox)
    vg.set_voxel_size((2, 2, 2))
    try:
        (ia, _), (ib, _) = _image(vg, ra), _image(vg, rb)
        assert np.array_equal(ia[0], ib[0])
    finally:
        vg.set_voxel_size((1, 1, 1))
        L.vox_destroy_tree(ra)
        L.vox_destroy_tree(rb)


def test_dropin_query_after_gpu_make_tree(vg):
    """A single drop-in query on a GPU-built tree returns the host tree's own
    leaf pointers, as the reference's search does."""
    from voxvision_gb300 import workloads as wl
    L = vg.lib()
    vox = wl.voxels_from_mask(wl.noise_volume(64, 8, 0.2))
    (ra, _), (rb, _) = _both(vg, vox)
    try:
        rng = np.random.default_rng(3)
        for _ in range(50):
            o = (rng.random(3) * 120 - 28).astype(np.float32)
            d = (rng.random(3) - 0.5).astype(np.float32)
            pa, pb = np.zeros(3, np.float32), np.zeros(3, np.float32)
            na = L.vox_ray_tree_intersection(C.c_void_p(ra), o.ctypes.data_as(C.c_void_p),
                                             d.ctypes.data_as(C.c_void_p), pa.ctypes.data_as(C.c_void_p))
            nb = L.vox_ray_tree_intersection(C.c_void_p(rb), o.ctypes.data_as(C.c_void_p),
                                             d.ctypes.data_as(C.c_void_p), pb.ctypes.data_as(C.c_void_p))
            assert (na is None) == (nb is None)
            if na is not None:
                assert np.array_equal(pa.view(np.uint32), pb.view(np.uint32))
                fa = orc.dump_tree(na)["boxes"][0]
                fb = orc.dump_tree(nb)["boxes"][0]
                assert np.array_equal(fa, fb)
    finally:
        L.vox_destroy_tree(ra)
        L.vox_destroy_tree(rb)
