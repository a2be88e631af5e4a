"""Trees built on the GPU (vox_cuda_tree_build*, vox_cuda_tree_build_raw,
vox_cuda_read_raw_data): the device image must equal the host build
(vox_make_tree, restated from tree.c and pinned to the reference's golden
trees) followed by vox_cuda_tree_upload, byte for byte -- records, voxel runs
and the pre-order id map -- and the golden trees of the reference decode from
it directly."""
import ctypes as C
import os

import numpy as np
import pytest

from tests.helpers import dumps_equal, image_dump, load, tree_dump

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
    yield m
    m.set_voxel_size((1, 1, 1))


def _host_image(vg, vox):
    h = vg.HostTree.from_voxels(vox)
    dt = vg.DeviceTree(h.ptr)
    img = dt.image()
    info = dt.info()
    dt.close()
    h.close()
    return img, info


def _same_build(vg, vox, voxel=(1, 1, 1)):
    vg.set_voxel_size(voxel)
    try:
        (hu, hi), hinfo = _host_image(vg, vox)
        dt = vg.DeviceTree.build(vox)
        du, di = dt.image()
        dinfo = dt.info()
        dt.close()
    finally:
        vg.set_voxel_size((1, 1, 1))
    assert du.shape == hu.shape and di.shape == hi.shape, (du.shape, hu.shape, di.shape, hi.shape)
    bad = np.nonzero((du != hu).any(axis=1))[0]
    assert bad.size == 0, f"{bad.size} image units differ, first at {bad[:5]}"
    assert np.array_equal(di, hi)
    for k in ("nodes", "inner", "leaves", "dense_leaves", "dots", "depth"):
        assert dinfo[k] == hinfo[k], (k, dinfo[k], hinfo[k])
    return dinfo


@pytest.mark.parametrize("case", ["ball12", "overflow", "voxsize", "dense", "holes", "cloud48", "render64"])
def test_build_matches_reference_golden_trees(vg, case):
    g = load(case)
    voxel = tuple(float(x) for x in g["voxel"])
    vox = np.ascontiguousarray(g["voxels"], np.float32)
    _same_build(vg, vox, voxel)
    vg.set_voxel_size(voxel)
    try:
        dt = vg.DeviceTree.build(vox)
        u, ids = dt.image()
        dt.close()
    finally:
        vg.set_voxel_size((1, 1, 1))
    ok, key = dumps_equal(image_dump(u, ids, voxel), tree_dump(g))
    assert ok, f"device-built tree differs from the reference's in {key}"


@pytest.mark.parametrize("n,seed,solid", [(64, 3, 0.10), (128, 4, 0.25), (256, 2, 0.08)])
def test_build_noise_volumes(vg, n, seed, solid):
    from voxvision_gb300 import workloads as wl
    vox = wl.voxels_from_mask(wl.noise_volume(n, seed, solid))
    info = _same_build(vg, vox)
    assert info["inner"] > 0


def test_build_large_set_rounds_its_sums(vg):
    """4.2M voxels: the root's coordinate sums pass 2^30, so most additions
    round; the chunked two-state sums must round exactly as the serial loop."""
    rng = np.random.default_rng(21)
    vox = np.unique(rng.integers(0, 400, (5_000_000, 3)), axis=0).astype(np.float32)
    vox = vox[rng.permutation(len(vox))]
    _same_build(vg, vox)


@pytest.mark.parametrize("voxel", [(0.37, 1.9, 2.5), (0.5, 0.25, 4.0)])
def test_build_non_grid_coordinates(vg, voxel):
    """Fractional voxel sizes and off-grid float coordinates: the differences
    summed for the centres have fraction bits at every binade."""
    rng = np.random.default_rng(5)
    g = rng.integers(-90, 90, (400_000, 3)).astype(np.float64)
    vox = (g * np.asarray(voxel) + rng.random((400_000, 3)) * 0.01).astype(np.float32)
    _same_build(vg, vox, voxel)


def test_build_edge_sets(vg):
    _same_build(vg, np.zeros((0, 3), np.float32))
    _same_build(vg, np.array([[1, 2, 3]], np.float32))
    # duplicates only: one overflowed leaf at the root
    _same_build(vg, np.tile(np.array([[4, 5, 6]], np.float32), (5000, 1)))
    # a full cube: one dense leaf
    _same_build(vg, np.mgrid[0:40, 0:40, 0:40].reshape(3, -1).T.astype(np.float32))
    # everything in one octant but one voxel; then the reverse order
    a = np.concatenate([np.mgrid[0:30, 0:30, 0:9].reshape(3, -1).T * 2, [[100, 100, 100]]]).astype(np.float32)
    _same_build(vg, a)
    _same_build(vg, a[::-1].copy())
    # negative and signed-zero coordinates, large magnitudes
    b = np.concatenate([np.mgrid[-20:20:3, -20:20:3, -20:20:3].reshape(3, -1).T, [[0, 0, 0]]]).astype(np.float32)
    b[-1] = [-0.0, -0.0, -0.0]
    _same_build(vg, b)
    _same_build(vg, (np.random.default_rng(3).integers(-2 ** 20, 2 ** 20, (50000, 3))).astype(np.float32))
    # many duplicates inside a larger set (overflowed leaves below the root)
    rng = np.random.default_rng(9)
    c = rng.integers(0, 50, (60000, 3)).astype(np.float32)
    _same_build(vg, c)


def test_built_tree_draws_like_uploaded(vg):
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    vox = wl.voxels_from_mask(wl.noise_volume(128, 6, 0.12))
    h = vg.HostTree.from_voxels(vox)
    up = vg.DeviceTree(h.ptr)
    bt = vg.DeviceTree.build(vox)
    assert bt.node(0) is None
    cam = HostCamera(0)
    cam.set_window_size(640, 480)
    cam.set_position((300.0, -180.0, 200.0))
    cam.look_at(np.array([64.0, 64.0, 64.0], np.float32))
    tex = wl.texture32(7)
    for q in (0, 2):
        a = up.render_quality(cam.gpu_struct(), 640, 480, q, tex)
        b = bt.render_quality(cam.gpu_struct(), 640, 480, q, tex)
        assert np.array_equal(a, b)
    rng = np.random.default_rng(4)
    o = (rng.random((20000, 3)) * 300 - 80).astype(np.float32)
    d = (rng.random((20000, 3)) - 0.5).astype(np.float32)
    la, _, pa = up.rays(o, d)
    lb, _, pb = bt.rays(o, d)
    assert np.array_equal(la, lb) and np.array_equal(pa.view(np.uint32), pb.view(np.uint32))


def test_build_device_input(vg):
    from voxvision_gb300 import workloads as wl
    vox = wl.voxels_from_mask(wl.noise_volume(96, 8, 0.2))
    t = torch.from_numpy(vox).cuda()
    bt = vg.DeviceTree.build_device(t)
    before = t.cpu().numpy()
    assert np.array_equal(before, vox), "the device set must not be modified"
    (hu, hi), _ = _host_image(vg, vox)
    du, di = bt.image()
    assert np.array_equal(du, hu) and np.array_equal(di, hi)


def _raw_host_image(vg, mask):
    from voxvision_gb300 import workloads as wl
    return _host_image(vg, wl.voxels_from_mask(mask))


def test_raw_reader_u8_band(vg):
    from voxvision_gb300 import workloads as wl
    vol = wl.value_noise_u8(128, 11)
    lo, hi = 100, 140
    dt = vg.DeviceTree.from_raw(vol.tobytes(), vol.shape, 1, lo, hi)
    (hu, hi_), _ = _raw_host_image(vg, (vol >= lo) & (vol <= hi))
    du, di = dt.image()
    assert np.array_equal(du, hu) and np.array_equal(di, hi_)


def test_raw_reader_u16_predicate_and_voxel_size(vg):
    from voxvision_gb300 import workloads as wl
    vol = (wl.value_noise_u8(96, 12).astype(np.uint16) * 251 + 7).astype(np.uint16)
    pred = lambda s: (s % 7) < 3 and s > 9000       # noqa: E731
    vg.set_voxel_size((0.5, 2.0, 1.25))
    try:
        dt = vg.DeviceTree.from_raw(vol.astype("<u2").tobytes(), vol.shape, 2, test=pred)
        du, di = dt.image()
        m = np.vectorize(pred)(vol)
        from voxvision_gb300 import workloads as w2
        (hu, hi), _ = _host_image(vg, w2.voxels_from_mask(m, (0.5, 2.0, 1.25)))
    finally:
        vg.set_voxel_size((1, 1, 1))
    assert np.array_equal(du, hu) and np.array_equal(di, hi)


def test_raw_reader_file_and_errors(vg, tmp_path):
    from voxvision_gb300 import workloads as wl
    vol = wl.value_noise_u8(64, 13)
    # 3-byte samples: value = b0 | b1 << 8 | b2 << 16 (datareader.c:61-72)
    raw = np.stack([vol, vol[::-1], np.full_like(vol, 1)], axis=-1)
    p = tmp_path / "vol.raw"
    p.write_bytes(raw.tobytes())
    val = vol.astype(np.uint32) | (vol[::-1].astype(np.uint32) << 8) | (1 << 16)
    lo, hi = (1 << 16) + 30000, (1 << 16) + 50000
    dt = vg.DeviceTree.read_raw(str(p), vol.shape, 3, lo, hi)
    (hu, hi_), _ = _raw_host_image(vg, (val >= lo) & (val <= hi))
    du, di = dt.image()
    assert np.array_equal(du, hu) and np.array_equal(di, hi_)
    with pytest.raises(vg.VoxCudaError, match="Wrong size of dataset"):
        vg.DeviceTree.read_raw(str(p), (64, 64, 63), 3, lo, hi)
    with pytest.raises(vg.VoxCudaError):
        vg.DeviceTree.read_raw(str(tmp_path / "missing.raw"), vol.shape, 1, 1, 2)
    # nothing solid: the empty tree
    e = vg.DeviceTree.read_raw(str(p), vol.shape, 3, 0, 0)
    assert e.info()["nodes"] == 0
