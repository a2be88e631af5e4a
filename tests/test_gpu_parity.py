"""GPU parity: every result of the CUDA path through the C ABI equals the
reference's (golden vectors) and the oracle's, bit for bit.

Leaf ids, voxel slots and ball booleans are compared exactly; intersection
points bit-exactly (all NaNs counted equal), which is stricter than the
1e-5 relative tolerance the drop-in promises; frames pixel-exactly.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import MISS, TREE_CASES, load, same_points, tree_dump

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300  # noqa: F401


def vg():
    import voxvision_gb300
    return voxvision_gb300


def _host_tree(g):
    """(host tree object, pointer): the library's vox_make_tree when the case
    has a voxel set, else the reference's insertion-built tree rebuilt from
    its dump (same node layout)."""
    vg().set_voxel_size(tuple(g["voxel"]))
    orc.set_voxel(tuple(g["voxel"]))
    if "voxels" in g:
        t = vg().HostTree.from_voxels(g["voxels"].astype(np.float32))
        return t, t.ptr
    t = orc.OracleTree.from_dump(tree_dump(g))
    return t, t.ptr


def _reset_voxel():
    vg().set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))


@pytest.mark.parametrize("case", TREE_CASES)
def test_rays_match_reference_golden(case):
    g = load(case)
    ht, ptr = _host_tree(g)
    dt = vg().DeviceTree(ptr)
    leaf, slot, pts = dt.rays(g["ray_origins"], g["ray_dirs"])
    assert np.array_equal(leaf, g["ray_leaf"]), f"{(leaf != g['ray_leaf']).sum()} leaf ids differ"
    hit = leaf != MISS
    ok, nbad = same_points(pts, g["ray_points"], hit)
    assert ok, f"{nbad} points differ"
    # the winning voxel, against the oracle's leaf loop
    _, oslot, _, _ = orc.ray_batch(ptr, g["ray_origins"], g["ray_dirs"])
    assert np.array_equal(slot, oslot)
    _reset_voxel()


@pytest.mark.parametrize("case", TREE_CASES)
def test_leaf_rooted_rays_match_reference_golden(case):
    g = load(case)
    if "root_ids" not in g:
        pytest.skip("no leaves")
    ht, ptr = _host_tree(g)
    dt = vg().DeviceTree(ptr)
    leaf, slot, pts = dt.rays(g["root_origins"], g["root_dirs"], roots=g["root_ids"])
    assert np.array_equal(leaf, g["root_leaf"])
    ok, nbad = same_points(pts, g["root_points"], leaf != MISS)
    assert ok, f"{nbad} points differ"
    _reset_voxel()


@pytest.mark.parametrize("case", TREE_CASES)
def test_balls_match_reference_golden(case):
    g = load(case)
    ht, ptr = _host_tree(g)
    dt = vg().DeviceTree(ptr)
    hit = dt.balls(g["ball_centres"], g["ball_radii"])
    assert np.array_equal(hit, g["ball_hit"])
    _reset_voxel()


@pytest.mark.parametrize("case", TREE_CASES)
def test_small_host_batches_match_reference_golden(case):
    """Host batches of up to 256 queries take the page-locked small-batch
    path (the drop-in single queries' path): the golden rays, leaf-rooted
    rays and balls in batches of 1, 37 and 256 give the reference's answers,
    and the points of misses keep the caller's values."""
    g = load(case)
    ht, ptr = _host_tree(g)
    dt = vg().DeviceTree(ptr)
    L = vg().lib()
    for size in (1, 37, 256):
        for i in range(0, min(len(g["ray_origins"]), 3 * size), size):
            o = np.ascontiguousarray(g["ray_origins"][i:i + size]); d = np.ascontiguousarray(g["ray_dirs"][i:i + size])
            n = len(o)
            leaf = np.empty(n, np.uint32); slot = np.empty(n, np.uint8); pts = np.full((n, 3), 7.0, np.float32)
            assert L.vox_cuda_ray_batch(dt.h, o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p), None, n,
                                        leaf.ctypes.data_as(C.c_void_p), slot.ctypes.data_as(C.c_void_p),
                                        pts.ctypes.data_as(C.c_void_p), None) == 0
            assert np.array_equal(leaf, g["ray_leaf"][i:i + n])
            hit = leaf != MISS
            assert same_points(pts, g["ray_points"][i:i + n], hit)[0]
            assert np.all(pts[~hit] == 7.0)
        if "root_ids" in g:
            for i in range(0, min(len(g["root_origins"]), 2 * size), size):
                leaf, _, pts = dt.rays(g["root_origins"][i:i + size], g["root_dirs"][i:i + size],
                                       roots=g["root_ids"][i:i + size])
                assert np.array_equal(leaf, g["root_leaf"][i:i + size])
                assert same_points(pts, g["root_points"][i:i + size], leaf != MISS)[0]
        for i in range(0, min(len(g["ball_centres"]), 3 * size), size):
            hit = dt.balls(g["ball_centres"][i:i + size], g["ball_radii"][i:i + size])
            assert np.array_equal(hit, g["ball_hit"][i:i + size])
    _reset_voxel()


def test_regression_ray_of_reference_tests():
    """tests.c:600-659 -- the ray from (-2,-2,0) along (1,1,-1) hits."""
    g = load("g676d50c")
    ht, ptr = _host_tree(g)
    dt = vg().DeviceTree(ptr)
    leaf, _, pts = dt.rays(g["regress_origin"], g["regress_dir"])
    assert leaf[0] != MISS and leaf[0] == g["regress_leaf"][0]
    assert same_points(pts, g["regress_point"], np.array([True]))[0]


def _golden_cam(g):
    return dict(kind=0, position=g["cam_position"], rotation=g["cam_rotation"], mul=g["cam_mul"],
                xsub=g["cam_xsub"], ysub=g["cam_ysub"])


def _expected_colours(points, leaf, tex, voxel=(1, 1, 1)):
    hit = leaf != MISS
    q = np.trunc(points / np.asarray(voxel, np.float32)).astype(np.int64)
    idx = np.abs(q) & 31
    c = tex[idx[:, 0] * 1024 + idx[:, 1] * 32 + idx[:, 2]].astype(np.uint32)
    return np.where(hit, 0xFF000000 | (c << 16) | (c << 8) | c, 0).astype(np.uint32)


def test_render64_matches_reference_golden():
    """Config-1 frame (64^3 blobs, 256x256): every pixel's colour is the one
    the reference's hit gives."""
    from voxvision_gb300 import workloads as wl
    g = load("render64")
    _reset_voxel()
    ht = vg().HostTree.from_voxels(g["voxels"].astype(np.float32))
    dt = vg().DeviceTree(ht.ptr)
    tex = wl.texture32(7)
    cam = vg().camera_struct(_golden_cam(g))
    img = dt.render(cam, int(g["w"]), int(g["h"]), tex)
    assert np.array_equal(img.ravel(), _expected_colours(g["pix_points"], g["pix_leaf"], tex))
    # the same rays through the batch entry point
    orig = np.repeat(g["cam_position"][None, :], g["pix_dirs"].shape[0], 0)
    leaf, _, pts = dt.rays(orig, g["pix_dirs"])
    assert np.array_equal(leaf, g["pix_leaf"])
    assert same_points(pts, g["pix_points"], leaf != MISS)[0]


@pytest.fixture(scope="module")
def tree256():
    """Config-2 volume: 256^3 value noise, ~8% solid, unit voxels."""
    from voxvision_gb300 import workloads as wl
    _reset_voxel()
    vox = wl.voxels_from_mask(wl.noise_volume(256, 2, 0.08))
    ht = vg().HostTree.from_voxels(vox)
    dt = vg().DeviceTree(ht.ptr)
    return ht, dt


def _orbit_state(frame, w=1920, h=1080, kind=0):
    from voxvision_gb300.cameras import orbit_camera
    cam = orbit_camera(frame, 120, w, h, (128, 128, 128), 1.5 * 256 * 3 ** 0.5, kind=kind)
    return cam.state()


@pytest.mark.parametrize("frame", [0, 17, 61])
def test_render_1080p_orbit_matches_oracle(tree256, frame):
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    tex = wl.texture32(7)
    st = _orbit_state(frame)
    img = dt.render(vg().camera_struct(st), 1920, 1080, tex)
    ref, _ = orc.render_best(ht.ptr, st, 1920, 1080, tex)
    assert (img != 0).mean() > 0.01
    assert np.array_equal(img, ref), f"{(img != ref).sum()} pixels differ"


@pytest.mark.parametrize("quality", [0, 1, 2, 2 | 4, 2 | 8])
def test_render_quality_modes_match_oracle(tree256, quality):
    """FAST / ADAPTIVE / ray-merge frames (renderer.c:215-318)."""
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    tex = wl.texture32(7)
    st = _orbit_state(5, 640, 480)
    img = dt.render_quality(vg().camera_struct(st), 640, 480, quality, tex)
    ref, _ = orc.render_quality(ht.ptr, st, 640, 480, quality, tex)
    assert np.array_equal(img, ref), f"{(img != ref).sum()} pixels differ"


def test_doom_camera_frame_matches_oracle(tree256):
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    tex = wl.texture32(7)
    st = _orbit_state(30, 640, 480, kind=1)
    img = dt.render(vg().camera_struct(st), 640, 480, tex)
    ref, _ = orc.render_best(ht.ptr, st, 640, 480, tex)
    assert np.array_equal(img, ref)


def test_incoherent_rays_16m_match_oracle(tree256):
    """Config 3: 16M rays, origins in a box twice the tree's, directions
    uniform on the sphere."""
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    o, d = wl.incoherent_rays(1 << 24, -128.0, 384.0, 3)
    leaf, slot, pts = dt.rays(o, d)
    oleaf, oslot, opts, _ = orc.ray_batch(ht.ptr, o, d)
    assert np.array_equal(leaf, oleaf), f"{(leaf != oleaf).sum()} leaf ids differ"
    assert np.array_equal(slot, oslot)
    assert same_points(pts, opts, leaf != MISS)[0]
    assert (leaf != MISS).mean() > 0.05


def test_balls_1m_match_oracle(tree256):
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    c, r = wl.balls(1 << 20, 0.0, 256.0, 0.5, 8.0, 4)
    hit = dt.balls(c, r)
    ohit, _ = orc.ball_batch(ht.ptr, c, r)
    assert np.array_equal(hit, ohit)
    assert 0.05 < hit.mean() < 0.95


def test_work_counters_match_oracle(tree256):
    """The counting kernels tally exactly the nodes, inner nodes and voxels
    the reference's recursion visits (the basis of the bytes-per-ray figure)."""
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    st = _orbit_state(9, 640, 480)
    cnt = torch.zeros(3, dtype=torch.int64, device="cuda")
    dt.render_counts_device(vg().camera_struct(st), 640, 480, cnt)
    torch.cuda.synchronize()
    _, ocnt = orc.render_best(ht.ptr, st, 640, 480, wl.texture32(7))
    assert cnt.cpu().numpy().tolist() == ocnt.tolist()
    o, d = wl.incoherent_rays(1 << 18, -128.0, 384.0, 31)
    to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    cnt.zero_()
    dt.ray_counts_device(to, td, cnt)
    torch.cuda.synchronize()
    _, _, _, ocnt = orc.ray_batch(ht.ptr, o, d)
    assert cnt.cpu().numpy().tolist() == ocnt.tolist()
    c, r = wl.balls(1 << 16, 0.0, 256.0, 0.5, 8.0, 41)
    cnt.zero_()
    dt.ball_counts_device(torch.from_numpy(c).cuda(), torch.from_numpy(r).cuda(), cnt)
    torch.cuda.synchronize()
    _, ocnt = orc.ball_batch(ht.ptr, c, r)
    assert cnt.cpu().numpy().tolist()[0] == int(ocnt[0]) and cnt.cpu().numpy().tolist()[2] == int(ocnt[2])


def test_device_entry_points_on_a_torch_stream(tree256):
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    o, d = wl.incoherent_rays(1 << 16, -128.0, 384.0, 77)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
        leaf = torch.empty(o.shape[0], dtype=torch.int32, device="cuda")
        slot = torch.empty(o.shape[0], dtype=torch.uint8, device="cuda")
        pts = torch.zeros(o.shape[0], 3, dtype=torch.float32, device="cuda")
        dt.rays_device(to, td, leaf, slot, pts, stream=s.cuda_stream)
    s.synchronize()
    hleaf, hslot, hpts = dt.rays(o, d)
    assert np.array_equal(leaf.cpu().numpy().view(np.uint32), hleaf)
    assert np.array_equal(slot.cpu().numpy(), hslot)
    assert same_points(pts.cpu().numpy(), hpts, hleaf != MISS)[0]


def test_ray_order_changes_no_result(tree256):
    """Batches of 2^16 rays or more are traced in coherent order: the same
    300k rays (half of them leaf-rooted) in one batch and in 2^15-ray batches
    (traced as given) give identical leaves, slots and points."""
    from voxvision_gb300 import workloads as wl
    ht, dt = tree256
    n = 300_000
    o, d = wl.incoherent_rays(n, -128.0, 384.0, 91)
    nodes = dt.info()["nodes"]
    rng = np.random.default_rng(92)
    roots = np.where(rng.random(n) < 0.5, rng.integers(0, nodes, n), MISS).astype(np.uint32)
    leaf, slot, pts = dt.rays(o, d, roots)
    parts = [dt.rays(o[i:i + 32768], d[i:i + 32768], roots[i:i + 32768]) for i in range(0, n, 32768)]
    l2 = np.concatenate([p[0] for p in parts])
    s2 = np.concatenate([p[1] for p in parts])
    p2 = np.concatenate([p[2] for p in parts])
    hit = leaf != MISS
    assert np.array_equal(leaf, l2) and np.array_equal(slot, s2)
    assert np.array_equal(pts[hit].view(np.uint32), p2[hit].view(np.uint32))
    assert 0.1 < hit.mean() < 0.9


def test_dropin_single_queries_return_reference_nodes():
    """vox_ray_tree_intersection / vox_tree_ball_collidep with the reference's
    signatures return the same host node / boolean as the oracle."""
    g = load("ball12")
    _reset_voxel()
    L = vg().lib()
    ht = vg().HostTree.from_voxels(g["voxels"])
    n = int(orc.lib().orc_count_nodes(ht.ptr))
    nodes = np.zeros(n, np.uint64)
    orc.lib().orc_preorder(ht.ptr, nodes.ctypes.data_as(C.c_void_p))
    for i in range(0, 400):
        o = np.ascontiguousarray(g["ray_origins"][i]); d = np.ascontiguousarray(g["ray_dirs"][i])
        res = np.full(3, 7.0, np.float32)
        r = L.vox_ray_tree_intersection(ht.ptr, o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                                        res.ctypes.data_as(C.c_void_p))
        expect = g["ray_leaf"][i]
        if expect == MISS:
            assert not r and np.all(res == 7.0)
        else:
            assert r == int(nodes[expect])
            assert same_points(res[None], g["ray_points"][i:i + 1], np.array([True]))[0]
    for i in range(0, 200):
        c = np.ascontiguousarray(g["ball_centres"][i])
        assert L.vox_tree_ball_collidep(ht.ptr, c.ctypes.data_as(C.c_void_p),
                                        float(g["ball_radii"][i])) == g["ball_hit"][i]
    L.vox_cuda_forget_tree(ht.ptr)


def test_renderer_context_api(tree256):
    """vox_make_context_headless / set_scene / set_camera / set_quality /
    vox_render / vox_redraw produce the oracle's frame."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree256
    L = vg().lib()
    ctx = L.vox_make_context_headless(640, 480)
    assert ctx
    assert L.vox_make_context_headless(100, 480) is None
    cam = orbit_camera(3, 120, 640, 480, (128, 128, 128), 665.0)
    L.vox_context_set_camera(ctx, cam.obj)
    L.vox_context_set_scene(ctx, ht.ptr)
    assert L.vox_context_set_quality(ctx, 4) == 0           # ray merge needs ADAPTIVE
    for q in (0, 2, 2 | 8):
        assert L.vox_context_set_quality(ctx, q) == 1
        L.vox_render(ctx)
        assert L.vox_context_status(ctx) == 0
        L.vox_redraw(ctx)
        px = np.ctypeslib.as_array(C.cast(L.vox_context_pixels(ctx), C.POINTER(C.c_uint32)), (480 * 640,))
        ref, _ = orc.render_quality(ht.ptr, cam.state(), 640, 480, q, wl.texture32(7))
        assert np.array_equal(px.reshape(480, 640), ref)
    L.vox_destroy_context(ctx)


def test_renderer_context_frames_in_sequence(tree256):
    """A context's frame is its own, so each vox_render clears only what the
    previous frame drew outside the new tree rectangle.  A sequence of
    cameras that moves the rectangle around -- other sides of the orbit, a
    near camera whose rectangle is the whole frame, one looking away (empty
    rectangle) -- in BEST, ADAPTIVE and FAST quality: every frame is the
    oracle's, with no pixel left from an earlier one."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree256
    L = vg().lib()
    W, H = 320, 240
    ctx = L.vox_make_context_headless(W, H)
    cam = HostCamera(0)
    L.vox_context_set_camera(ctx, cam.obj)
    L.vox_context_set_scene(ctx, ht.ptr)
    centre = np.float32([128, 128, 128])
    poses = [(665.0, 0.3, 20.0, False), (665.0, 2.4, 40.0, False), (230.0, 1.0, 10.0, False),
             (665.0, 4.0, 5.0, True), (900.0, 5.1, 30.0, False), (665.0, 2.4, 40.0, False), (400.0, 0.7, 25.0, False)]
    tex = wl.texture32(7)
    drawn = 0
    for k, (r, az, el, away) in enumerate(poses):
        pos = wl.pose_position(centre, r, az, el)
        cam.set_position(pos)
        cam.look_at(tuple(2 * np.asarray(pos) - centre) if away else tuple(centre))
        q = (0, 2, 1)[k % 3]
        assert L.vox_context_set_quality(ctx, q) == 1
        L.vox_render(ctx)
        assert L.vox_context_status(ctx) == 0
        L.vox_redraw(ctx)
        px = np.ctypeslib.as_array(C.cast(L.vox_context_pixels(ctx), C.POINTER(C.c_uint32)), (H * W,))
        ref, _ = orc.render_quality(ht.ptr, cam.state(), W, H, q, tex)
        assert np.array_equal(px.reshape(H, W), ref), (k, q)
        drawn += int((ref != 0).sum())
        if away:
            assert not ref.any()
    assert drawn > 10000
    L.vox_destroy_context(ctx)


def test_errors_and_empty_tree():
    _reset_voxel()
    dt = vg().DeviceTree(None)
    leaf, slot, pts = dt.rays(np.zeros((4, 3), np.float32), np.ones((4, 3), np.float32))
    assert (leaf == MISS).all() and (slot == 0xFF).all()
    assert (dt.balls(np.zeros((3, 3), np.float32), np.full(3, 5, np.float32)) == 0).all()
    cam = vg().camera_struct(dict(position=(0, 0, 0), mul=0.01, xsub=1, ysub=1))
    with pytest.raises(vg().VoxCudaError) as e:
        dt.render(cam, 100, 64, np.zeros(32768, np.uint8))
    assert e.value.code == -7
    img = dt.render(cam, 64, 32, np.zeros(32768, np.uint8))
    assert (img == 0).all()


def test_collision_detector_keeps_camera_out_of_the_scene(tree256):
    """cd.c:34-55: a move into the scene is undone, a move through free space
    is kept; the decision is the reference ball query's."""
    import ctypes as C
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree256
    L = vg().lib()
    ctx = L.vox_make_context_headless(64, 32)
    cam = HostCamera(0)
    L.vox_context_set_camera(ctx, cam.obj)
    L.vox_context_set_scene(ctx, ht.ptr)
    cd = L.vox_make_cd()
    start = np.array([-40.0, -40.0, -40.0], np.float32)
    cam.set_position(start)
    L.vox_cd_attach_camera(cd, cam.obj, C.c_float(3.0))
    L.vox_cd_attach_context(cd, ctx)
    vox = wl.voxels_from_mask(wl.noise_volume(256, 2, 0.08))
    inside = vox[len(vox) // 2] + 0.5                      # centre of a solid voxel
    for target in (inside, np.array([-60.0, -50.0, -45.0], np.float32), inside + 0.25):
        before = cam.position().copy()
        cam.set_position(target)
        L.vox_cd_collide(cd)
        hit, _ = orc.ball_batch(ht.ptr, np.asarray([target], np.float32), np.asarray([3.0], np.float32))
        expect = before if hit[0] else np.asarray(target, np.float32)
        assert np.array_equal(cam.position(), expect)
    C.CDLL(None).free(C.c_void_p(cd))
    L.vox_destroy_context(ctx)
