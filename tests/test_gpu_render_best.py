"""GPU parity of the BEST frame kernel under every setting (culled to the
tree's screen rectangle or not, overlapped with the previous kernel of the
stream or not): each frame equals the oracle's pixel for pixel, every pixel
of the output is written (the ones outside the rectangle are cleared), stream
order holds for the texture and the frame when consecutive kernels overlap,
and the setting API validates its input."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CONFIGS = [(1, 1), (1, 0), (0, 1), (0, 0)]
GARBAGE = 0x5EADBEEF


@pytest.fixture(scope="module", autouse=True)
def built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as vg
    saved = vg.render_config()
    yield
    vg.set_render_config(saved["cull"], saved["overlap"])


def vg():
    import voxvision_gb300
    return voxvision_gb300


@pytest.fixture(scope="module")
def tree256():
    from voxvision_gb300 import workloads as wl
    vg().set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    ht = vg().HostTree.from_voxels(wl.voxels_from_mask(wl.noise_volume(256, 2, 0.08)))
    return ht, vg().DeviceTree(ht.ptr)


@pytest.fixture(scope="module")
def tree64():
    from voxvision_gb300 import workloads as wl
    vg().set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    ht = vg().HostTree.from_voxels(wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20)))
    return ht, vg().DeviceTree(ht.ptr)


def render_device(dt, cam, w, h, tex):
    """Through vox_cuda_render_device into a buffer full of garbage."""
    d_tex = torch.from_numpy(tex).cuda()
    out = torch.full((w * h,), GARBAGE, dtype=torch.int64).to(torch.int32).cuda()
    dt.render_device(cam, w, h, d_tex, out, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return out.cpu().numpy().view(np.uint32).reshape(h, w)


@pytest.mark.parametrize("frame", [0, 44, 90])
def test_orbit_frames_equal_oracle_under_every_setting(tree256, frame):
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree256
    tex = wl.texture32(7)
    cam = orbit_camera(frame, 120, 1920, 1080, (128, 128, 128), 1.5 * 256 * 3 ** 0.5)
    ref, _ = orc.render_best(ht.ptr, cam.state(), 1920, 1080, tex)
    for cfg in CONFIGS:
        vg().set_render_config(*cfg)
        img = render_device(dt, cam.gpu_struct(), 1920, 1080, tex)
        assert np.array_equal(img, ref), f"setting {cfg}: {(img != ref).sum()} pixels differ"


def _cameras():
    """Simple and doom cameras near, far, off-centre, inside the tree's box
    and looking away from it; fields of view 0.3..2."""
    from voxvision_gb300 import workloads as wl
    rng = np.random.default_rng(5)
    centre = np.array([32.0, 32.0, 32.0])
    out = []
    for kind in (0, 1):
        for dist in (1.05, 1.5, 3.0, 30.0):
            for _ in range(2):
                pos = wl.pose_position(centre, dist * 55.4, rng.uniform(0, 6.28), rng.uniform(-50, 50))
                out.append((kind, pos, centre + rng.normal(0, 20, 3), float(rng.choice([0.3, 1.0, 2.0]))))
        out.append((kind, centre + 2.5, centre + 30.0, 1.0))
        out.append((kind, centre + [0, 200.0, 5.0], centre + [0, 400.0, 5.0], 1.0))
    return out


@pytest.mark.parametrize("cfg", [(1, 1), (0, 0)])
def test_many_cameras_equal_oracle(tree64, cfg):
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree64
    tex = wl.texture32(7)
    vg().set_render_config(*cfg)
    for kind, pos, target, fov in _cameras():
        for w, h in ((128, 96), (336, 200)):
            cam = HostCamera(kind)
            cam.set_fov(fov)
            cam.set_window_size(w, h)
            cam.set_position(pos)
            cam.look_at(np.asarray(target, np.float32))
            ref, _ = orc.render_best(ht.ptr, cam.state(), w, h, tex)
            img = render_device(dt, cam.gpu_struct(), w, h, tex)
            assert np.array_equal(img, ref), f"{kind} {pos} {w}x{h}: {(img != ref).sum()} pixels differ"
            host = dt.render(cam.gpu_struct(), w, h, tex)
            assert np.array_equal(host, ref)


def test_smallest_frame_and_empty_tree(tree64):
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree64
    tex = wl.texture32(7)
    vg().set_render_config(1, 1)
    cam = HostCamera(0)
    cam.set_window_size(16, 4)
    cam.set_position((32.0, -60.0, 32.0))
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    ref, _ = orc.render_best(ht.ptr, cam.state(), 16, 4, tex)
    assert np.array_equal(render_device(dt, cam.gpu_struct(), 16, 4, tex), ref)
    empty = vg().DeviceTree(None)
    cam.set_window_size(64, 32)
    assert (render_device(empty, cam.gpu_struct(), 64, 32, tex) == 0).all()


def test_stream_order_holds_when_frames_overlap(tree64):
    """Frames rendered back to back into one buffer, the texture rewritten by
    a torch kernel and the frame copied out between them, all on one stream:
    each copy shows the frame of the camera and texture before it."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree64
    vg().set_render_config(1, 1)
    texs = [wl.texture32(7), wl.texture32(8)]
    stream = torch.cuda.current_stream()
    d_tex = torch.from_numpy(texs[0]).cuda()
    d_texs = [torch.from_numpy(t).cuda() for t in texs]
    w, h = 336, 200
    out = torch.full((w * h,), GARBAGE, dtype=torch.int64).to(torch.int32).cuda()
    cams, copies = [], []
    rng = np.random.default_rng(9)
    for i in range(12):
        cam = HostCamera(i % 2)
        cam.set_window_size(w, h)
        cam.set_position(wl.pose_position((32, 32, 32), rng.uniform(60, 200), rng.uniform(0, 6.28),
                                          rng.uniform(-40, 40)))
        cam.look_at(np.asarray((32, 32, 32) + rng.normal(0, 10, 3), np.float32))
        d_tex.copy_(d_texs[i % 2])
        dt.render_device(cam.gpu_struct(), w, h, d_tex, out, stream=stream.cuda_stream)
        copies.append(out.clone())
        cams.append(cam)
    torch.cuda.synchronize()
    for i, (cam, cp) in enumerate(zip(cams, copies)):
        ref, _ = orc.render_best(ht.ptr, cam.state(), w, h, texs[i % 2])
        img = cp.cpu().numpy().view(np.uint32).reshape(h, w)
        assert np.array_equal(img, ref), f"frame {i}: {(img != ref).sum()} pixels differ"


def test_host_frame_pinned_and_pageable(tree256):
    """vox_cuda_render into a page-locked host frame (drawn in place over the
    host link) and into a pageable one (drawn on the device, copied out): both
    equal the oracle's frame, every pixel written."""
    import ctypes as C
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree256
    vg().set_render_config(1, 1)
    tex = wl.texture32(7)
    L = vg().lib()
    for frame in (3, 70):
        cam = orbit_camera(frame, 120, 1920, 1080, (128, 128, 128), 1.5 * 256 * 3 ** 0.5)
        ref, _ = orc.render_best(ht.ptr, cam.state(), 1920, 1080, tex)
        pinned = torch.full((1920 * 1080,), GARBAGE, dtype=torch.int32).pin_memory()
        pageable = np.full(1920 * 1080, GARBAGE, np.uint32)
        cs = cam.gpu_struct()
        for buf in (pinned.data_ptr(), pageable.ctypes.data):
            rc = L.vox_cuda_render(dt.h, C.byref(cs), 1920, 1080, tex.ctypes.data_as(C.c_void_p),
                                   C.c_void_p(buf), None)
            assert rc == 0
        img = pinned.numpy().view(np.uint32).reshape(1080, 1920)
        assert np.array_equal(img, ref), f"pinned: {(img != ref).sum()} pixels differ"
        assert np.array_equal(pageable.reshape(1080, 1920), ref)


def test_host_frames_call_equals_single_frames(tree256):
    """vox_cuda_render_frames: an orbit's frames into distinct host buffers,
    pinned (drawn in place, frames overlapping) and pageable mixed, each
    equal to the oracle's frame with every pixel written."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree256
    vg().set_render_config(1, 1)
    tex = wl.texture32(9)
    w, h = 960, 544
    cams = [orbit_camera(f, 24, w, h, (128, 128, 128), 1.5 * 256 * 3 ** 0.5) for f in range(0, 24, 3)]
    bufs = [torch.full((h, w), GARBAGE, dtype=torch.int32).pin_memory() if i % 3 else
            np.full((h, w), GARBAGE, np.uint32) for i in range(len(cams))]
    dt.render_frames([c.gpu_struct() for c in cams], w, h, tex, bufs)
    for i, (cam, b) in enumerate(zip(cams, bufs)):
        ref, _ = orc.render_best(ht.ptr, cam.state(), w, h, tex)
        img = b if isinstance(b, np.ndarray) else b.numpy().view(np.uint32)
        assert np.array_equal(img, ref), f"frame {i}: {(img != ref).sum()} pixels differ"


def test_host_frames_call_last_frames_of_every_kind(tree64):
    """The last frames of a vox_cuda_render_frames launch reach the host in
    two parts (the zeros outside the traced rectangle early, the rectangle
    once drawn): with those frames of every kind -- the tree in part of the
    frame, the camera inside the tree (the whole frame traced), the camera
    looking away (no rectangle) -- into garbage-filled pinned and pageable
    buffers, every frame equals the oracle's."""
    import ctypes as C
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera, orbit_camera
    ht, dt = tree64
    tex = wl.texture32(13)
    w, h = 320, 240
    cams = [orbit_camera(f, 12, w, h, (32, 32, 32), 1.5 * 64 * 3 ** 0.5) for f in range(0, 12, 2)]
    for pos, at in (((32.0, 30.0, 33.0), (60.0, 50.0, 40.0)),       # inside the tree
                    ((150.0, -80.0, 90.0), (300.0, -300.0, 90.0)),  # looking away
                    ((90.0, -40.0, 70.0), (32.0, 32.0, 32.0))):     # near, off to one side
        c = HostCamera(0)
        c.set_window_size(w, h)
        c.set_position(pos)
        c.look_at(np.array(at, np.float32))
        cams.append(c)
    for order in (cams, cams[::-1]):
        bufs = [torch.full((h, w), GARBAGE, dtype=torch.int32).pin_memory() if i % 2 else
                np.full((h, w), GARBAGE, np.uint32) for i in range(len(order))]
        dt.render_frames([c.gpu_struct() for c in order], w, h, tex, bufs)
        for i, (cam, b) in enumerate(zip(order, bufs)):
            ref, _ = orc.render_best(ht.ptr, cam.state(), w, h, tex)
            img = b if isinstance(b, np.ndarray) else b.numpy().view(np.uint32)
            assert np.array_equal(img, ref), f"frame {i}: {(img != ref).sum()} pixels differ"
    bb = np.zeros(6, np.float32)
    vg().lib().vox_bounding_box(C.c_void_p(ht.ptr), bb.ctypes.data_as(C.c_void_p))
    kinds = [vg().frame_rect(bb, c.gpu_struct(), w, h) for c in cams[-3:]]
    assert kinds[0] == (0, 0, w, h) and kinds[1][2] <= kinds[1][0]
    assert 0 < kinds[2][0] < kinds[2][2] < w and 0 < kinds[2][1] < kinds[2][3] < h


def test_host_frames_call_reuses_device_frames(tree64):
    """More frames than the 2 GiB of device frames hold (36 frames of 4096^2):
    the slots are reused round robin, each only after its copy finished."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree64
    tex = wl.texture32(3)
    w = h = 4096
    cams = [orbit_camera(f, 36, w, h, (32, 32, 32), 1.5 * 64 * 3 ** 0.5).gpu_struct() for f in range(36)]
    bufs = [np.full((h, w), GARBAGE, np.uint32) for _ in cams]
    dt.render_frames(cams, w, h, tex, bufs)
    d_tex = torch.from_numpy(tex).cuda()
    d_frame = torch.empty((h, w), dtype=torch.int32, device="cuda")
    for i in (0, 1, 31, 32, 35):
        dt.render_device(cams[i], w, h, d_tex, d_frame)
        torch.cuda.synchronize()
        assert np.array_equal(bufs[i], d_frame.cpu().numpy().view(np.uint32)), f"frame {i} differs"


def test_host_frames_call_many_small_frames_and_empty_tree(tree64):
    """1100 small frames (more than one launch holds) equal the single-frame
    call's; an empty tree gives all-zero frames."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    ht, dt = tree64
    tex = wl.texture32(5)
    w, h = 32, 16
    cams = [orbit_camera(f, 1100, w, h, (32, 32, 32), 1.5 * 64 * 3 ** 0.5).gpu_struct() for f in range(1100)]
    bufs = dt.render_frames(cams, w, h, tex)
    for i in (0, 1, 511, 1023, 1024, 1099):
        assert np.array_equal(bufs[i], dt.render(cams[i], w, h, tex)), f"frame {i} differs"
    empty = vg().DeviceTree(None)
    zs = empty.render_frames(cams[:5], w, h, tex, [np.full((h, w), GARBAGE, np.uint32) for _ in range(5)])
    assert all(not z.any() for z in zs)


def test_host_calls_follow_texture_changes(tree64):
    """The host-buffer call keeps the last texture on the device and uploads
    a new one only when its bytes change: frames drawn with textures A, B, A,
    and A edited in place, each equal the oracle's frame with that texture."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    ht, dt = tree64
    cam = HostCamera(0)
    cam.set_window_size(160, 120)
    cam.set_position((150.0, -80.0, 90.0))
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    a, b = wl.texture32(7), wl.texture32(11)
    edited = a.copy()
    for tex in (a, b, a, edited):
        if tex is edited:
            edited[::3] ^= 0x5A                       # same buffer object as before, new bytes
        img = dt.render(cam.gpu_struct(), 160, 120, tex)
        ref, _ = orc.render_best(ht.ptr, cam.state(), 160, 120, tex)
        assert np.array_equal(img, ref)


def test_setting_api_validates():
    with pytest.raises(vg().VoxCudaError):
        vg().set_render_config(2, 1)
    with pytest.raises(vg().VoxCudaError):
        vg().set_render_config(1, 2)
    vg().set_render_config(0, 1)
    assert vg().render_config() == {"cull": 0, "overlap": 1}
