"""The batched form: one persistent kernel over many frames, replayed from a
CUDA graph, gives every frame bit-identical to the plain per-frame call, for
every autotuner configuration and after camera changes."""
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
    vols = [wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20)),
            wl.voxels_from_mask(wl.noise_volume(96, 5, 0.10)),
            wl.voxels_from_mask(wl.noise_volume(128, 6, 0.15))]
    hosts = [vg.HostTree.from_voxels(v) for v in vols]
    devs = [vg.DeviceTree(h.ptr) for h in hosts]
    sizes = [(64, 32), (320, 240), (640, 480), (160, 120), (48, 64)]
    tex = torch.from_numpy(wl.texture32(7)).cuda()
    from voxvision_gb300.cameras import HostCamera
    rng = np.random.default_rng(3)
    jobs, meta = [], []
    for i in range(14):
        ti = i % 3
        w, h = sizes[i % len(sizes)]
        n = [64, 96, 128][ti]
        cam = HostCamera(i % 2)
        cam.set_window_size(w, h)
        az, el = rng.uniform(0, 2 * np.pi), rng.uniform(5, 45)
        cam.set_position(wl.pose_position((n / 2,) * 3, 1.5 * n * 3 ** 0.5, az, el))
        cam.look_at((n / 2,) * 3)
        out = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        jobs.append((devs[ti], cam.gpu_struct(), w, h, tex, out))
        meta.append((ti, cam))
    return vg, hosts, devs, jobs, meta, tex


def _plain(vg, job):
    tree, cam, w, h, tex, _ = job
    ref = torch.empty(w * h, dtype=torch.int32, device="cuda")
    tree.render_device(cam, w, h, tex, ref)
    torch.cuda.synchronize()
    return ref.cpu().numpy()


def test_batch_frames_equal_plain_frames(scene):
    vg, hosts, devs, jobs, meta, tex = scene
    b = vg.FrameBatch(jobs)
    b.launch()
    torch.cuda.synchronize()
    for j in jobs:
        assert np.array_equal(j[5].cpu().numpy(), _plain(vg, j))
    # and one frame against the CPU oracle
    ti, cam = meta[2]
    w, h = jobs[2][2], jobs[2][3]
    ref, _ = orc.render_best(hosts[ti].ptr, cam.state(), w, h, tex.cpu().numpy())
    assert np.array_equal(jobs[2][5].cpu().numpy().view(np.uint32).reshape(h, w), ref)
    b.close()


@pytest.mark.parametrize("cfg", [(8, 4, 1, 4), (16, 2, 2, 8), (32, 1, 4, 4), (8, 8, 1, 8), (16, 4, 2, 4),
                                 (8, 4, 2, 8, 1), (8, 4, 2, 8, 2)])
def test_every_config_gives_the_same_frames(scene, cfg):
    vg, hosts, devs, jobs, meta, tex = scene
    b = vg.FrameBatch(jobs, vg.BatchConfig(*cfg))
    for j in jobs:
        j[5].fill_(0x5A5A5A5A)
    b.launch()
    b.launch()           # replay the same graph
    torch.cuda.synchronize()
    for j in jobs:
        assert np.array_equal(j[5].cpu().numpy(), _plain(vg, j))
    assert b.config() == dict(zip(("tile_w", "tile_h", "tiles_per_grab", "blocks_per_sm", "stack_class"),
                                  cfg + (0,) * (5 - len(cfg))))
    b.close()


def test_autotune_and_camera_change(scene):
    vg, hosts, devs, jobs, meta, tex = scene
    b = vg.FrameBatch(jobs)
    cfg, ms = b.autotune(reps=1)
    assert ms > 0 and cfg["tile_w"] * cfg["tile_h"] in (32, 64)
    # move one camera; the next replay draws the new view
    from voxvision_gb300.cameras import HostCamera
    cam = HostCamera(0)
    w, h = jobs[5][2], jobs[5][3]
    cam.set_window_size(w, h)
    cam.set_position((200, -50, 90))
    cam.look_at((48, 48, 48))
    b.set_camera(5, cam.gpu_struct())
    b.launch()
    torch.cuda.synchronize()
    tree = jobs[5][0]
    ref = torch.empty(w * h, dtype=torch.int32, device="cuda")
    tree.render_device(cam.gpu_struct(), w, h, tex, ref)
    torch.cuda.synchronize()
    assert np.array_equal(jobs[5][5].cpu().numpy(), ref.cpu().numpy())
    b.close()


def test_batch_rejects_bad_jobs(scene):
    vg, hosts, devs, jobs, meta, tex = scene
    bad = list(jobs[:2])
    t, c, w, h, tx, out = bad[0]
    bad[0] = (t, c, 100, h, tx, out)
    with pytest.raises(vg.VoxCudaError) as e:
        vg.FrameBatch(bad)
    assert e.value.code == -7
    with pytest.raises(vg.VoxCudaError):
        vg.FrameBatch(jobs, vg.BatchConfig(12, 4, 1, 4))


def test_culled_rectangles_follow_camera_changes(scene):
    """Cameras inside a tree's box (whole frame traced), looking away from it
    (nothing traced, whole frame cleared), far away and off-centre: every
    frame equals the plain call's with the output full of garbage before each
    replay, also after set_camera changes how many tiles each frame has."""
    vg, hosts, devs, jobs, meta, tex = scene
    from voxvision_gb300.cameras import HostCamera
    poses = [((30, 35, 40), (60, 60, 60)),          # inside the 64^3 box
             ((32, 250, 30), (32, 500, 30)),       # looking away
             ((32, -900, 32), (32, 32, 32)),       # far: a few tiles
             ((140, -40, 60), (90, 90, 20))]       # tree partly off-screen
    kinds = [0, 1, 0, 1]
    mk = []
    for i, ((pos, at), kind) in enumerate(zip(poses, kinds)):
        w, h = [(336, 200), (64, 32), (320, 240), (160, 120)][i]
        cam = HostCamera(kind)
        cam.set_window_size(w, h)
        cam.set_position(pos)
        cam.look_at(np.asarray(at, np.float32))
        out = torch.zeros(w * h, dtype=torch.int32, device="cuda")
        mk.append((devs[0], cam.gpu_struct(), w, h, tex, out))
    b = vg.FrameBatch(mk)
    for rnd in range(3):
        for j in mk:
            j[5].fill_(0x5A5A5A5A)
        b.launch()
        torch.cuda.synchronize()
        for j in mk:
            assert np.array_equal(j[5].cpu().numpy(), _plain(vg, j)), f"round {rnd}"
        # rotate the poses among the frames (each keeps its size)
        nxt = []
        for i, j in enumerate(mk):
            pos, at = poses[(i + rnd + 1) % 4]
            cam = HostCamera(kinds[(i + rnd + 1) % 4])
            cam.set_window_size(j[2], j[3])
            cam.set_position(pos)
            cam.look_at(np.asarray(at, np.float32))
            b.set_camera(i, cam.gpu_struct())
            nxt.append((j[0], cam.gpu_struct(), j[2], j[3], j[4], j[5]))
        mk = nxt
    b.close()
