"""The mixed-camera load of the batched form, checked frame by frame against
the oracle: 64 cameras of resolutions 320x240 .. 3840x2160 over the four
resident noise-volume trees (64^3 .. 512^3, 5-20% solid), drawn by one
persistent batch launch.  The oracle builds its own trees from the same
voxels (tree.c restated), sets up its own cameras (simple-camera.c restated)
and draws every frame with its BEST loop (renderer.c:200-319)."""
import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def mixed():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as vg
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    vg.set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    sides, hosts, devs, otrees = [], [], [], []
    for n, seed, solid in wl.BATCH_TREES:
        vox = wl.voxels_from_mask(wl.noise_volume(n, seed, solid))
        h = vg.HostTree.from_voxels(vox)
        sides.append(n)
        hosts.append(h)
        devs.append(vg.DeviceTree(h.ptr))
        otrees.append(orc.OracleTree.from_voxels(vox))
    tex_h = wl.texture32(7)
    tex = torch.from_numpy(tex_h).cuda()
    jobs, oracle_cams = [], []
    for ti, (w, h), az, el in wl.batch_poses(64, len(devs), 14):
        n = sides[ti]
        pos = wl.pose_position((n / 2,) * 3, 1.5 * n * 3 ** 0.5, az, el)
        cam = HostCamera(0)
        cam.set_window_size(w, h)
        cam.set_position(pos)
        cam.look_at((n / 2,) * 3)
        jobs.append((devs[ti], cam.gpu_struct(), w, h, tex, torch.empty(w * h, dtype=torch.int32, device="cuda")))
        oracle_cams.append((ti, orc.camera_simple(pos, (n / 2,) * 3, w, h, 1.0)))
    yield vg, jobs, oracle_cams, otrees, tex_h, devs, sides
    del jobs
    torch.cuda.synchronize()


def _check_all(jobs, oracle_cams, otrees, tex_h):
    bad = []
    for k, (j, (ti, st)) in enumerate(zip(jobs, oracle_cams)):
        w, h = j[2], j[3]
        ref, _ = orc.render_best(otrees[ti].ptr, st, w, h, tex_h)
        if not np.array_equal(j[5].cpu().numpy().view(np.uint32).reshape(h, w), ref):
            bad.append((k, w, h, ti))
    return bad


@pytest.mark.parametrize("cfg", [None, (16, 4, 2, 8)])
def test_mixed_batch_frames_equal_oracle(mixed, cfg):
    """Every frame of the 64-camera batch (126.5 M pixels, up to 3840x2160, the
    512^3 tree among them), after two graph replays into frames full of
    garbage, equals the oracle's frame."""
    vg, jobs, oracle_cams, otrees, tex_h, devs, sides = mixed
    b = vg.FrameBatch(jobs, vg.BatchConfig(*cfg) if cfg else None)
    for j in jobs:
        j[5].fill_(0x5A5A5A5A)
    b.launch()
    b.launch()
    torch.cuda.synchronize()
    b.close()
    assert sum(j[2] * j[3] for j in jobs) == 126_489_600
    bad = _check_all(jobs, oracle_cams, otrees, tex_h)
    assert not bad, f"{len(bad)} frames differ from the oracle: {bad[:5]}"


@pytest.mark.parametrize("on_device", [True, False])
def test_served_mixed_load_equals_oracle(mixed, on_device):
    """The served form on the same load: the 64 frames of the mixed set and
    16 batches of 1k-64k balls over the four trees, submitted together to a
    server (frames kept on the device, or copied to host memory); every frame
    and every ball answer equals the oracle's."""
    vg, jobs, oracle_cams, otrees, tex_h, devs, sides = mixed
    from voxvision_gb300 import workloads as wl
    # the server's default shape: 256 admitted, 32 a launch, 16 streams, 32 launches in flight
    srv = vg.Server(tex_h, vg.ServerConfig(40 << 30, 8 << 30, 256, 32, 16, 32, 1 if on_device else 0))
    ids = [srv.add_tree(d) for d in devs]
    tree_of_job = [ti for ti, _ in oracle_cams]
    reqs = []
    for k, j in enumerate(jobs):
        reqs.append(("frame", k, srv.submit_frame(ids[tree_of_job[k]], j[1], j[2], j[3])))
    rng = np.random.default_rng(15)
    for i in range(16):
        ti = i % len(devs)
        c, r = wl.balls(int(rng.integers(1000, 64001)), 0.0, float(sides[ti]), 0.5, 8.0, 200 + i)
        reqs.append(("balls", (ti, c, r), srv.submit_balls(ids[ti], c, r)))
    bad = []
    for kind, what, t in reqs:
        assert srv.wait(t, 120000) == 0
        if kind == "frame":
            got, _ = srv.result(t, on_device=on_device)
            ti, st = oracle_cams[what]
            w, h = jobs[what][2], jobs[what][3]
            ref, _ = orc.render_best(otrees[ti].ptr, st, w, h, tex_h)
            if not np.array_equal(got.view(np.uint32).reshape(h, w), ref):
                bad.append(("frame", what))
        else:
            ti, c, r = what
            got, _ = srv.result(t)
            ref, _ = orc.ball_batch(otrees[ti].ptr, c, r)
            if not np.array_equal(got, ref):
                bad.append(("balls", ti))
        srv.release(t)
    srv.close()
    assert not bad, bad[:5]
