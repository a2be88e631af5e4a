"""vox_cuda_render_frames_noalloc: frames drawn without any allocation, for
callers that may not allocate GPU memory while they render (a loop that must
not stall on cudaMalloc, a host that hands out all device memory itself, a
device that is nearly full).  Its scratch is a fixed array inside the library,
shared by every call.

Each frame must equal the one vox_cuda_render_device draws for the same tree,
camera and size (ARGB pixels, compared exactly), on two calls in a row --
the second with a different job list, so a stale job table or an unreset
queue head from the first call would show -- also when the two calls are
issued back to back on one stream with no wait between them, behind a kernel
that is still running.  This file is collected last so a failure here cannot
hide the results of the other tests.
"""
import time

import numpy as np
import pytest

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
    from voxvision_gb300.cameras import HostCamera
    vg.set_voxel_size((1, 1, 1))
    hosts = [vg.HostTree.from_voxels(wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20))),
             vg.HostTree.from_voxels(wl.voxels_from_mask(wl.noise_volume(128, 6, 0.12)))]
    trees = [vg.DeviceTree(h.ptr) for h in hosts]
    tex = torch.from_numpy(wl.texture32(7)).cuda()

    def make_jobs(n, seed):
        rng = np.random.default_rng(seed)
        sizes = [(64, 32), (160, 120), (320, 240), (48, 64)]
        jobs = []
        for i in range(n):
            ti = i % 2
            side = (64, 128)[ti]
            w, h = sizes[rng.integers(len(sizes))]
            cam = HostCamera(int(rng.integers(2)))
            cam.set_window_size(w, h)
            cam.set_position(wl.pose_position((side / 2,) * 3, 1.5 * side * 3 ** 0.5,
                                              rng.uniform(0, 2 * np.pi), rng.uniform(5, 45)))
            cam.look_at((side / 2,) * 3)
            jobs.append((trees[ti], cam.gpu_struct(), w, h,
                         torch.full((w * h,), 0x7B7B7B7B, dtype=torch.int32, device="cuda")))
        return jobs

    return vg, hosts, trees, tex, make_jobs


def _call(vg, jobs, tex, stream=None):
    arr = (vg.FrameJob * len(jobs))()
    for i, (tree, cam, w, h, out) in enumerate(jobs):
        arr[i].tree = tree.h.value
        arr[i].camera = cam
        arr[i].w, arr[i].h = w, h
        arr[i].texture = tex.data_ptr()
        arr[i].argb = out.data_ptr()
    return vg.lib().vox_cuda_render_frames_noalloc(arr, len(jobs), stream)


def _check_against_plain(jobs, tex):
    torch.cuda.synchronize()
    for tree, cam, w, h, out in jobs:
        ref = torch.empty(w * h, dtype=torch.int32, device="cuda")
        tree.render_device(cam, w, h, tex, ref)
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref.cpu().numpy())


def test_noalloc_frames_equal_plain_frames_on_two_calls(scene):
    vg, hosts, trees, tex, make_jobs = scene
    first = make_jobs(9, 1)
    assert _call(vg, first, tex) == 0
    _check_against_plain(first, tex)
    second = make_jobs(5, 2)           # fewer jobs, other cameras: the array keeps call 1's table
    assert _call(vg, second, tex) == 0
    _check_against_plain(second, tex)


def test_noalloc_rejects_requests_beyond_its_capacity(scene):
    vg, hosts, trees, tex, make_jobs = scene
    cap = 64
    jobs = make_jobs(cap + 1, 3)
    assert _call(vg, jobs, tex) == -11                      # VOX_CUDA_ECAPACITY
    assert vg.lib().vox_cuda_strerror(-11).startswith(b"request exceeds")
    assert _call(vg, jobs[:cap], tex) == 0
    _check_against_plain(jobs[:cap], tex)


def test_noalloc_calls_back_to_back_on_a_busy_stream(scene):
    """Two calls with different job lists on one non-default stream, queued
    behind a kernel that is still running and with no synchronisation between
    them: both return before that kernel ends (the job table travels as a
    kernel argument; nothing waits for the stream), and after one
    synchronisation every frame of both lists equals the plain frame."""
    vg, hosts, trees, tex, make_jobs = scene
    s = torch.cuda.Stream()
    a, b = make_jobs(7, 4), make_jobs(6, 5)
    assert _call(vg, a[:1], tex, s.cuda_stream) == 0      # set-up done before timing
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        torch.cuda._sleep(400_000_000)                    # a busy kernel, ~0.2 s at 2 GHz
    t0 = time.perf_counter()
    assert _call(vg, a, tex, s.cuda_stream) == 0
    assert _call(vg, b, tex, s.cuda_stream) == 0
    returned_s = time.perf_counter() - t0
    still_busy = not s.query()
    s.synchronize()
    _check_against_plain(a, tex)
    _check_against_plain(b, tex)
    assert still_busy, "the stream finished before the calls returned: they waited for it"
    assert returned_s < 0.05
