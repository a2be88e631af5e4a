"""The request server: requests from several threads, admitted by a memory
budget and batched continuously; every result equals the same request run
alone through the plain entry points and the oracle's answer over its own
tree (frames pixel-exact, ball hits exact)."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def setup():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    import voxvision_gb300 as vg
    from voxvision_gb300 import workloads as wl
    vg.set_voxel_size((1, 1, 1))
    from oracle import oracle as orc
    orc.set_voxel((1, 1, 1))
    vols = [wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20)),
            wl.voxels_from_mask(wl.noise_volume(128, 8, 0.10))]
    hosts = [vg.HostTree.from_voxels(v) for v in vols]
    trees = [vg.DeviceTree(h.ptr) for h in hosts]
    tex = wl.texture32(7)
    global _OTREES
    _OTREES = [orc.OracleTree.from_voxels(v) for v in vols]   # the oracle's own trees of the same voxels
    return vg, wl, hosts, trees, tex


_OTREES = None


def _oracle(tex, req):
    """The oracle's answer to a request: its BEST frame (camera state as the
    library's camera class set it up, pinned separately to the reference's
    camera plugins) or its ball answers, over the oracle-built tree."""
    from oracle import oracle as orc
    if req[0] == "frame":
        _, ti, cam, w, h, state = req
        ref, _ = orc.render_best(_OTREES[ti].ptr, state, w, h, tex)
        return ref.ravel().view(np.uint8)
    _, ti, c, r = req
    hit, _ = orc.ball_batch(_OTREES[ti].ptr, c, r)
    return hit


def _requests(wl, n, seed):
    from voxvision_gb300.cameras import HostCamera
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        ti = int(rng.integers(2))
        side = (64, 128)[ti]
        if rng.random() < 0.7:
            w, h = [(64, 32), (160, 120), (320, 240), (640, 480)][int(rng.integers(4))]
            cam = HostCamera(int(rng.integers(2)))
            cam.set_window_size(w, h)
            cam.set_position(wl.pose_position((side / 2,) * 3, 1.5 * side * 3 ** 0.5,
                                              rng.uniform(0, 2 * np.pi), rng.uniform(5, 45)))
            cam.look_at((side / 2,) * 3)
            out.append(("frame", ti, cam.gpu_struct(), w, h, cam.state()))
        else:
            k = int(rng.integers(1000, 20000))
            c, r = wl.balls(k, 0.0, float(side), 0.5, 8.0, seed * 1000 + i)
            out.append(("balls", ti, c, r))
    return out


def _alone(trees, tex, req):
    if req[0] == "frame":
        _, ti, cam, w, h = req[:5]
        return trees[ti].render(cam, w, h, tex).ravel().view(np.uint8)
    _, ti, c, r = req
    return trees[ti].balls(c, r)


def _run_mixed(vg, trees, tex, reqs, config, nthreads=4):
    srv = vg.Server(tex, config)
    ids = [srv.add_tree(t) for t in trees]
    tickets = [None] * len(reqs)

    def client(k):
        for i in range(k, len(reqs), nthreads):
            q = reqs[i]
            if q[0] == "frame":
                tickets[i] = srv.submit_frame(ids[q[1]], q[2], q[3], q[4])
            else:
                tickets[i] = srv.submit_balls(ids[q[1]], q[2], q[3])

    th = [threading.Thread(target=client, args=(k,)) for k in range(nthreads)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    results = []
    for t in tickets:
        assert srv.wait(t, 60000) == 0
        arr, times = srv.result(t)
        assert times[0] <= times[1] <= times[2]
        results.append(arr)
        srv.release(t)
    stats = srv.stats()
    srv.close()
    return results, stats


def test_mixed_requests_equal_requests_alone(setup):
    vg, wl, hosts, trees, tex = setup
    reqs = _requests(wl, 48, 1)
    cfg = vg.ServerConfig(1 << 34, 1 << 32, 64, 16, 4, 8)
    results, stats = _run_mixed(vg, trees, tex, reqs, cfg)
    for q, got in zip(reqs, results):
        assert np.array_equal(got, _alone(trees, tex, q)), q[0]
        assert np.array_equal(got, _oracle(tex, q)), q[0]
    assert stats["completed"] == stats["submitted"] == len(reqs)
    assert stats["launches"] >= 1


def test_frames_on_device_equal_oracle(setup):
    """A server whose frames stay in device memory: every frame (read from the
    device pointer the server hands out) and every ball answer of a mixed
    request stream equals the oracle's and the plain call's; a kept frame
    holds its device bytes until it is released, and nothing of it goes
    through host memory."""
    vg, wl, hosts, trees, tex = setup
    reqs = _requests(wl, 40, 5)
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 1 << 32, 64, 16, 4, 8, 1))
    ids = [srv.add_tree(t) for t in trees]
    resident = srv.stats()["bytes_in_use"]
    tickets = []
    for q in reqs:
        if q[0] == "frame":
            tickets.append(srv.submit_frame(ids[q[1]], q[2], q[3], q[4]))
        else:
            tickets.append(srv.submit_balls(ids[q[1]], q[2], q[3]))
    for t in tickets:
        assert srv.wait(t, 60000) == 0
    held = srv.stats()["bytes_in_use"] - resident
    frame_bytes = sum(q[3] * q[4] * 4 for q in reqs if q[0] == "frame")
    assert held >= frame_bytes                            # every finished frame is still on the device
    for q, t in zip(reqs, tickets):
        got, _ = srv.result(t, on_device=q[0] == "frame")
        assert np.array_equal(got, _alone(trees, tex, q)), q[0]
        assert np.array_equal(got, _oracle(tex, q)), q[0]
        srv.release(t)
    st = srv.stats()
    assert st["bytes_in_use"] == resident and st["frame_bytes_out"] == 0
    srv.close()


def _pinned_class(nbytes):
    c = 4096
    while c < nbytes:
        c <<= 1
    return c


def test_tight_budget_queues_but_stays_exact(setup):
    """A pinned-host budget that holds about two 640x480 results (plus two
    of the largest ball requests) forces admission to wait for memory;
    results are unchanged and the budget is never exceeded."""
    vg, wl, hosts, trees, tex = setup
    reqs = _requests(wl, 24, 2)
    host_budget = 2 * _pinned_class(640 * 480 * 4) + 2 * (_pinned_class(20000) + _pinned_class(20000 * 16))
    cfg = vg.ServerConfig(1 << 34, host_budget, 8, 4, 2, 2)
    results, stats = _run_mixed(vg, trees, tex, reqs, cfg, nthreads=3)
    for q, got in zip(reqs, results):
        assert np.array_equal(got, _alone(trees, tex, q)), q[0]
        assert np.array_equal(got, _oracle(tex, q)), q[0]
    assert 0 < stats["host_peak_bytes"] <= host_budget


def test_budget_refusal_and_bounded_wait(setup):
    """A frame whose result could never fit the pinned-host budget is refused
    at submission; two that fit one at a time are served one after the
    other, the second's wait bounded."""
    vg, wl, hosts, trees, tex = setup
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, _pinned_class(320 * 240 * 4) + 4096, 4, 4, 1, 1))
    ids = [srv.add_tree(t) for t in trees]
    from voxvision_gb300.cameras import HostCamera
    cam = HostCamera(0)
    cam.set_window_size(640, 480)
    cam.set_position((200, 0, 50))
    cam.look_at((32, 32, 32))
    with pytest.raises(vg.VoxCudaError) as e:         # can never fit
        srv.submit_frame(ids[0], cam.gpu_struct(), 640, 480)
    assert e.value.code == -8
    cam.set_window_size(320, 240)
    t1 = srv.submit_frame(ids[0], cam.gpu_struct(), 320, 240)
    t2 = srv.submit_frame(ids[0], cam.gpu_struct(), 320, 240)   # waits for t1's memory
    r2 = srv.wait(t2, 0)
    assert r2 in (0, -9)                                # done already, or a bounded wait gave up
    assert srv.wait(t1, 60000) == 0 and srv.wait(t2, 60000) == 0
    a1, _ = srv.result(t1)
    a2, _ = srv.result(t2)
    assert np.array_equal(a1, a2)
    assert np.array_equal(a1, _alone(trees, tex, ("frame", 0, cam.gpu_struct(), 320, 240)))
    srv.close()


def test_replay_serves_a_poisson_trace(setup):
    """vox_cuda_server_replay: a trace of frames and ball batches at Poisson
    arrival times; every request completes, with its server times in order
    (result exactness is the mixed-request test's)."""
    vg, wl, hosts, trees, tex = setup
    reqs = _requests(wl, 40, 4)
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 1 << 32, 64, 16, 4, 8))
    ids = [srv.add_tree(t) for t in trees]
    arrivals = np.cumsum(np.random.default_rng(4).exponential(1 / 2000.0, len(reqs)))
    trace = []
    for q, at in zip(reqs, arrivals):
        if q[0] == "frame":
            trace.append(("frame", ids[q[1]], q[2], q[3], q[4], float(at)))
        else:
            trace.append(("balls", ids[q[1]], q[2], q[3], float(at)))
    res = srv.replay(trace, collectors=3)
    assert (res[:, 0] == 0).all()
    assert (res[:, 1] <= res[:, 2]).all() and (res[:, 2] <= res[:, 3]).all()
    st = srv.stats()
    assert st["completed"] == st["submitted"] == len(reqs)
    srv.close()


def _frame_request(wl, w=160, h=120, az=0.7):
    from voxvision_gb300.cameras import HostCamera
    cam = HostCamera(0)
    cam.set_window_size(w, h)
    cam.set_position(wl.pose_position((32.0,) * 3, 1.5 * 64 * 3 ** 0.5, az, 20.0))
    cam.look_at((32.0,) * 3)
    return ("frame", 0, cam.gpu_struct(), w, h)


def test_injected_request_error_spares_other_requests(setup):
    """A launch whose enqueue fails (a host-side injected fault) ends its own
    requests with VOX_CUDA_ECUDA; the requests before and after it are
    served exactly, and the server's accounting stays whole."""
    vg, wl, hosts, trees, tex = setup
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 1 << 30, 16, 4, 1, 1))
    ids = [srv.add_tree(t) for t in trees]
    req = _frame_request(wl)
    expect = _alone(trees, tex, req)
    t0 = srv.submit_frame(ids[0], req[2], req[3], req[4])
    assert srv.wait(t0) == 0
    srv.inject(1)
    t1 = srv.submit_frame(ids[0], req[2], req[3], req[4])
    assert srv.wait(t1) == -3
    with pytest.raises(vg.VoxCudaError) as e:
        srv.result(t1)
    assert e.value.code == -3
    srv.release(t1)
    t2 = srv.submit_frame(ids[0], req[2], req[3], req[4])
    c, r = wl.balls(5000, 0.0, 64.0, 0.5, 8.0, 77)
    t3 = srv.submit_balls(ids[0], c, r)
    assert srv.wait(t2) == 0 and srv.wait(t3) == 0
    for t in (t0, t2):
        assert np.array_equal(srv.result(t)[0], expect)
    assert np.array_equal(srv.result(t3)[0], trees[0].balls(c, r))
    for t in (t0, t2, t3):
        srv.release(t)
    st = srv.stats()
    assert st["submitted"] == st["completed"] == 4
    assert st["inflight"] == 0 and st["pending"] == 0
    srv.close()


def test_injected_worker_failure_ends_requests_and_refuses_new_ones(setup):
    """An allocation failure in the server's worker (injected on the host):
    the requests it had not launched end with VOX_CUDA_ENOMEM instead of
    hanging their waiters, later submissions are refused with
    VOX_CUDA_ENOMEM, finished results stay readable and the server is
    destroyed cleanly."""
    vg, wl, hosts, trees, tex = setup
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 1 << 30, 16, 4, 1, 1))
    ids = [srv.add_tree(t) for t in trees]
    resident = srv.stats()["bytes_in_use"]          # the trees
    req = _frame_request(wl, az=2.0)
    t0 = srv.submit_frame(ids[0], req[2], req[3], req[4])
    assert srv.wait(t0) == 0
    srv.inject(2)
    pending = [srv.submit_frame(ids[0], req[2], req[3], req[4]) for _ in range(3)]
    for t in pending:
        assert srv.wait(t, 20000) == -2
    with pytest.raises(vg.VoxCudaError) as e:
        srv.submit_frame(ids[0], req[2], req[3], req[4])
    assert e.value.code == -2
    assert np.array_equal(srv.result(t0)[0], _alone(trees, tex, req))
    for t in [t0] + pending:
        srv.release(t)
    st = srv.stats()
    assert st["submitted"] == st["completed"] == 4
    assert st["inflight"] == 0 and st["pending"] == 0
    assert st["bytes_in_use"] == resident and st["host_bytes_in_use"] == 0
    srv.close()


def test_reused_result_buffers_hold_exact_frames(setup):
    """Result buffers are reused, and a frame copies out only the box that
    covers its tree's screen rectangle and what the buffer's previous frame
    left there.  Requests one at a time (each buffer goes back before the
    next request takes it) walk one 128 KiB buffer class through every case:
    a new buffer, frames of the same size from other poses, a frame that
    sees nothing (the old picture must be cleared), frames of another row
    pitch or height in the same class, and a buffer last used for ball hits.
    Every frame equals the plain call's and the oracle's, and fewer bytes
    than the frames hold cross to the host."""
    vg, wl, hosts, trees, tex = setup
    from voxvision_gb300.cameras import HostCamera
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 1 << 30, 16, 4, 1, 1))
    ids = [srv.add_tree(t) for t in trees]

    def frame(w, h, az, el=20.0, away=False, dist=1.5):
        cam = HostCamera(0)
        cam.set_window_size(w, h)
        pos = wl.pose_position((32.0,) * 3, dist * 64 * 3 ** 0.5, az, el)
        cam.set_position(pos)
        cam.look_at(tuple(2 * np.asarray(pos) - 32.0) if away else (32.0,) * 3)
        return ("frame", 0, cam.gpu_struct(), w, h, cam.state())

    c, r = wl.balls(100000, 0.0, 64.0, 0.5, 8.0, 91)      # 100000 hit bytes: the same 128 KiB class
    seq = [frame(160, 120, 0.3), frame(160, 120, 2.1, 40.0), frame(160, 120, 4.0, 5.0, dist=0.9),
           frame(160, 120, 1.0, away=True), frame(160, 120, 5.5), frame(176, 176, 0.8),
           frame(160, 120, 3.3, 30.0), frame(160, 200, 2.6, 10.0), frame(160, 120, 0.1, 45.0),
           frame(160, 200, 4.4), ("balls", 0, c, r), frame(160, 120, 1.7, 25.0), frame(160, 120, 1.7, 25.0)]
    for q in seq:
        t = srv.submit_frame(ids[0], q[2], q[3], q[4]) if q[0] == "frame" else srv.submit_balls(ids[0], q[2], q[3])
        assert srv.wait(t, 60000) == 0
        got, _ = srv.result(t)
        srv.release(t)
        assert np.array_equal(got, _alone(trees, tex, q)), q[0]
        assert np.array_equal(got, _oracle(tex, q)), q[0]
    st = srv.stats()
    assert st["frame_bytes_full"] == sum(q[3] * q[4] * 4 for q in seq if q[0] == "frame")
    assert 0 < st["frame_bytes_out"] < st["frame_bytes_full"]
    srv.close()


def test_default_configuration_serves(setup):
    """A server created with no configuration (the defaults: 40 GiB device
    and 16 GiB pinned-host budgets, half of the latter pinned at creation in
    128 MiB slabs, 16 streams, 32 launches in flight) serves a frame and a
    ball batch exactly."""
    vg, wl, hosts, trees, tex = setup
    srv = vg.Server(tex)
    ids = [srv.add_tree(t) for t in trees]
    req = _frame_request(wl, az=1.1)
    c, r = wl.balls(3000, 0.0, 64.0, 0.5, 8.0, 31)
    t1 = srv.submit_frame(ids[0], req[2], req[3], req[4])
    t2 = srv.submit_balls(ids[0], c, r)
    assert srv.wait(t1) == 0 and srv.wait(t2) == 0
    assert np.array_equal(srv.result(t1)[0], _alone(trees, tex, req))
    assert np.array_equal(srv.result(t2)[0], trees[0].balls(c, r))
    srv.release(t1)
    srv.release(t2)
    st = srv.stats()
    assert st["host_slabs"] >= (8 << 30) // (128 << 20)
    srv.close()


def test_smaller_request_takes_a_larger_free_buffer(setup):
    """With no pinned slabs to carve from (a pinned-host budget below one
    slab, so every buffer is pinned on its own), a request whose size class
    has no free buffer takes a free buffer of a larger class instead of
    pinning another, and every frame drawn into such a buffer -- after one
    of another row pitch -- is the plain call's and the oracle's."""
    vg, wl, hosts, trees, tex = setup
    from voxvision_gb300.cameras import HostCamera
    srv = vg.Server(tex, vg.ServerConfig(1 << 34, 16 << 20, 4, 4, 1, 1))
    ids = [srv.add_tree(t) for t in trees]

    def frame(w, h, az):
        cam = HostCamera(0)
        cam.set_window_size(w, h)
        cam.set_position(wl.pose_position((32.0,) * 3, 1.5 * 64 * 3 ** 0.5, az, 20.0))
        cam.look_at((32.0,) * 3)
        return ("frame", 0, cam.gpu_struct(), w, h, cam.state())

    seq = [frame(640, 480, 0.4), frame(320, 240, 1.3), frame(640, 480, 2.2), frame(320, 240, 3.1),
           frame(320, 240, 4.0)]
    for q in seq:
        t = srv.submit_frame(ids[0], q[2], q[3], q[4])
        assert srv.wait(t, 60000) == 0
        got, _ = srv.result(t)
        srv.release(t)
        assert np.array_equal(got, _alone(trees, tex, q))
        assert np.array_equal(got, _oracle(tex, q))
    st = srv.stats()
    assert st["host_slabs"] == 0
    # the first frame's result and job table are pinned; every later request
    # reuses them (the 320x240 frames the 640x480 frame's larger buffer)
    assert st["host_pins"] <= 3
    srv.close()
