#!/usr/bin/env python
"""Benchmark: Mrays/s of the BEST-quality frame path at 1920x1080 over a
256^3 volume, along a 120-frame orbit.

Workload (one "step" = one full orbit = 120 frames = 248,832,000 rays):
256^3 u8 value noise (17^3 lattice, spacing 16, seed 2), band-thresholded to
~8% solid, built into a tree by the library's vox_make_tree; camera
simple-camera, fov 1.0 (90 degrees), orbit radius 1.5 x the bounding-box
diagonal (665.1) at 20 degrees elevation around (128, 128, 128); texture
32^3 u8 from splitmix64 seed 7.

  value  device throughput: the 120-frame orbit as one vox_cuda_batch of
         120 jobs (one persistent batch kernel launch from a CUDA graph per
         step, configuration autotuned once before timing), tree, texture and
         the 120 frames resident in HBM, timed with a pair of CUDA events per
         step on the launching stream; L2 flushed (256 MiB write) between
         steps, outside the timed events.  roofline.plain gives the same
         orbit as 120 vox_cuda_render_device launches back to back.
  e2e    the same orbit through the host-buffer call vox_cuda_render_frames:
         every step copies the texture and cameras in and delivers each
         8.3 MB frame into its own page-locked host buffer (copied out while
         the next frames are drawn), timed on the host; per_call_value gives
         the same frames through one synchronous vox_cuda_render call each.
  roofline  algorithmic bytes per frame (32 B per node box tested, 16 B per
         inner node entered, 16 B per voxel tested, 4 B per pixel stored;
         counted by the counting kernel, less the root test of the rays
         outside the tree's screen rectangle, which the kernel does not
         trace) over the mean time per frame, against the measured HBM copy
         bandwidth; a measured L2 copy bandwidth is reported beside it.
  cpu_baseline  the CPU oracle (C restatement of the reference's search and
         render loop) on all host cores over a bounded sample of orbit frames.
  quality  (extras) the same orbit's frames in every vox_render quality
         (BEST, FAST, ADAPTIVE with and without ray merging), Mpixels/s per
         quality on the GPU and of the oracle on the host cores.

--impl reference times that CPU implementation on the full orbit instead.
Under torchrun each rank renders its own replica of the workload (the path
has no exchange step); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

W, H = 1920, 1080
NFRAMES = 120
VOLUME, SEED, SOLID = 256, 2, 0.08
CENTRE = (128.0, 128.0, 128.0)
RADIUS = 1.5 * 256 * math.sqrt(3.0)
METRIC = "Mrays/s at 1080p on 256^3"
PEAKS_PATH = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC_SUMMARY = os.path.join(ROOT, "profiles", "batch_orbit_1080p_256.json")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the incoherent-query and batched-frame measurements")
    p.add_argument("--frames", type=int, default=NFRAMES,
                   help="orbit frames per step (profiling runs only; the benchmark uses 120)")
    p.add_argument("--batch-config", default=None, metavar="TW,TH,GRAB,BPS",
                   help="batch kernel configuration instead of autotuning (profiling runs)")
    p.add_argument("--kernels-only", action="store_true",
                   help="time only the batched orbit (no plain launches, e2e or extras; profiling runs)")
    p.add_argument("--tree-build", type=int, default=0, metavar="N",
                   help="only time the device tree build of the N^3 noise volume (profiling runs)")
    p.add_argument("--reps", type=int, default=5, help="timed repetitions of --tree-build")
    p.add_argument("--quality", type=int, default=0, metavar="N",
                   help="only time every vox_render quality on N orbit frames (profiling runs)")
    p.add_argument("--batched", action="store_true",
                   help="only time the 64-frame mixed-camera batch against plain launches (profiling runs)")
    return p.parse_args()


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of `values` over the ranks of the default process
    group (a job takes its slowest rank's time); unchanged without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_rate(units_per_rank, world, seconds):
    """Whole-job throughput of `world` replicas that each processed
    `units_per_rank` units in `seconds` (the slowest rank's time)."""
    return world * units_per_rank / seconds


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload_config(voxels, nframes=NFRAMES):
    """The workload as both arms name it (the same dict in both lines)."""
    return {"workload": "orbit-1080p-256^3-best", "volume": "256^3 u8 value noise, seed 2, band ~8% solid",
            "voxels": int(voxels), "frames_per_step": nframes, "resolution": f"{W}x{H}", "quality": "BEST",
            "camera": "simple-camera fov 1.0, orbit r=665.1 elev 20deg",
            "rays_per_step": nframes * W * H, "l2": "flushed between steps (256 MiB write)"}


def workloads():
    """The seeded workload generators (voxvision_gb300/workloads.py, numpy
    only), loaded from their file so that the reference arm imports nothing
    of the library package."""
    import importlib.util
    mod = sys.modules.get("_orbit_workloads")
    if mod is None:
        spec = importlib.util.spec_from_file_location("_orbit_workloads",
                                                      os.path.join(ROOT, "voxvision_gb300", "workloads.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        sys.modules["_orbit_workloads"] = mod
    return mod


def make_workload(build_tree):
    wl = workloads()
    vox = wl.voxels_from_mask(wl.noise_volume(VOLUME, SEED, SOLID))
    tree = build_tree(vox)
    return vox, tree, wl.texture32(7)


def orbit_states():
    """The library's simple-camera set up for every orbit frame."""
    from voxvision_gb300.cameras import orbit_camera
    return [orbit_camera(f, NFRAMES, W, H, CENTRE, RADIUS).state() for f in range(NFRAMES)]


def oracle_orbit_states():
    """The same cameras set up by the oracle's restatement of simple-camera.c
    (bit-identical to the library's: tests/test_oracle_golden.py)."""
    from oracle import oracle as orc
    wl = workloads()
    return [orc.camera_simple(wl.orbit_pose(f, NFRAMES, CENTRE, RADIUS, 20.0), CENTRE, W, H, 1.0)
            for f in range(NFRAMES)]


def cpu_model():
    """The host CPU's model name (lscpu), or what /proc/cpuinfo says."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def cpu_reference_details(tree_ptr, states, tex, cores):
    """Beside the all-core figure: the CPU model, one core's Mrays/s (the
    oracle's BEST render on one thread over two orbit frames), and the same
    frames drawn by the restatement compiled with floating-point contraction
    on (the compiler's default in the reference's release build): its speed
    and how many pixels differ from the contraction-off frames."""
    from oracle import oracle as orc
    picked = [0, 61]
    t0 = time.perf_counter()
    off = [orc.render_best(tree_ptr, states[f], W, H, tex, nthreads=1)[0] for f in picked]
    single = len(picked) * W * H / (time.perf_counter() - t0) / 1e6
    t0 = time.perf_counter()
    on = [orc.render_best_contracted(tree_ptr, states[f], W, H, tex, nthreads=cores)[0] for f in picked]
    fc_value = len(picked) * W * H / (time.perf_counter() - t0) / 1e6
    t0 = time.perf_counter()
    for f in picked:
        orc.render_best(tree_ptr, states[f], W, H, tex, nthreads=cores)
    off_value = len(picked) * W * H / (time.perf_counter() - t0) / 1e6
    differ = int(sum(int((a != b).sum()) for a, b in zip(off, on)))
    return {"cpu_model": cpu_model(), "single_core_value": single,
            "single_core_sample": f"orbit frames {picked} at {W}x{H}, BEST, 1 thread",
            "fp_contract_fast": {"value": fc_value, "value_contract_off": off_value, "cores": cores,
                                 "pixels_differing": differ, "pixels": len(picked) * W * H,
                                 "what": "the restatement compiled with -ffp-contract=fast (liboracle_fc.so), "
                                         "same tree and frames"}}


class ClockSampler:
    """nvidia-smi clock / throttle samples taken while the timed region runs."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(PEAKS_PATH) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_per_launch(nframes):
    """DRAM bytes (read + write) per batch launch of `nframes` orbit frames,
    from the committed ncu figures of the kernel (scaled by frames, which the
    reads of tree misses and the frame stores both follow), if any."""
    try:
        with open(TRAFFIC_SUMMARY) as f:
            p = json.load(f)
        return float(p["traffic_bytes_per_launch"]) * nframes / float(p["frames_per_launch"])
    except (OSError, KeyError, ValueError, ZeroDivisionError):
        return None


def l2_read_gbs(L, mib=32, reps=1000):
    """L2 read bandwidth: one kernel reading a 32 MiB buffer (inside the
    129 MB L2) 1000 times over with L1-bypassing loads, CUDA-event timed
    (vox_cuda_measure_l2_read); best of 3."""
    import ctypes as C
    best = 0.0
    for _ in range(3):
        g = C.c_float()
        if L.vox_cuda_measure_l2_read(mib << 20, reps, C.byref(g)) == 0:
            best = max(best, float(g.value))
    return best


def issue_figures(nframes, traced_rays, launch_s, nsm, sm_mhz):
    """The issue roofline of the kernel: its warp instructions per launch
    (from the committed ncu summary of the 24-frame orbit, scaled to this
    launch by frames) over the launch time measured here, against the issue
    peak of the device (4 schedulers a SM, one warp instruction a cycle each,
    at the SM clock sampled during the timed region); and the instructions
    per traced ray."""
    try:
        with open(TRAFFIC_SUMMARY) as f:
            p = json.load(f)
        inst = float(p["warp_inst_per_launch"]) * nframes / float(p["frames_per_launch"])
        achieved = inst / launch_s / 1e9
        peak = nsm * 4 * sm_mhz * 1e6 / 1e9 if sm_mhz else None
        return {"achieved_ginst_s": achieved, "peak_ginst_s": peak, "frac": achieved / peak if peak else None,
                "unit": "G warp instructions/s",
                "warp_inst_per_traced_ray": inst / traced_rays,
                "thread_inst_per_traced_ray": inst * float(p["lanes_active_per_inst"]) / traced_rays,
                "lanes_active_per_inst": float(p["lanes_active_per_inst"]),
                "issue_slots_busy": float(p["issue_slots_busy"]),
                "l2_throughput_pct_of_peak": float(p["l2_throughput_pct"]),
                "source": "ncu --set full of batch_kernel on the 24-frame orbit, " + p.get("captured", "")}
    except (OSError, KeyError, ValueError, ZeroDivisionError):
        return None


def cpu_baseline_sample(tree_ptr, states, tex, budget_s=3.0):
    """The oracle's BEST render on every host core over orbit frames (every
    7th) until ~budget_s of wall time has passed."""
    from oracle import oracle as orc
    n = orc.nthreads_default()
    frames, t0 = 0, time.perf_counter()
    order = list(range(0, NFRAMES, 7)) + [f for f in range(NFRAMES) if f % 7]
    for f in order:
        orc.render_best(tree_ptr, states[f], W, H, tex, nthreads=n)
        frames += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": frames * W * H / dt / 1e6, "unit": "Mrays/s", "cores": n, "kind": "port",
            "sample": f"{frames} of the {NFRAMES} orbit frames at {W}x{H}, BEST, {dt:.2f} s wall"}




def oracle_check_orbit(frames_dev, vox, lib_tree_ptr, tex, nf):
    """Every frame of the timed batch launch against the oracle: the tree
    built by the oracle's restatement of tree.c from the same voxels (and
    compared node for node with the library's), the cameras set up by its
    restatement of simple-camera.c, each frame drawn by its BEST loop."""
    from oracle import oracle as orc
    orc.set_voxel((1, 1, 1))
    t0 = time.perf_counter()
    ot = orc.OracleTree.from_voxels(vox)
    a, b = orc.dump_tree(lib_tree_ptr), ot.dump()
    tree_same = a.keys() == b.keys() and all(np.array_equal(a[k], b[k]) for k in a)
    states = oracle_orbit_states()
    host = frames_dev.cpu().numpy().view(np.uint32)
    n = orc.nthreads_default()
    bad = []
    for f in range(nf):
        ref, _ = orc.render_best(ot.ptr, states[f], W, H, tex, nthreads=n)
        if not np.array_equal(host[f].reshape(H, W), ref):
            bad.append(f)
    return {"frames_checked": nf, "frames_identical_oracle": not bad, "frames_differing": bad[:10],
            "tree_identical_oracle": bool(tree_same), "oracle_tree_nodes": int(ot.node_count()),
            "check_s": time.perf_counter() - t0,
            "what": "every frame of the timed batch launch vs the oracle's BEST render over the oracle-built "
                    "tree with oracle-set-up cameras; the library's tree vs the oracle's, node for node"}


def timed_reps(torch, fn, reps, flush):
    """Best-of and mean CUDA-event time (ms) of fn() over reps runs, L2 flushed before each."""
    stream = torch.cuda.current_stream()
    ts = []
    for _ in range(reps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return min(ts), float(np.mean(ts))


def measure_incoherent(torch, vg, dt, flush):
    """16M rays (origins uniform in twice the tree's box, directions uniform on
    the sphere) and 1M balls (centres in the box, radii U[0.5, 8]) on the
    256^3 tree, through the device entry points."""
    from voxvision_gb300 import workloads as wl
    sp = torch.cuda.current_stream().cuda_stream
    n = 1 << 24
    o, d = wl.incoherent_rays(n, -128.0, 384.0, 3)
    to, td = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    leaf = torch.empty(n, dtype=torch.int32, device="cuda")
    slot = torch.empty(n, dtype=torch.uint8, device="cuda")
    pts = torch.empty(n, 3, dtype=torch.float32, device="cuda")
    nb = 1 << 20
    c, r = wl.balls(nb, 0.0, 256.0, 0.5, 8.0, 4)
    tc, tr = torch.from_numpy(c).cuda(), torch.from_numpy(r).cuda()
    hit = torch.empty(nb, dtype=torch.uint8, device="cuda")
    rays = lambda: dt.rays_device(to, td, leaf, slot, pts, stream=sp)
    balls = lambda: dt.balls_device(tc, tr, hit, stream=sp)
    for _ in range(3):
        rays(); balls()
    rb, rm = timed_reps(torch, rays, 5, flush)
    bb, bm = timed_reps(torch, balls, 5, flush)
    return {"rays": n, "rays_ms": rm, "rays_mrays_s": n / (rm * 1e-3) / 1e6,
            "ray_hit_fraction": float((leaf != -1).float().mean().item()),
            "balls": nb, "balls_ms": bm, "balls_mq_s": nb / (bm * 1e-3) / 1e6,
            "ball_hit_fraction": float(hit.float().mean().item()),
            "inputs": "rays: origins U[-128,384)^3 seed 3, dirs uniform on S^2; balls: centres U[0,256)^3, "
                      "r U[0.5,8] seed 4"}


QUALITIES = {"best": 0, "fast": 1, "adaptive": 2, "adaptive_ray_merge": 2 | 4,
             "adaptive_ray_merge_accurate": 2 | 8}


def measure_quality(torch, vg, dt, ht_ptr, states, tex, d_tex, flush, cpu=True, nframes=24):
    """The orbit at 1080p (every 5th frame) in every quality vox_render offers,
    through vox_cuda_render_quality_device (BEST: the frame kernel; FAST and
    ADAPTIVE: the squares kernel, each 4x4 square's sequence of
    renderer.c:215-318 on half a warp), one call per frame back to back, in
    pixels per second.  With the CPU-baseline leg on (no --no-cpu-baseline), frame 0 of
    each quality is checked against the oracle and the oracle's restatement
    of the same loop times a few frames of each on every host core."""
    sp = torch.cuda.current_stream().cuda_stream
    picked = list(range(0, NFRAMES, max(1, NFRAMES // nframes)))[:nframes]
    cams = [vg.camera_struct(states[f]) for f in picked]
    out = torch.empty((len(cams), H * W), dtype=torch.int32, device="cuda")   # 199 MB of frames: > L2
    res = {"frames": len(cams), "resolution": f"{W}x{H}", "unit": "Mpixels/s"}
    for name, q in QUALITIES.items():
        def run():
            for i, c in enumerate(cams):
                dt.render_quality_device(c, W, H, q, d_tex, out[i], stream=sp)
        for _ in range(3):
            run()
        _, mean_ms = timed_reps(torch, run, 5, flush)
        e = {"quality": q, "ms_per_frame": mean_ms / len(cams),
             "value": len(cams) * W * H / (mean_ms * 1e-3) / 1e6}
        if cpu:   # the CPU-baseline leg: the oracle checks frame 0 and is timed beside the GPU
            from oracle import oracle as orc
            ref, _ = orc.render_quality(ht_ptr, states[picked[0]], W, H, q, tex)
            e["frame0_identical"] = bool(np.array_equal(out[0].cpu().numpy().view(np.uint32).reshape(H, W), ref))
            n, t0, k = orc.nthreads_default(), time.perf_counter(), 0
            for f in picked[:3]:
                orc.render_quality(ht_ptr, states[f], W, H, q, tex, nthreads=n)
                k += 1
            cpu_s = time.perf_counter() - t0
            e["cpu_value"] = k * W * H / cpu_s / 1e6
            e["cpu_cores"] = n
            e["vs_cpu"] = e["value"] / e["cpu_value"]
        res[name] = e
    return res


def measure_dropin(vg, ht_ptr, nframes=24):
    """The drop-in renderer as a voxvision program drives it: a 1080p context
    (vox_make_context_headless) over the library's host tree, the built-in
    simple camera moved along the orbit, and per frame one synchronous
    vox_render (the frame drawn into the context's device frame) and one
    vox_redraw (the frame copied to the page-locked buffer vox_context_pixels
    returns), host-timed, in the default ADAPTIVE quality and in BEST."""
    import ctypes as C
    from voxvision_gb300.cameras import orbit_camera
    L = vg.lib()
    ctx = L.vox_make_context_headless(W, H)
    picked = list(range(0, NFRAMES, max(1, NFRAMES // nframes)))[:nframes]
    cams = [orbit_camera(f, NFRAMES, W, H, CENTRE, RADIUS) for f in picked]
    L.vox_context_set_scene(ctx, ht_ptr)
    out = {"frames": len(cams), "resolution": f"{W}x{H}",
           "call": "vox_render then vox_redraw per frame, a vox_make_context_headless context"}
    for name, q in (("adaptive", QUALITIES["adaptive"]), ("best", QUALITIES["best"])):
        L.vox_context_set_quality(ctx, q)
        render_ms, redraw_ms = [], []
        for rep in range(4):
            for cam in cams:
                L.vox_context_set_camera(ctx, cam.obj)
                t0 = time.perf_counter()
                L.vox_render(ctx)
                t1 = time.perf_counter()
                L.vox_redraw(ctx)
                t2 = time.perf_counter()
                if L.vox_context_status(ctx):
                    raise vg.VoxCudaError(L.vox_context_status(ctx), "vox_render")
                if rep:                       # the first pass warms up
                    render_ms.append((t1 - t0) * 1e3)
                    redraw_ms.append((t2 - t1) * 1e3)
        out[name] = {"quality": q, "render_ms": float(np.median(render_ms)),
                     "render_p99_ms": float(np.percentile(render_ms, 99)),
                     "redraw_ms": float(np.median(redraw_ms)),
                     "mpixels_s": W * H / (float(np.median(render_ms)) * 1e-3) / 1e6}
    L.vox_destroy_context(ctx)
    # the reference's single queries, one call each (host-timed; the first
    # call of each kind uploads the tree, untimed)
    rng = np.random.default_rng(17)
    n = 2000
    org = rng.uniform(-100.0, 356.0, (n, 3)).astype(np.float32)
    tgt = rng.uniform(64.0, 192.0, (n, 3)).astype(np.float32)
    dirs = (tgt - org).astype(np.float32)
    res = np.zeros(3, np.float32)
    rp = res.ctypes.data_as(C.c_void_p)
    L.vox_ray_tree_intersection(C.c_void_p(ht_ptr), org[0].ctypes.data_as(C.c_void_p),
                                dirs[0].ctypes.data_as(C.c_void_p), rp)
    t0 = time.perf_counter()
    hits = 0
    for i in range(n):
        hits += bool(L.vox_ray_tree_intersection(C.c_void_p(ht_ptr), org[i].ctypes.data_as(C.c_void_p),
                                                 dirs[i].ctypes.data_as(C.c_void_p), rp))
    t1 = time.perf_counter()
    for i in range(n):
        L.vox_tree_ball_collidep(C.c_void_p(ht_ptr), tgt[i].ctypes.data_as(C.c_void_p), 3.0)
    t2 = time.perf_counter()
    L.vox_cuda_forget_tree(C.c_void_p(ht_ptr))
    out["single_queries"] = {"calls": n, "ray_us": (t1 - t0) / n * 1e6, "ball_us": (t2 - t1) / n * 1e6,
                             "ray_hits": hits,
                             "call": "vox_ray_tree_intersection / vox_tree_ball_collidep (radius 3) on the "
                                     "256^3 tree, rays from U[-100,356)^3 towards U[64,192)^3, seed 17"}
    return out


def measure_editing(vg, vox, edits=1000, seed=16):
    """Live editing of the 256^3 tree: `edits` single-voxel insertions and
    deletions through the library's vox_insert_voxel / vox_delete_voxel on
    a separate host copy of the tree, then vox_cuda_tree_refresh of its
    device copy (re-flatten and copy in place); a fresh upload for
    comparison."""
    import ctypes as C
    L = vg.lib()
    pts = np.ascontiguousarray(vox, dtype=np.float32).copy()
    root = C.c_void_p(L.vox_make_tree(pts.ctypes.data_as(C.c_void_p), pts.shape[0]))
    dt = vg.DeviceTree(root.value)
    rng = np.random.default_rng(seed)
    ops = []
    for i in range(edits):
        if i % 2 == 0:
            ops.append((L.vox_insert_voxel, rng.integers(0, 256, 3).astype(np.float32)))
        else:
            ops.append((L.vox_delete_voxel, vox[int(rng.integers(len(vox)))].astype(np.float32).copy()))
    t0 = time.perf_counter()
    changed = sum(fn(C.byref(root), a.ctypes.data_as(C.c_void_p)) for fn, a in ops)
    t_edit = time.perf_counter() - t0
    t0 = time.perf_counter()
    vg.check(L.vox_cuda_tree_refresh(dt.h, root), "vox_cuda_tree_refresh")
    t_refresh = time.perf_counter() - t0
    t0 = time.perf_counter()
    fresh = vg.DeviceTree(root.value)
    t_upload = time.perf_counter() - t0
    fresh.close()
    dt.close()
    L.vox_destroy_tree(root)
    return {"edits": edits, "changed": int(changed), "edit_ms": t_edit * 1e3,
            "edit_us_each": t_edit / edits * 1e6, "refresh_ms": t_refresh * 1e3,
            "fresh_upload_ms": t_upload * 1e3,
            "what": "alternating insertions (random voxels of the 256^3 box) and deletions (voxels of the "
                    "volume) on the host tree, then vox_cuda_tree_refresh of its device copy"}


def measure_tree_build(vg, sizes=((256, 2, 0.08), (512, 3, 0.10)), reps=5):
    """Time to a searchable device tree for the noise volumes: the host build
    (vox_make_tree_host, tree.c's algorithm on one host thread, then
    vox_cuda_tree_upload); the drop-in path (vox_make_tree, which builds sets
    this large on the GPU and makes the host tree from the image, then
    vox_cuda_tree_upload, which takes the device copy it kept); and the tree
    built on the GPU without a host tree from the voxel set in host memory
    (vox_cuda_tree_build), already on the device (vox_cuda_tree_build_device)
    and from the raw u8 samples with the band test on the GPU
    (vox_cuda_tree_build_raw).  Medians of `reps` after one warm-up;
    wall-clock, all synchronous calls."""
    import ctypes as C

    import torch
    from voxvision_gb300 import workloads as wl
    out = []
    for n, seed, solid in sizes:
        vol = wl.value_noise_u8(n, seed)
        lo, w = wl.band_for_fraction(vol, solid)
        vox = wl.voxels_from_mask((vol >= lo) & (vol < lo + w))
        raw = vol.tobytes()
        d_vox = torch.from_numpy(vox).cuda()

        def timed(fn):
            fn().close()
            ts = []
            for _ in range(reps):
                t0 = time.perf_counter()
                r = fn()
                ts.append(time.perf_counter() - t0)
                r.close()
            return float(np.median(ts)) * 1e3

        L = vg.lib()

        def built_by(fn):
            s = np.ascontiguousarray(vox, np.float32).copy()   # the build reorders its set
            t0 = time.perf_counter()
            h = vg.HostTree(fn(s.ctypes.data_as(C.c_void_p), s.shape[0]))
            t1 = time.perf_counter()
            d = vg.DeviceTree(h.ptr)
            t2 = time.perf_counter()
            d.close()
            h.close()
            return (t1 - t0) * 1e3, (t2 - t1) * 1e3

        def median_of(fn, k):
            fn()
            runs = [fn() for _ in range(k)]
            return [float(np.median([r[i] for r in runs])) for i in range(2)]

        host_make, host_up = median_of(lambda: built_by(L.vox_make_tree_host), reps if n <= 256 else 1)
        drop_make, drop_up = median_of(lambda: built_by(L.vox_make_tree), reps)
        rec = {"volume": f"{n}^3 u8 value noise, seed {seed}, band {lo}..{lo + w - 1}", "voxels": int(len(vox)),
               "host_make_tree_ms": host_make, "upload_ms": host_up, "host_path_ms": host_make + host_up,
               "dropin_make_tree_ms": drop_make, "dropin_first_upload_ms": drop_up,
               "dropin_path_ms": drop_make + drop_up,
               "device_build_ms": timed(lambda: vg.DeviceTree.build(vox)),
               "device_build_resident_ms": timed(lambda: vg.DeviceTree.build_device(d_vox)),
               "device_build_raw_ms": timed(lambda: vg.DeviceTree.from_raw(raw, vol.shape, 1, lo, lo + w - 1))}
        rec["speedup_vs_host_path"] = rec["host_path_ms"] / rec["device_build_ms"]
        rec["dropin_speedup_vs_host_path"] = rec["host_path_ms"] / rec["dropin_path_ms"]
        out.append(rec)
        del d_vox
    return out


def build_batch_trees(vg):
    from voxvision_gb300 import workloads as wl
    trees = []
    for n, seed, solid in wl.BATCH_TREES:
        ht = vg.HostTree.from_voxels(wl.voxels_from_mask(wl.noise_volume(n, seed, solid)))
        trees.append((n, ht, vg.DeviceTree(ht.ptr)))
    return trees


def measure_served(vg, trees, tex, rates=(1000, 2000, 5000, 10000, 15000, 20000), duration=1.0, seed=15,
                   frames_on_device=False):
    """Served load: 256 clients with Poisson arrivals (merged: one Poisson
    stream at the aggregate rate); 70% frames (resolution uniform over
    320x240..3840x2160, tree uniform, random orbit pose), 30% batches of
    1k-64k ball queries; 4 resident trees under a 40 GB device budget.  The
    trace is replayed by the library's native replay (a submitting thread at
    the arrival times, 8 collector threads); latency = submission to result
    in host memory (or, with frames_on_device, to the frame complete in the
    server's device memory), on the server's clock."""
    import ctypes as C
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    # the server's default configuration: 256 requests admitted at once (a few
    # milliseconds of GPU work), up to 32 per launch, 32 launches in flight on
    # 16 streams
    srv = vg.Server(tex, vg.ServerConfig(40 << 30, 24 << 30, 256, 32, 16, 32, 1 if frames_on_device else 0))
    ids = [srv.add_tree(t[2]) for t in trees]
    rng = np.random.default_rng(seed)
    ball_pool = []
    for i in range(16):
        k = int(rng.integers(1000, 64001))
        side = trees[i % len(trees)][0]
        ball_pool.append((i % len(trees), wl.balls(k, 0.0, float(side), 0.5, 8.0, 100 + i)))

    def make_requests(n, arrivals):
        reqs = []
        for i in range(n):
            ti = int(rng.integers(len(trees)))
            if rng.random() < 0.7:
                w, h = wl.RESOLUTIONS[int(rng.integers(len(wl.RESOLUTIONS)))]
                side = trees[ti][0]
                cam = HostCamera(0)
                cam.set_window_size(w, h)
                cam.set_position(wl.pose_position((side / 2,) * 3, 1.5 * side * 3 ** 0.5,
                                                  rng.uniform(0, 2 * np.pi), rng.uniform(5, 45)))
                cam.look_at((side / 2,) * 3)
                reqs.append(("frame", ids[ti], cam.gpu_struct(), w, h, float(arrivals[i])))
            else:
                bi = int(rng.integers(len(ball_pool)))
                tb, (c, r) = ball_pool[bi]
                reqs.append(("balls", ids[tb], c, r, float(arrivals[i])))
        return reqs

    # warm the server's pinned result pool with a trace at the highest rate
    # (pinning new memory runs at about 14 GB/s; growing the pool inside a
    # timed trace would show up as latency)
    top = max(rates)
    srv.replay(make_requests(2 * top // 10, np.cumsum(rng.exponential(1.0 / top, 2 * top // 10))))
    out = {}
    for rate in rates:
        n = max(200, int(rate * duration))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
        reqs = make_requests(n, arrivals)
        st0 = srv.stats()
        res = srv.replay(reqs)
        st1 = srv.stats()
        ok = res[:, 0] == 0
        lat = (res[:, 3] - res[:, 1]) * 1e-6
        queued = (res[:, 2] - res[:, 1]) * 1e-6      # submission to launch
        ran = (res[:, 3] - res[:, 2]) * 1e-6         # launch to result
        is_frame = np.array([q[0] == "frame" for q in reqs]) & ok
        is_ball = np.array([q[0] == "balls" for q in reqs]) & ok
        span = (res[ok, 3].max() - res[ok, 1].min()) * 1e-9
        rays = sum(q[3] * q[4] for q, good in zip(reqs, ok) if q[0] == "frame" and good)
        out[str(rate)] = {"requests": n, "errors": int((~ok).sum()),
                          "frame_p50_ms": float(np.percentile(lat[is_frame], 50)),
                          "frame_p99_ms": float(np.percentile(lat[is_frame], 99)),
                          "frame_queue_p99_ms": float(np.percentile(queued[is_frame], 99)),
                          "frame_run_p99_ms": float(np.percentile(ran[is_frame], 99)),
                          "ball_p50_ms": float(np.percentile(lat[is_ball], 50)) if is_ball.any() else None,
                          "ball_p99_ms": float(np.percentile(lat[is_ball], 99)) if is_ball.any() else None,
                          "error_codes": sorted({int(x) for x in res[~ok, 0]}),
                          "mrays_s": rays / span / 1e6, "offered_hz": rate,
                          "achieved_hz": n / span,
                          "worker": {k: st1[k] - st0[k] for k in ("worker_busy_ns", "host_pin_ns", "host_pins",
                                                                  "device_alloc_ns", "frame_bytes_out",
                                                                  "frame_bytes_full", "host_slabs")}}
    stats = srv.stats()
    srv.close()
    busy = {k: stats[k] for k in ("worker_busy_ns", "build_ns", "host_pin_ns", "host_pins", "device_alloc_ns",
                                  "frame_bytes_out", "frame_bytes_full")}
    # the plain path: the same kind of frames, one synchronous call at a time
    # -- vox_cuda_render into a page-locked host frame, or with the frames on
    # the device vox_cuda_render_device into a device frame, then wait
    import torch
    L = vg.lib()
    reqs = [q for q in make_requests(300, np.zeros(300)) if q[0] == "frame"][:150]
    tex_c = np.ascontiguousarray(tex)
    tree_of = {ids[i]: trees[i][2] for i in range(len(trees))}
    if frames_on_device:
        dframe = torch.empty(3840 * 2160, dtype=torch.int32, device="cuda")
        dtex = torch.from_numpy(tex_c).cuda()
        stream = torch.cuda.current_stream()

        def one(q):
            rc = L.vox_cuda_render_device(tree_of[q[1]].h, C.byref(q[2]), q[3], q[4], C.c_void_p(dtex.data_ptr()),
                                          C.c_void_p(dframe.data_ptr()), C.c_void_p(stream.cuda_stream))
            stream.synchronize()
            return rc
        call = "vox_cuda_render_device into a device frame, then wait; one frame at a time"
    else:
        host = torch.empty(3840 * 2160, dtype=torch.int32).pin_memory()

        def one(q):
            return L.vox_cuda_render(tree_of[q[1]].h, C.byref(q[2]), q[3], q[4], tex_c.ctypes.data_as(C.c_void_p),
                                     C.c_void_p(host.data_ptr()), None)
        call = "vox_cuda_render, one frame at a time, page-locked host frame"
    for q in reqs[:5]:
        one(q)
    lat = []
    t_all = time.perf_counter()
    for q in reqs:
        t1 = time.perf_counter()
        rc = one(q)
        if rc:
            raise vg.VoxCudaError(rc, "plain frame")
        lat.append((time.perf_counter() - t1) * 1e3)
    span = time.perf_counter() - t_all
    plain = {"frame_p50_ms": float(np.percentile(lat, 50)), "frame_p99_ms": float(np.percentile(lat, 99)),
             "mrays_s": sum(q[3] * q[4] for q in reqs) / span / 1e6, "frames": len(reqs), "call": call}
    best = max(out.values(), key=lambda v: v["mrays_s"])
    return {"rates": out, "plain": plain, "budget_gb": 40, "clients": 256, "peak_bytes": stats["peak_bytes"],
            "frames_on_device": bool(frames_on_device),
            "speedup_vs_plain_sync": best["mrays_s"] / plain["mrays_s"],
            "launches": stats["launches"], "replay": "vox_cuda_server_replay, 8 collector threads", "stats": busy}


def measure_batched(torch, vg, flush, tex_dev, trees=None):
    """Mixed-camera load: 64 frames, resolutions uniform over 320x240..3840x2160,
    trees uniform over the 64^3..512^3 noise volumes, random orbit poses; one
    persistent kernel replayed from a CUDA graph (autotuned) against 64 plain
    per-frame launches."""
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import HostCamera
    sp = torch.cuda.current_stream().cuda_stream
    if trees is None:
        trees = build_batch_trees(vg)
    jobs = []
    for ti, (w, h), az, el in wl.batch_poses(64, len(trees), 14):
        n, _, dt = trees[ti]
        cam = HostCamera(0)
        cam.set_window_size(w, h)
        cam.set_position(wl.pose_position((n / 2,) * 3, 1.5 * n * 3 ** 0.5, az, el))
        cam.look_at((n / 2,) * 3)
        jobs.append((dt, cam.gpu_struct(), w, h, tex_dev, torch.empty(w * h, dtype=torch.int32, device="cuda")))
    rays = sum(w * h for _, _, w, h, _, _ in jobs)

    def plain():
        for dt, cam, w, h, tex, out in jobs:
            dt.render_device(cam, w, h, tex, out, stream=sp)

    for _ in range(3):
        plain()
    pb, pm = timed_reps(torch, plain, 5, flush)

    # the plain path as a caller that waits for each frame sees it (what the
    # drop-in vox_render does): one launch, then wait, per frame; host-timed
    def plain_sync():
        for dt, cam, w, h, tex, out in jobs:
            dt.render_device(cam, w, h, tex, out, stream=sp)
            torch.cuda.current_stream().synchronize()

    plain_sync()
    sync_ms = []
    for _ in range(3):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        plain_sync()
        sync_ms.append((time.perf_counter() - t0) * 1e3)
    psm = float(np.median(sync_ms))
    batch = vg.FrameBatch(jobs)
    cfg, tune_ms = batch.autotune(stream=sp, reps=2)
    launch = lambda: batch.launch(stream=sp)
    for _ in range(3):
        launch()
    bb, bm = timed_reps(torch, launch, 5, flush)
    # identical frames: the batch's output against the plain launches
    outs = [j[5].clone() for j in jobs]
    plain()
    torch.cuda.synchronize()
    same = all(bool(torch.equal(a, j[5])) for a, j in zip(outs, jobs))
    batch.close()
    return {"frames": len(jobs), "rays": rays, "trees": [t[0] for t in trees],
            "plain_ms": pm, "plain_mrays_s": rays / (pm * 1e-3) / 1e6,
            "plain_sync_ms": psm, "plain_sync_mrays_s": rays / (psm * 1e-3) / 1e6,
            "batched_ms": bm, "batched_mrays_s": rays / (bm * 1e-3) / 1e6,
            "speedup": pm / bm, "speedup_vs_sync": psm / bm, "autotuned": cfg, "frames_identical": same,
            "plain": "64 vox_cuda_render_device launches back to back (consecutive kernels overlap)",
            "plain_sync": "the same launches, each waited for before the next (host-timed)",
            "form": "persistent kernel, work queue, CUDA graph replay"}

# ------------------------------------------------------------------ our arm

def run_ours(args):
    import ctypes as C

    import torch
    import torch.distributed as dist

    import voxvision_gb300 as vg
    from voxvision_gb300.build import build

    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    if rank == 0 or not os.path.exists(vg._lib.LIB_PATH):
        build()
    if world > 1:
        dist.barrier()
    L = vg.lib()
    vg.set_voxel_size((1, 1, 1))
    vox, ht, tex = make_workload(vg.HostTree.from_voxels)
    states = orbit_states()
    cams = [vg.camera_struct(s) for s in states[:args.frames]]
    nf = len(cams)
    dt = vg.DeviceTree(ht.ptr)
    info = dt.info()

    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    d_tex = torch.from_numpy(tex).cuda()
    frame = torch.empty(H * W, dtype=torch.int32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # algorithmic work of one orbit (untimed)
    counts = torch.zeros(3, dtype=torch.int64, device="cuda")
    for c in cams:
        dt.render_counts_device(c, W, H, counts, stream=sp)
    torch.cuda.synchronize()
    nodes, inner, voxels = (int(x) for x in counts.cpu().tolist())
    rays_step = nf * W * H
    alg_bytes_step = 32 * nodes + 16 * inner + 16 * voxels + 4 * rays_step
    # the kernel traces only the tree's screen rectangle: every other ray is a
    # miss whose one box test (of the root) the counting kernel included
    bb = np.zeros(6, np.float32)
    L.vox_bounding_box(C.c_void_p(ht.ptr), bb.ctypes.data_as(C.c_void_p))
    culled = 0
    for c in cams:
        x0, y0, x1, y1 = vg.frame_rect(bb, c, W, H)
        culled += W * H - (x1 - x0) * (y1 - y0)
    traced_bytes_step = alg_bytes_step - 32 * culled

    fn = L.vox_cuda_render_device
    tex_p, frame_p = C.c_void_p(d_tex.data_ptr()), C.c_void_p(frame.data_ptr())
    cam_refs = [C.byref(c) for c in cams]

    # the orbit as one batch: nf frames into their own device frames, drawn by
    # the persistent batch kernel (warp tiles of every frame from one work
    # queue), replayed from a CUDA graph; tuned once, untimed
    frames_dev = torch.empty((nf, H * W), dtype=torch.int32, device="cuda")
    batch = vg.FrameBatch([(dt, cams[i], W, H, d_tex, frames_dev[i]) for i in range(nf)])
    if args.batch_config:
        batch.set_config(vg.BatchConfig(*[int(x) for x in args.batch_config.split(",")]))
        tuned = batch.config()
    else:
        tuned, _ = batch.autotune(stream=sp, reps=3)

    def step():
        batch.launch(sp)

    def plain_step():
        for cr in cam_refs:
            rc = fn(dt.h, cr, W, H, tex_p, frame_p, sp)
            if rc:
                raise vg.VoxCudaError(rc, "vox_cuda_render_device")

    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = L.vox_cuda_launch_count()
    all_evs = []
    for _ in range(args.steps):
        flush.zero_()
        # one event pair per orbit: an event between two frame launches would
        # end the overlap of one frame's kernel with the next
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        evs[0].record(stream)
        step()
        evs[1].record(stream)
        all_evs.append(evs)
    torch.cuda.synchronize()
    launches = L.vox_cuda_launch_count() - launches0
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clk = clocks.stop()
    step_ms = [evs[0].elapsed_time(evs[1]) for evs in all_evs]
    if args.kernels_only:
        total_s = max_over_ranks([sum(step_ms) * 1e-3], "cuda")[0]
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": job_rate(rays_step * args.steps, world, total_s) / 1e6,
                              "unit": "Mrays/s", "ms_per_step": sum(step_ms) / len(step_ms),
                              "batch_config": tuned, "gpu_launches": int(launches), "clocks": clk}), flush=True)
        if world > 1:
            dist.destroy_process_group()
        return
    # the same orbit as nf plain per-frame launches back to back (their kernels
    # overlap); one event pair per orbit, as an event between launches would
    # end the overlap
    plain_ms = []
    for r in range(args.warmup + args.steps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        plain_step()
        b.record(stream)
        b.synchronize()
        if r >= args.warmup:
            plain_ms.append(a.elapsed_time(b))
    # one frame alone (events on both sides, so no overlap), for reference
    alone = []
    for i in range(0, nf, max(1, nf // 12)):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True); b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn(dt.h, cam_refs[i], W, H, tex_p, frame_p, sp)
        b.record(stream)
        b.synchronize()
        alone.append(a.elapsed_time(b))
    total_s = max_over_ranks([sum(step_ms) * 1e-3], "cuda")[0]
    value = job_rate(rays_step * args.steps, world, total_s) / 1e6

    # e2e: the orbit through the host-buffer entry point vox_cuda_render_frames:
    # every step copies the host texture in and delivers all nf frames into
    # their own page-locked host buffers (drawn in place over the host link)
    host_frames = torch.empty((nf, H * W), dtype=torch.int32).pin_memory()
    frame_ptrs = (C.c_void_p * nf)(*[host_frames[i].data_ptr() for i in range(nf)])
    cam_arr = (vg.CameraStruct * nf)(*cams)
    htex = np.ascontiguousarray(tex)
    htex_p = htex.ctypes.data_as(C.c_void_p)
    for _ in range(max(1, args.warmup)):
        vg.check(L.vox_cuda_render_frames(dt.h, cam_arr, nf, W, H, htex_p, frame_ptrs, sp), "vox_cuda_render_frames")
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        rc = L.vox_cuda_render_frames(dt.h, cam_arr, nf, W, H, htex_p, frame_ptrs, sp)
        if rc:
            raise vg.VoxCudaError(rc, "vox_cuda_render_frames")
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    # the same frames one synchronous vox_cuda_render call each (one host frame)
    hf_p = C.c_void_p(host_frames[0].data_ptr())
    fn_h = L.vox_cuda_render
    for cr in cam_refs[:8]:
        fn_h(dt.h, cr, W, H, htex_p, hf_p, sp)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for cr in cam_refs:
            rc = fn_h(dt.h, cr, W, H, htex_p, hf_p, sp)
            if rc:
                raise vg.VoxCudaError(rc, "vox_cuda_render")
    torch.cuda.synchronize()
    single_s = time.perf_counter() - t0
    e2e_s, single_s = max_over_ranks([e2e_s, single_s], "cuda")
    e2e = {"value": job_rate(rays_step * args.steps, world, e2e_s) / 1e6, "unit": "Mrays/s",
           "h2d_bytes_per_step": 32768 + nf * C.sizeof(vg.CameraStruct), "d2h_bytes_per_step": nf * W * H * 4,
           "call": "vox_cuda_render_frames (host texture and cameras in; each frame drawn on the device and "
                   "copied into its own page-locked host buffer on a second stream while the next frames are "
                   "drawn, the last four as their zeros early and their traced rectangle when drawn; returns "
                   "when all are in host memory)",
           "per_call_value": job_rate(rays_step * args.steps, world, single_s) / 1e6,
           "per_call": "vox_cuda_render, one synchronous call per frame (same frames, one host frame)"}
    del host_frames

    if rank != 0:
        dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    mean_launch_s = float(np.mean(step_ms)) * 1e-3
    achieved = traced_bytes_step / mean_launch_s / 1e9
    traffic = traffic_per_launch(nf)
    l2 = l2_read_gbs(L)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                else "fallback 6.8 TB/s",
                "traffic": traffic,
                "kernel": f"batch_kernel (persistent, {nf} BEST frames a launch, fused ray gen + search + colour)",
                "batch_config": tuned,
                "alg_bytes_per_launch": traced_bytes_step,
                "alg_bytes_per_launch_every_pixel": alg_bytes_step,
                "culled_rays_per_launch": culled,
                "mean_launch_ms": mean_launch_s * 1e3,
                "ms_per_frame": mean_launch_s * 1e3 / nf,
                "plain": {"value": job_rate(rays_step, world, float(np.mean(plain_ms)) * 1e-3) / 1e6,
                          "ms_per_frame": float(np.mean(plain_ms)) / nf,
                          "kernel": "render_kernel, one vox_cuda_render_device launch per frame, consecutive "
                                    "launches overlapping"},
                "launch_alone_ms": float(np.median(alone)),
                "bytes_per_ray": traced_bytes_step / rays_step,
                "visits_per_ray": {"nodes": nodes / rays_step, "inner": inner / rays_step,
                                   "voxels": voxels / rays_step},
                "traced_rays_per_launch": rays_step - culled,
                "traced_mrays_s": (rays_step - culled) / mean_launch_s / 1e6,
                "l2_gbs_measured": l2, "l2_frac": achieved / l2 if l2 else None,
                "l2_probe": "vox_cuda_measure_l2_read: one kernel reading a 32 MiB buffer 1000 times, "
                            "L1 bypassed (ld.global.cg)",
                "issue": issue_figures(nf, rays_step - culled, mean_launch_s,
                                       torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count,
                                       clk["sm_mhz"] if clk else None)}
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sum(step_ms) / len(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(len(vox), nf), "roofline": roofline, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk,
            "tree": {"nodes": info["nodes"], "depth": info["depth"], "device_bytes": info["device_bytes"]}}
    if not args.no_extras:
        btrees = build_batch_trees(vg)
        line["quality"] = measure_quality(torch, vg, dt, ht.ptr, states, tex, d_tex, flush,
                                          cpu=not args.no_cpu_baseline)
        line["dropin"] = measure_dropin(vg, ht.ptr)
        line["incoherent"] = measure_incoherent(torch, vg, dt, flush)
        line["batched"] = measure_batched(torch, vg, flush, d_tex, btrees)
        line["editing"] = measure_editing(vg, vox)
        line["tree_build"] = measure_tree_build(vg)
        line["served"] = measure_served(vg, btrees, tex)
        line["served_device"] = measure_served(vg, btrees, tex, frames_on_device=True,
                                               rates=(1000, 2000, 5000, 10000, 15000, 20000, 30000))
    if not args.no_cpu_baseline:
        # the CPU leg: the oracle checks every timed frame (the last launch's
        # nf device frames) over its own tree and cameras, then is timed
        line["parity"] = oracle_check_orbit(frames_dev, vox, ht.ptr, tex, nf)
        cb = cpu_baseline_sample(ht.ptr, states, tex)
        cb.update(cpu_reference_details(ht.ptr, states, tex, cb["cores"]))
        line["cpu_baseline"] = cb
    if not args.no_extras:
        # compact summaries last, where a truncated log still shows them
        b = line["batched"]
        line["batched_summary"] = {"frames": b["frames"], "batched_mrays_s": round(b["batched_mrays_s"]),
                                   "plain_mrays_s": round(b["plain_mrays_s"]),
                                   "plain_sync_mrays_s": round(b["plain_sync_mrays_s"]),
                                   "speedup_vs_plain": round(b["speedup"], 2),
                                   "speedup_vs_plain_sync": round(b["speedup_vs_sync"], 2),
                                   "frames_identical": b["frames_identical"]}

        def served_summary(sv):
            d = {r: [round(v["achieved_hz"]), round(v["frame_p50_ms"], 2), round(v["frame_p99_ms"], 2),
                     round(v["mrays_s"])] for r, v in sv["rates"].items()}
            d["plain_sync_mrays_s"] = round(sv["plain"]["mrays_s"])
            d["best_vs_plain_sync"] = round(sv["speedup_vs_plain_sync"], 2)
            return d
        line["served_summary"] = {"fields": "offered Hz: [served Hz, frame p50 ms, frame p99 ms, Mrays/s]",
                                  "host_frames": served_summary(line["served"]),
                                  "device_frames": served_summary(line["served_device"])}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ------------------------------------------------------------ reference arm

def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.set_voxel((1, 1, 1))
    vox, tree, tex = make_workload(orc.OracleTree.from_voxels)
    states = oracle_orbit_states()
    n = orc.nthreads_default()

    def step():
        for st in states:
            orc.render_best(tree.ptr, st, W, H, tex, nthreads=n)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    value = NFRAMES * W * H * args.steps / dt / 1e6
    line = {"metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(len(vox)), "impl": "reference",
            "cpu_baseline": dict({"value": value, "unit": "Mrays/s", "cores": n, "kind": "port",
                                  "sample": f"full {NFRAMES}-frame orbit per step, {W}x{H}, BEST, "
                                            f"C restatement of tree.c/search.c/renderer.c/simple-camera.c "
                                            f"on {n} threads"},
                                 **cpu_reference_details(tree.ptr, states, tex, n)),
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.tree_build:
        import voxvision_gb300 as vg
        vg.set_voxel_size((1, 1, 1))
        size = {256: (256, 2, 0.08), 512: (512, 3, 0.10)}.get(args.tree_build, (args.tree_build, 2, 0.08))
        print(json.dumps({"tree_build": measure_tree_build(vg, (size,), reps=args.reps)}), flush=True)
        return
    if args.quality:
        import torch

        import voxvision_gb300 as vg
        vg.set_voxel_size((1, 1, 1))
        vox, ht, tex = make_workload(vg.HostTree.from_voxels)
        dt = vg.DeviceTree(ht.ptr)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        q = measure_quality(torch, vg, dt, ht.ptr, orbit_states(), tex, torch.from_numpy(tex).cuda(), flush,
                            cpu=not args.no_cpu_baseline, nframes=args.quality)
        print(json.dumps({"quality": q}), flush=True)
        return
    if args.batched:
        import torch

        import voxvision_gb300 as vg
        vg.set_voxel_size((1, 1, 1))
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        tex = workloads().texture32(7)
        print(json.dumps({"batched": measure_batched(torch, vg, flush, torch.from_numpy(tex).cuda())}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
