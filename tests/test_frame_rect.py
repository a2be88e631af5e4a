"""The screen rectangle that the BEST frame kernel traces (vox_cuda_frame_rect)
is conservative: every pixel whose ray enters the tree's bounding box in the
oracle's search -- and so every pixel the reference can draw -- lies inside
it.  Host arithmetic only; no GPU."""
import math

import numpy as np
import pytest

from oracle import oracle as orc
import voxvision_gb300 as vg
from voxvision_gb300 import workloads as wl
from voxvision_gb300.cameras import HostCamera
from voxvision_gb300._lib import CAMERA_DOOM, CAMERA_SIMPLE

W, H = 128, 96


@pytest.fixture(scope="module")
def scene():
    vg.set_voxel_size((1, 1, 1))
    orc.set_voxel((1, 1, 1))
    vox = wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20))
    tree = orc.OracleTree.from_voxels(vox)
    bbox = tree.dump()["boxes"][0]
    return tree, bbox


def entered_pixels(tree, cam: HostCamera):
    """(H, W) bool: the ray of the pixel enters the root box in the oracle's
    search (inner node entered, voxel tested or any deeper node tested)."""
    d = np.array([cam.screen2world(x, y) for y in range(H) for x in range(W)], np.float32)
    o = np.tile(cam.position(), (W * H, 1)).astype(np.float32)
    c = orc.ray_counts_per_ray(tree.ptr, o, d)
    return ((c[:, 0] > 1) | (c[:, 1] > 0) | (c[:, 2] > 0)).reshape(H, W)


def cameras():
    rng = np.random.default_rng(21)
    centre = np.array([32.0, 32.0, 32.0])
    half_diag = 32.0 * math.sqrt(3.0)
    out = []
    for kind in (CAMERA_SIMPLE, CAMERA_DOOM):
        for dist in (1.05, 1.3, 2.0, 5.0, 60.0):
            for _ in range(3):
                az, el = rng.uniform(0, 2 * math.pi), rng.uniform(-60, 60)
                pos = wl.pose_position(centre, dist * half_diag, az, el)
                target = centre + rng.normal(0, 25.0, 3)            # tree partly or wholly off-screen
                out.append((kind, pos, target, float(rng.choice([0.3, 1.0, 2.0])), None))
        out.append((kind, centre + 3.0, centre + 40.0, 1.0, "full"))                  # inside the box
        out.append((kind, centre + [0, 200.0, 5.0], centre + [0, 400.0, 5.0], 1.0, "empty"))   # looking away
    return out


@pytest.mark.parametrize("case", range(len(cameras())))
def test_rect_holds_every_pixel_that_enters_the_tree(scene, case):
    tree, bbox = scene
    kind, pos, target, fov, expect = cameras()[case]
    cam = HostCamera(kind)
    cam.set_fov(fov)
    cam.set_window_size(W, H)
    cam.set_position(pos)
    cam.look_at(np.asarray(target, np.float32))
    x0, y0, x1, y1 = vg.frame_rect(bbox, cam.gpu_struct(), W, H)
    assert x0 % 8 == 0 and y0 % 4 == 0 and x1 <= W and y1 <= H
    assert (x0 < x1 and y0 < y1) or (x0, y0, x1, y1) == (0, 0, 0, 0)
    inside = np.zeros((H, W), bool)
    inside[y0:y1, x0:x1] = True
    entered = entered_pixels(tree, cam)
    assert not (entered & ~inside).any(), f"{int((entered & ~inside).sum())} pixels enter outside the rectangle"
    frame, _ = orc.render_best(tree.ptr, cam.state(), W, H, wl.texture32(7))
    assert not ((frame != 0) & ~inside).any()
    if expect == "full":
        assert (x0, y0, x1, y1) == (0, 0, W, H), "a camera inside the box sees every pixel"
    if expect == "empty":
        assert (x0, y0, x1, y1) == (0, 0, 0, 0), "a box behind the camera has no pixel"


def test_rect_is_tight_for_a_distant_tree(scene):
    """The 64^3 tree seen from far away covers a small part of the frame."""
    tree, bbox = scene
    cam = HostCamera(CAMERA_SIMPLE)
    cam.set_window_size(1920, 1080)
    cam.set_position((32.0, -600.0, 32.0))
    cam.look_at(np.array([32.0, 32.0, 32.0], np.float32))
    x0, y0, x1, y1 = vg.frame_rect(bbox, cam.gpu_struct(), 1920, 1080)
    assert 0 < (x1 - x0) * (y1 - y0) < 0.05 * 1920 * 1080


def test_rect_rejects_bad_arguments(scene):
    _, bbox = scene
    cam = HostCamera(CAMERA_SIMPLE)
    cam.set_window_size(W, H)
    with pytest.raises(vg.VoxCudaError):
        vg.frame_rect(bbox, cam.gpu_struct(), 100, 96)
    bad = cam.gpu_struct()
    bad.kind = 7
    with pytest.raises(vg.VoxCudaError):
        vg.frame_rect(bbox, bad, W, H)
    nan = cam.gpu_struct()
    nan.mul = float("nan")
    assert vg.frame_rect(bbox, nan, W, H) == (0, 0, W, H)
