"""The decomposition behind the GPU's FAST and ADAPTIVE frames
(render_squares_kernel), checked on the CPU with the oracle's own search:
every pixel's search from the root made first; then, per 4x4 square, rounds
in which every pixel still to be walked makes the search from the leaf the
walk holds, followed by renderer.c:215-318's walk over those results, which
ends the round wherever it moves to a leaf the round did not search from.
This gives the oracle's sequential frame pixel for pixel -- for random
cameras of both classes, every quality, and a non-unit voxel size.  No GPU
is used."""
import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import MISS

ORDER = [0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15]   # renderer.c:23-25
F = np.float32


def _sqr(a, b):
    r = F(0)
    for i in range(3):
        d = F(F(a[i]) - F(b[i]))
        r = F(r + F(d * d))
    return r


def _color(p, tex, voxel):
    x, y, z = (abs(int(F(F(p[i]) / F(voxel[i])))) & 31 for i in range(3))
    c = int(tex[x * 1024 + y * 32 + z])
    return 0xFF000000 | (c << 16) | (c << 8) | c


def two_phase(tree, state, w, h, quality, tex, voxel):
    pre = tree.preorder()
    origin = np.asarray(state["position"], F)
    dirs = np.array([[orc.screen2world(state, x, y) for x in range(w)] for y in range(h)], F)
    # phase 1: every pixel's search from the root
    leaf, _, pts, _ = tree.rays(np.tile(origin, (w * h, 1)), dirs.reshape(-1, 3), nthreads=1)
    leaf, pts = leaf.reshape(h, w), pts.reshape(h, w, 3)
    out = np.zeros((h, w), np.uint32)
    rounds = 0
    rnd, merge_mode = quality & 3, quality & 12
    for ys in range(0, h, 4):
        for xs in range(0, w, 4):
            sq = np.zeros(16, np.uint32)
            have, leaf_id, inter = False, None, None
            mode, istart, iend, merge = rnd, 0, 16, False
            if mode == 2:                                        # ADAPTIVE: renderer.c:240-282
                merge, istart, mode = merge_mode == 4, 1, 1
                have = leaf[ys, xs] != MISS
                if have:
                    leaf_id, inter, iend = int(leaf[ys, xs]), pts[ys, xs], 15
                    sq[0] = _color(inter, tex, voxel)
                    if leaf[ys + 3, xs + 3] != MISS:
                        i2 = pts[ys + 3, xs + 3]
                        sq[15] = _color(i2, tex, voxel)
                        d1 = _sqr(inter, origin)
                        d2 = _sqr(dirs[ys, xs], (0, 0, 0))
                        with np.errstate(all="ignore"):
                            crit = F(F(d1 / d2) * _sqr(dirs[ys, xs], dirs[ys + 3, xs + 3]))
                            ratio = F(_sqr(inter, i2) / crit)
                        if float(ratio) > 1.69:
                            mode = 0
                        if d1 > F(22500):
                            merge = True if (mode == 1 and merge_mode == 8) else merge
                        else:
                            merge = False
            # the walk in rounds: searches from one leaf for every pixel still
            # to come, then the reference's decisions over them
            res = {}                                            # pixel -> (have, point, merged)
            pos = istart
            while pos < iend:
                searched, frm = mode == 1 and have, leaf_id
                found = {}
                if searched:
                    for i in range(pos, iend):
                        if merge and (i & 1):
                            continue
                        p = ORDER[i]
                        py, px = ys + p // 4, xs + p % 4
                        lf, _, lp, _ = tree.rays(origin[None], dirs[py, px][None], root=int(pre[frm]), nthreads=1)
                        found[p] = (lf[0] != MISS, lp[0], int(lf[0]))
                stop = iend
                i = pos
                while i < stop:
                    p = ORDER[i]
                    py, px = ys + p // 4, xs + p % 4
                    m = merge and (i & 1)
                    if not m:
                        from_root = True
                        if mode == 1 and have and found[p][0]:   # the search from the leaf met a voxel
                            inter, leaf_id, from_root = found[p][1], found[p][2], False
                        if from_root:                           # ... else the pixel's root result
                            have = leaf[py, px] != MISS
                            if have:
                                inter = pts[py, px]
                                if mode == 1 and not (searched and int(leaf[py, px]) == frm):
                                    stop = i + 1                # later pixels search from another leaf
                                leaf_id = int(leaf[py, px])
                    res[p] = (have, inter, m)
                    i += 1
                rounds += 1
                pos = stop
            colour = {p: _color(v[1], tex, voxel) for p, v in res.items() if v[0] and not v[2]}
            for p, (hv, _, m) in res.items():
                if hv:
                    sq[p] = sq[ORDER[ORDER.index(p) - 1]] if m else colour[p]
            out[ys:ys + 4, xs:xs + 4] = sq.reshape(4, 4)
    return out, rounds


@pytest.fixture(scope="module")
def scene():
    from voxvision_gb300 import workloads as wl
    vox = wl.voxels_from_mask(wl.blobs_volume(48, 16, 5, 0.22)).astype(F)
    return vox, wl.texture32(11)


@pytest.mark.parametrize("voxel", [(1.0, 1.0, 1.0), (0.5, 1.0, 2.0)])
def test_two_phase_frames_equal_the_sequential_loop(scene, voxel):
    from voxvision_gb300.cameras import HostCamera
    vox, tex = scene
    orc.set_voxel(voxel)
    try:
        tree = orc.OracleTree.from_voxels(vox * np.asarray(voxel, F))
        centre = np.asarray(voxel, F) * F(24)
        rng = np.random.default_rng(21)
        w, h = 48, 32
        checked, fast_differs = 0, 0
        for k in range(6):
            cam = HostCamera(k % 2)
            cam.set_window_size(w, h)
            az, el, r = rng.uniform(0, 2 * np.pi), rng.uniform(-0.6, 0.9), rng.uniform(45, 120)
            cam.set_position(centre + r * np.array([np.cos(az) * np.cos(el), np.sin(az) * np.cos(el), np.sin(el)]))
            cam.look_at(centre + rng.uniform(-8, 8, 3))
            st = cam.state()
            frames = {}
            for q in (0, 1, 2, 2 | 4, 2 | 8):
                ref, _ = orc.render_quality(tree.ptr, st, w, h, q, tex, nthreads=1)
                got, _ = two_phase(tree, st, w, h, q, tex, voxel)
                assert np.array_equal(got, ref), (k, q)
                checked += int((ref != 0).sum())
                frames[q] = ref
            fast_differs += int((frames[1] != frames[0]).sum())
        assert checked > 1000          # the cameras see the scene
        assert fast_differs > 0        # and FAST's searches from a leaf change pixels BEST draws otherwise
    finally:
        orc.set_voxel((1.0, 1.0, 1.0))
