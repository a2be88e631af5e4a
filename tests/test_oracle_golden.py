"""Pin the CPU oracle to the reference's own outputs (tests/golden/*.npz,
generated by tests/golden/make_golden.py from the reference sources)."""
import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import MISS, TREE_CASES, dumps_equal, load, same_points, tree_dump


def _tree_for(g):
    orc.set_voxel(tuple(g["voxel"]))
    if "voxels" in g:
        t = orc.OracleTree.from_voxels(g["voxels"].astype(np.float32))
        ok, key = dumps_equal(t.dump(), tree_dump(g))
        assert ok, f"oracle vox_make_tree differs from the reference in {key}"
        return t
    return orc.OracleTree.from_dump(tree_dump(g))


@pytest.mark.parametrize("case", TREE_CASES)
def test_oracle_rays_match_reference(case):
    g = load(case)
    t = _tree_for(g)
    leaf, slot, pts, _ = t.rays(g["ray_origins"], g["ray_dirs"], nthreads=2)
    assert np.array_equal(leaf, g["ray_leaf"])
    hit = leaf != MISS
    ok, nbad = same_points(pts, g["ray_points"], hit)
    assert ok, f"{nbad} intersection points differ"
    # a dense leaf reports slot 0xFF, a regular leaf a valid dot index
    flags = tree_dump(g)["flags"]
    dn = tree_dump(g)["dots_num"]
    for i in np.nonzero(hit)[0]:
        f = flags[leaf[i]]
        if f & 2:
            assert slot[i] == 0xFF
        else:
            assert slot[i] < dn[leaf[i]]
    orc.set_voxel((1, 1, 1))


@pytest.mark.parametrize("case", TREE_CASES)
def test_oracle_leaf_rooted_rays(case):
    g = load(case)
    if "root_ids" not in g:
        pytest.skip("no leaves")
    t = _tree_for(g)
    pre = t.preorder()
    for i in range(len(g["root_ids"])):
        rid = int(g["root_ids"][i])
        leaf, slot, pts, _ = t.rays(g["root_origins"][i:i + 1], g["root_dirs"][i:i + 1],
                                    root=int(pre[rid]), nthreads=1)
        assert leaf[0] == g["root_leaf"][i]
        if leaf[0] != MISS:
            assert same_points(pts, g["root_points"][i:i + 1], np.array([True]))[0]
    orc.set_voxel((1, 1, 1))


@pytest.mark.parametrize("case", TREE_CASES)
def test_oracle_balls_match_reference(case):
    g = load(case)
    t = _tree_for(g)
    hit, _ = t.balls(g["ball_centres"], g["ball_radii"], nthreads=2)
    assert np.array_equal(hit, g["ball_hit"])
    orc.set_voxel((1, 1, 1))


def test_regression_ray_hits():
    """tests.c:600-659: the ray from (-2,-2,0) along (1,1,-1) hits the cross."""
    g = load("g676d50c")
    t = orc.OracleTree.from_dump(tree_dump(g))
    leaf, _, pts, _ = t.rays(g["regress_origin"], g["regress_dir"], nthreads=1)
    assert leaf[0] != MISS and leaf[0] == g["regress_leaf"][0]


def test_oracle_screen2world_matches_reference_cameras():
    g = load("cameras")
    for i in range(int(g["ncams"])):
        st = {k[len(f"c{i}_"):]: g[k] for k in g if k.startswith(f"c{i}_")}
        for (x, y), ray in zip(st["pixels"], st["rays"]):
            r = orc.screen2world(st, int(x), int(y))
            assert np.array_equal(r.view(np.uint32), ray.astype(np.float32).view(np.uint32)), (i, x, y)


def test_oracle_render_matches_reference_search():
    """BEST-quality frame: every pixel colour follows from the reference's hit."""
    g = load("render64")
    orc.set_voxel((1, 1, 1))
    t = orc.OracleTree.from_voxels(g["voxels"].astype(np.float32))
    ok, key = dumps_equal(t.dump(), tree_dump(g))
    assert ok, key
    from voxvision_gb300 import workloads as wl
    tex = wl.texture32(7)
    st = dict(kind=0, position=g["cam_position"], rotation=g["cam_rotation"], mul=g["cam_mul"],
              xsub=g["cam_xsub"], ysub=g["cam_ysub"])
    w, h = int(g["w"]), int(g["h"])
    img, _ = orc.render_best(t.ptr, st, w, h, tex, nthreads=2)
    hit = g["pix_leaf"] != MISS
    pts = g["pix_points"]
    idx = (np.abs(np.trunc(pts).astype(np.int64)) & 31)
    c = tex[idx[:, 0] * 1024 + idx[:, 1] * 32 + idx[:, 2]].astype(np.uint32)
    expect = np.where(hit, 0xFF000000 | (c << 16) | (c << 8) | c, 0).astype(np.uint32)
    assert np.array_equal(img.ravel(), expect)


def test_oracle_ray_buffer_camera_draws_its_directions():
    """Camera kind 2 (a class known only by what its screen2world returns)
    draws, in every quality, the frame of the class whose directions it
    holds: here the reference-pinned simple camera of the render64 case."""
    g = load("render64")
    orc.set_voxel((1, 1, 1))
    t = orc.OracleTree.from_voxels(g["voxels"].astype(np.float32))
    from voxvision_gb300 import workloads as wl
    tex = wl.texture32(7)
    st = dict(kind=0, position=g["cam_position"], rotation=g["cam_rotation"], mul=g["cam_mul"],
              xsub=g["cam_xsub"], ysub=g["cam_ysub"])
    w, h = int(g["w"]), int(g["h"])
    table = np.array([[orc.screen2world(st, x, y) for x in range(w)] for y in range(h)], np.float32)
    buf = dict(kind=2, position=g["cam_position"], rays=table)
    assert np.array_equal(orc.screen2world(buf, 5, 3), table[3, 5])
    for q in (0, 1, 2, 2 | 4, 2 | 8):
        a, _ = orc.render_quality(t.ptr, st, w, h, q, tex, nthreads=2)
        b, _ = orc.render_quality(t.ptr, buf, w, h, q, tex, nthreads=2)
        assert np.array_equal(a, b), q


def test_oracle_camera_setup_matches_reference_cameras():
    """The oracle's simple-camera set-up (window size, position, look_at)
    leaves the reference camera's fields bit for bit (cameras.npz: the
    reference's simple-camera.c compiled here, driven through its vtable)."""
    g = load("cameras")
    checked = 0
    for i in range(int(g["ncams"])):
        if int(g[f"c{i}_kind"]) != 0 or np.isnan(g[f"c{i}_lookat"]).any():
            continue
        w, h = (int(x) for x in g[f"c{i}_wh"])
        st = orc.camera_simple(g[f"c{i}_setpos"], g[f"c{i}_lookat"], w, h, float(g[f"c{i}_fov"]))
        for k in ("position", "rotation", "mul", "xsub", "ysub"):
            a = np.asarray(st[k], np.float32).view(np.uint32)
            b = np.asarray(g[f"c{i}_{k}"], np.float32).view(np.uint32)
            assert np.array_equal(a, b), (i, k)
        checked += 1
    assert checked == 5


def test_oracle_orbit_cameras_match_library_cameras():
    """The 120 orbit cameras of the 1080p benchmark set up by the oracle equal
    the library's simple-camera set up the same way (both follow
    simple-camera.c; the benchmark's reference arm uses the oracle's)."""
    import math
    from voxvision_gb300 import workloads as wl
    from voxvision_gb300.cameras import orbit_camera
    centre, radius = (128.0, 128.0, 128.0), 1.5 * 256 * math.sqrt(3.0)
    for f in range(120):
        lib_st = orbit_camera(f, 120, 1920, 1080, centre, radius).state()
        orc_st = orc.camera_simple(wl.orbit_pose(f, 120, centre, radius, 20.0), centre, 1920, 1080, 1.0)
        for k in ("position", "rotation", "mul", "xsub", "ysub"):
            a = np.asarray(orc_st[k], np.float32).view(np.uint32)
            b = np.asarray(lib_st[k], np.float32).view(np.uint32)
            assert np.array_equal(a, b), (f, k)
