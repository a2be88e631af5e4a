"""Generate the golden vectors under tests/golden/ from the reference itself.

Run where the reference sources are present (REF = the voxvision source tree):

    make -C oracle ref REF=...    # compiles the reference's own voxtrees and
                                  # camera sources into oracle/_ref/
    python tests/golden/make_golden.py          # everything
    python tests/golden/make_golden.py edits    # the tree-editing fixtures only
    python tests/golden/make_golden.py vectops  # the vector-helper fixture only
    python tests/golden/make_golden.py geom     # the metrics and tree-dump fixture only
    make -C oracle ref-sse REF=... && python tests/golden/make_golden.py sse
                                                # the SSE-layout trees (x86 hosts only)
    make -C oracle ref-lights REF=... && python tests/golden/make_golden.py lights
                                                # the light manager and its M-tree

Every expected value here comes from the reference's compiled code:
vox_make_tree, vox_insert_voxel, vox_delete_voxel, vox_ray_tree_intersection,
vox_tree_ball_collidep, the geom.c metrics and vox_dump_tree
(src/voxtrees/tree.c, search.c, geom.c) and the simple-camera / doom-camera
plugins with their vector helpers (src/voxrnd/*-camera.c, vect-ops.c).
The oracle library is used only to serialise the reference-built trees
(orc_dump / orc_preorder walk the same struct layout).  The fixtures are
small .npz files that the tests read on any host; this script is the only
thing that needs the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as orc  # noqa: E402
from voxvision_gb300 import workloads as wl  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(ROOT, "oracle", "_ref")

ref = C.CDLL(os.path.join(REF, "libvoxtrees_ref.so"))
vp = C.c_void_p
ref.vox_make_tree.argtypes = [vp, C.c_size_t]; ref.vox_make_tree.restype = vp
ref.vox_destroy_tree.argtypes = [vp]
ref.vox_ray_tree_intersection.argtypes = [vp, vp, vp, vp]; ref.vox_ray_tree_intersection.restype = vp
ref.vox_tree_ball_collidep.argtypes = [vp, vp, C.c_float]; ref.vox_tree_ball_collidep.restype = C.c_int
ref.vox_insert_voxel.argtypes = [C.POINTER(vp), vp]; ref.vox_insert_voxel.restype = C.c_int
ref.vox_delete_voxel.argtypes = [C.POINTER(vp), vp]; ref.vox_delete_voxel.restype = C.c_int
ref.vox_set_voxel_size.argtypes = [C.c_float] * 3


def P(a):
    return a.ctypes.data_as(vp)


def set_voxel(v):
    ref.vox_set_voxel_size(*v)
    orc.set_voxel(v)


def ref_tree_from_voxels(vox):
    s = np.ascontiguousarray(vox, dtype=np.float32).copy()
    return ref.vox_make_tree(P(s), s.shape[0])


def preorder_map(tree):
    pre = orc.OracleTree(None)
    pre.ptr = None
    n = orc.lib().orc_count_nodes(tree)
    arr = np.zeros(max(n, 1), np.uint64)
    orc.lib().orc_preorder(tree, P(arr))
    return {int(p): i for i, p in enumerate(arr[:n])}, arr[:n]


def ref_rays(tree, roots, origins, dirs, pmap):
    n = origins.shape[0]
    leaf = np.full(n, 0xFFFFFFFF, np.uint32)
    pts = np.zeros((n, 3), np.float32)
    res = np.zeros(3, np.float32)
    for i in range(n):
        o = np.ascontiguousarray(origins[i]); d = np.ascontiguousarray(dirs[i])
        r = ref.vox_ray_tree_intersection(roots[i] if roots is not None else tree, P(o), P(d), P(res))
        if r:
            leaf[i] = pmap[int(r)]
            pts[i] = res
    return leaf, pts


def ref_balls(tree, centres, radii):
    out = np.zeros(centres.shape[0], np.uint8)
    for i in range(centres.shape[0]):
        c = np.ascontiguousarray(centres[i])
        out[i] = ref.vox_tree_ball_collidep(tree, P(c), C.c_float(float(radii[i])))
    return out


def edge_rays(box_min, box_max, n, seed, voxel):
    """A mix of random and degenerate rays around a bounding box."""
    rng = np.random.default_rng(seed)
    lo = np.asarray(box_min, np.float64); hi = np.asarray(box_max, np.float64)
    ext = hi - lo
    o, d = [], []
    k = n // 8
    # 1: random origins in a 2x box, random directions
    o.append(lo - ext / 2 + 2 * ext * rng.random((k, 3))); d.append(rng.normal(size=(k, 3)))
    # 2: axis-aligned directions from lattice points (voxel corners)
    g = np.floor(lo / voxel) * voxel + np.round(rng.random((k, 3)) * ext / voxel) * voxel
    axis = rng.integers(0, 3, k); sign = rng.choice([-1.0, 1.0], k)
    dd = np.zeros((k, 3)); dd[np.arange(k), axis] = sign
    g[np.arange(k), axis] = np.where(sign > 0, lo[axis] - 2 * voxel[axis], hi[axis] + 2 * voxel[axis])
    o.append(g); d.append(dd)
    # 3: one zero component (with signed zeros)
    r = rng.normal(size=(k, 3)); z = rng.integers(0, 3, k)
    r[np.arange(k), z] = np.where(rng.random(k) < 0.5, 0.0, -0.0)
    o.append(lo - ext / 2 + 2 * ext * rng.random((k, 3))); d.append(r)
    # 4: origins inside the box
    o.append(lo + ext * rng.random((k, 3))); d.append(rng.normal(size=(k, 3)))
    # 5: integer origins inside, integer directions (ties and exact faces)
    o.append(np.floor(lo + ext * rng.random((k, 3)))); d.append(rng.integers(-2, 3, (k, 3)).astype(np.float64))
    # 6: diagonal rays aimed at the centre from lattice points outside
    c = (lo + hi) / 2
    st = np.floor(lo - ext * rng.random((k, 3)))
    o.append(st); d.append(np.sign(c - st))
    # 7: aimed at random voxel corners from far away
    tgt = np.floor(lo + ext * rng.random((k, 3)))
    src = tgt + rng.normal(size=(k, 3)) * ext.max()
    o.append(src); d.append(tgt - src)
    # 8: two zero components, plus a few all-zero directions
    m = n - 7 * k
    dd = np.zeros((m, 3)); ax = rng.integers(0, 3, m)
    dd[np.arange(m), ax] = rng.normal(size=m)
    dd[: max(1, m // 50)] = 0.0
    o.append(lo - ext / 4 + 1.5 * ext * rng.random((m, 3))); d.append(dd)
    return (np.ascontiguousarray(np.concatenate(o).astype(np.float32)),
            np.ascontiguousarray(np.concatenate(d).astype(np.float32)))


def edge_balls(box_min, box_max, n, seed):
    rng = np.random.default_rng(seed)
    lo = np.asarray(box_min, np.float64); hi = np.asarray(box_max, np.float64)
    ext = hi - lo
    k = n // 2
    c1 = lo - ext / 4 + 1.5 * ext * rng.random((k, 3)); r1 = 8 * rng.random(k)
    c2 = np.round(lo + ext * rng.random((n - k, 3))); r2 = rng.choice([0.0, 0.5, 1.0, 1.5, 2.0, -1.0], n - k)
    return (np.ascontiguousarray(np.concatenate([c1, c2]).astype(np.float32)),
            np.ascontiguousarray(np.concatenate([r1, r2]).astype(np.float32)))


def save_case(name, tree, voxel, voxels=None, nrays=8000, nballs=4000, seed=0, extra=None,
              leaf_roots=1000):
    pmap, pre = preorder_map(tree)
    dump = orc.dump_tree(tree)
    out = {f"tree_{k}": v for k, v in dump.items()}
    out["voxel"] = np.asarray(voxel, np.float32)
    if voxels is not None:
        out["voxels"] = np.asarray(voxels, np.float32)
    if tree:
        bmin, bmax = dump["boxes"][0][:3], dump["boxes"][0][3:]
    else:
        bmin, bmax = np.zeros(3), np.ones(3)
    o, d = edge_rays(bmin, bmax, nrays, seed, np.asarray(voxel, np.float64))
    leaf, pts = ref_rays(tree, None, o, d, pmap)
    out.update(ray_origins=o, ray_dirs=d, ray_leaf=leaf, ray_points=pts)
    # searches rooted at a leaf (what FAST mode does, renderer.c:297)
    leaves = [i for i in range(len(pre)) if dump["flags"][i] & 3]
    if leaves and leaf_roots:
        rng = np.random.default_rng(seed + 1)
        ridx = rng.choice(np.asarray(leaves), leaf_roots).astype(np.uint32)
        lb = dump["boxes"][ridx]
        lo_, hi_ = lb[:, :3].astype(np.float64), lb[:, 3:].astype(np.float64)
        src = lo_ - 3 + (hi_ - lo_ + 6) * rng.random((leaf_roots, 3))
        tgt = lo_ + (hi_ - lo_) * rng.random((leaf_roots, 3))
        ro = np.ascontiguousarray(src.astype(np.float32))
        rd = np.ascontiguousarray((tgt - src).astype(np.float32))
        rl, rp = ref_rays(tree, [int(pre[i]) for i in ridx], ro, rd, pmap)
        out.update(root_ids=ridx, root_origins=ro, root_dirs=rd, root_leaf=rl, root_points=rp)
    c, r = edge_balls(bmin, bmax, nballs, seed + 2)
    out.update(ball_centres=c, ball_radii=r, ball_hit=ref_balls(tree, c, r))
    if extra:
        out.update(extra)
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: nodes={len(pre)} rays hit={np.mean(leaf != 0xFFFFFFFF):.3f} "
          f"balls hit={out['ball_hit'].mean():.3f} size={os.path.getsize(path)} B")


# ---------------------------------------------------------------- cameras

class SimpleCam(C.Structure):      # simple-camera.c:10-17
    _fields_ = [("iface", vp), ("xsub", C.c_float), ("ysub", C.c_float), ("position", C.c_float * 3),
                ("rotation", C.c_float * 4), ("mul", C.c_float), ("fov", C.c_float)]


class DoomCam(C.Structure):        # doom-camera.c:8-15
    _fields_ = [("iface", vp), ("xsub", C.c_float), ("ysub", C.c_float), ("position", C.c_float * 3),
                ("phi", C.c_float), ("sinphi", C.c_float), ("cosphi", C.c_float), ("k", C.c_float),
                ("mul", C.c_float), ("fov", C.c_float)]


class Module(C.Structure):
    _fields_ = [("type", C.c_int), ("methods", vp)]


S2W = C.CFUNCTYPE(None, vp, vp, C.c_int, C.c_int)
SETDOT = C.CFUNCTYPE(None, vp, C.c_char_p, vp)
SETNUM = C.CFUNCTYPE(None, vp, C.c_char_p, C.c_float)
DOTM = C.CFUNCTYPE(None, vp, vp)
WS = C.CFUNCTYPE(None, vp, C.c_int, C.c_int)
CONS = C.CFUNCTYPE(vp, vp)


class RefCamera:
    """A camera object from the reference plugin, driven through its vtable
    (camera.h:17-117: set_property_number, set_property_dot, screen2world,
    rotate_camera, move_camera, look_at, get_position, set_window_size,
    construct_camera, destroy_camera)."""

    def __init__(self, kind):
        self.kind = kind
        lib = C.CDLL(os.path.join(REF, f"lib{'simple' if kind == 0 else 'doom'}cam_ref.so"))
        lib.module_init.restype = C.POINTER(Module)
        meth = lib.module_init().contents.methods
        tbl = C.cast(meth, C.POINTER(vp * 10)).contents
        self.obj = CONS(tbl[8])(None)
        self.lib = lib
        itbl = C.cast(C.cast(self.obj, C.POINTER(vp))[0], C.POINTER(vp * 10)).contents
        self.set_num = SETNUM(itbl[0]); self.set_dot = SETDOT(itbl[1]); self.s2w = S2W(itbl[2])
        self.rotate = DOTM(itbl[3]); self.move = DOTM(itbl[4]); self.look_at = DOTM(itbl[5])
        self.set_ws = WS(itbl[7])

    def dot(self, name, v):
        a = np.asarray(v, np.float32)
        self.set_dot(self.obj, name.encode(), P(a))

    def state(self):
        st = C.cast(self.obj, C.POINTER(SimpleCam if self.kind == 0 else DoomCam)).contents
        s = dict(kind=self.kind, position=np.array(st.position[:], np.float32),
                 mul=st.mul, xsub=st.xsub, ysub=st.ysub, fov=st.fov)
        if self.kind == 0:
            s["rotation"] = np.array(st.rotation[:], np.float32)
        else:
            s.update(sinphi=st.sinphi, cosphi=st.cosphi, k=st.k, phi=st.phi)
        return s

    def ray(self, sx, sy):
        out = np.zeros(3, np.float32)
        self.s2w(self.obj, P(out), sx, sy)
        return out


def camera_cases():
    """Camera states after the reference's own set-up calls, plus screen2world
    outputs on a pixel sample."""
    rng = np.random.default_rng(5)
    recs = []
    setups = [
        (256, 256, (160, -96, 112), (32, 32, 32), None, 1.0),
        (1920, 1080, (128 + 665, 128, 350), (128, 128, 128), None, 1.0),
        (100, 100, (0, 0, 0), None, (0, 0, np.pi / 2), 1.0),
        (640, 480, (-100, 20, -20), (0, 0, 0), None, 0.8),
        (240, 320, (10, 300, 40), (5, 6, 7), None, 1.2),
        (3840, 2160, (500, 500, 500), (0, 0, 0), None, 1.0),
    ]
    for kind in (0, 1):
        for (w, h, pos, at, rot, fov) in setups:
            cam = RefCamera(kind)
            cam.set_num(cam.obj, b"fov", C.c_float(fov))
            cam.set_ws(cam.obj, w, h)
            cam.dot("position", pos)
            if rot is not None:
                cam.dot("rotation", rot)
            if at is not None:
                a = np.asarray(at, np.float32)
                cam.look_at(cam.obj, P(a))
            st = cam.state()
            px = np.stack([rng.integers(0, w, 64), rng.integers(0, h, 64)], 1)
            px = np.concatenate([px, [[0, 0], [w - 1, h - 1], [w // 2, h // 2], [w, h]]]).astype(np.int32)
            rays = np.stack([cam.ray(int(x), int(y)) for x, y in px])
            recs.append((st, w, h, pos, at, rot, fov, px, rays))
    out = {}
    for i, (st, w, h, pos, at, rot, fov, px, rays) in enumerate(recs):
        out[f"c{i}_kind"] = np.int32(st["kind"])
        out[f"c{i}_wh"] = np.array([w, h], np.int32)
        out[f"c{i}_fov"] = np.float32(fov)
        out[f"c{i}_setpos"] = np.asarray(pos, np.float32)
        out[f"c{i}_lookat"] = np.asarray(at if at is not None else (np.nan,) * 3, np.float32)
        out[f"c{i}_setrot"] = np.asarray(rot if rot is not None else (np.nan,) * 3, np.float32)
        for k in ("position", "rotation", "mul", "xsub", "ysub", "sinphi", "cosphi", "k", "fov"):
            if k in st:
                out[f"c{i}_{k}"] = np.asarray(st[k], np.float32)
        out[f"c{i}_pixels"] = px
        out[f"c{i}_rays"] = rays
    out["ncams"] = np.int32(len(recs))
    np.savez_compressed(os.path.join(OUT, "cameras.npz"), **out)
    print("cameras:", len(recs))


def vectops_case():
    """The vector helpers of vect-ops.c (exported by the reference's camera
    plugins) on random and special inputs: quaternion products, rotations of
    vectors and of quaternions' vector parts, normalisation."""
    lib = C.CDLL(os.path.join(REF, "libsimplecam_ref.so"))
    for name in ("vox_quat_mul", "vox_rotate_vector", "vox_rotate_vector_q"):
        getattr(lib, name).argtypes = [vp, vp, vp]
    for name in ("vox_quat_normalize", "vox_dot_normalize", "vox_quat_set_identity"):
        getattr(lib, name).argtypes = [vp]
    rng = np.random.default_rng(90)
    n = 2000
    q1 = rng.normal(0, 1, (n, 4)).astype(np.float32)
    q2 = rng.normal(0, 3, (n, 4)).astype(np.float32)
    v = rng.uniform(-500, 500, (n, 3)).astype(np.float32)
    special = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1], [0, 0, 0, 0],
                        [0.5, 0.5, 0.5, 0.5], [-0.0, 0, 0, 0], [4, 1, 2, 3], [2, 0, 2, 0]], np.float32)
    q1[:len(special)] = special
    q2[:len(special)] = special[::-1]
    with np.errstate(invalid="ignore"):        # the zero quaternion
        unit = np.nan_to_num(q1 / np.linalg.norm(q1, axis=1, keepdims=True)).astype(np.float32)
    prod = np.zeros_like(q1); rot = np.zeros_like(v); rotq = np.full_like(q1, 7.0)
    qn = q1.copy(); dn = v.copy()
    for i in range(n):
        lib.vox_quat_mul(P(q1[i]), P(q2[i]), P(prod[i]))
        lib.vox_rotate_vector(P(unit[i]), P(v[i]), P(rot[i]))
        lib.vox_rotate_vector_q(P(unit[i]), P(q2[i]), P(rotq[i]))
        lib.vox_quat_normalize(P(qn[i]))
        lib.vox_dot_normalize(P(dn[i]))
    ident = np.full(4, 9.0, np.float32)
    lib.vox_quat_set_identity(P(ident))
    np.savez_compressed(os.path.join(OUT, "vectops.npz"), q1=q1, q2=q2, unit=unit, v=v, prod=prod, rot=rot,
                        rotq=rotq, qn=qn, dn=dn, identity=ident)
    print("vectops:", n)


def capture_stdout(fn):
    """What fn() prints through the C library's stdout."""
    import tempfile
    libc = C.CDLL(None)
    libc.fflush.argtypes = [vp]
    sys.stdout.flush()
    libc.fflush(None)
    saved = os.dup(1)
    with tempfile.TemporaryFile() as f:
        os.dup2(f.fileno(), 1)
        try:
            fn()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        f.seek(0)
        return f.read().decode()


def geom_case():
    """geom.c's exported metrics and subspace index on random and special
    inputs, and tree.c's vox_dump_tree text of a small tree (pointers other
    than NULL masked)."""
    import re
    for name in ("vox_abs_metric", "vox_sqr_metric"):
        getattr(ref, name).argtypes = [vp, vp]
        getattr(ref, name).restype = C.c_float
    ref.vox_sqr_norm.argtypes = [vp]; ref.vox_sqr_norm.restype = C.c_float
    ref.get_subspace_idx.argtypes = [vp, vp]; ref.get_subspace_idx.restype = C.c_int
    ref.vox_dump_tree.argtypes = [vp]
    rng = np.random.default_rng(95)
    n = 3000
    a = rng.uniform(-1e3, 1e3, (n, 3)).astype(np.float32)
    b = rng.uniform(-1e3, 1e3, (n, 3)).astype(np.float32)
    b[:n // 4] = a[:n // 4] + rng.integers(-2, 3, (n // 4, 3)).astype(np.float32)   # ties and near ties
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40, -1e-40, 3e38, -3e38], np.float32)
    k = len(special)
    a[n // 4:n // 4 + k * k, 0] = np.repeat(special, k)
    b[n // 4:n // 4 + k * k, 0] = np.tile(special, k)
    absm = np.array([ref.vox_abs_metric(P(a[i]), P(b[i])) for i in range(n)], np.float32)
    sqrm = np.array([ref.vox_sqr_metric(P(a[i]), P(b[i])) for i in range(n)], np.float32)
    norm = np.array([ref.vox_sqr_norm(P(a[i])) for i in range(n)], np.float32)
    sub = np.array([ref.get_subspace_idx(P(a[i]), P(b[i])) for i in range(n)], np.int32)
    set_voxel((1.0, 1.0, 1.0))
    cube = np.mgrid[0:8, 0:8, 0:8].reshape(3, -1).T.astype(np.float32)
    holes = np.concatenate([cube[(cube.sum(1) % 5) != 0], np.tile([[20, 3, 3]], (9, 1))]).astype(np.float32)
    t = ref_tree_from_voxels(holes)
    text = capture_stdout(lambda: ref.vox_dump_tree(t))
    ref.vox_destroy_tree(t)
    text = re.sub(r"0x[0-9a-f]+", "PTR", text)
    np.savez_compressed(os.path.join(OUT, "geom.npz"), a=a, b=b, abs_metric=absm, sqr_metric=sqrm, sqr_norm=norm,
                        subspace=sub, dump_voxels=holes, dump_text=np.array(text))
    print("geom:", n, "dump lines:", text.count("\n"))


def render_case():
    """Config-1 workload (64^3 blobs, 256x256, camera at (160,-96,112) looking at
    (32,32,32)): per-pixel rays from the reference simple camera, hits from the
    reference search."""
    set_voxel((1.0, 1.0, 1.0))
    mask = wl.blobs_volume(64, 20, 1, 0.20)
    vox = wl.voxels_from_mask(mask)
    tree = ref_tree_from_voxels(vox)
    pmap, pre = preorder_map(tree)
    cam = RefCamera(0)
    w = h = 256
    cam.set_ws(cam.obj, w, h)
    cam.dot("position", (160, -96, 112))
    cam.look_at(cam.obj, P(np.asarray((32, 32, 32), np.float32)))
    st = cam.state()
    ys, xs = np.mgrid[0:h, 0:w]
    dirs = np.stack([cam.ray(int(x), int(y)) for x, y in zip(xs.ravel(), ys.ravel())]).astype(np.float32)
    orig = np.repeat(st["position"][None, :], w * h, 0).astype(np.float32)
    leaf, pts = ref_rays(tree, None, orig, dirs, pmap)
    dump = orc.dump_tree(tree)
    out = {f"tree_{k}": v for k, v in dump.items()}
    out.update(voxels=vox.astype(np.int16), voxel=np.ones(3, np.float32), w=np.int32(w), h=np.int32(h),
               cam_position=st["position"], cam_rotation=st["rotation"],
               cam_mul=np.float32(st["mul"]), cam_xsub=np.float32(st["xsub"]), cam_ysub=np.float32(st["ysub"]),
               pix_dirs=dirs, pix_leaf=leaf, pix_points=pts)
    np.savez_compressed(os.path.join(OUT, "render64.npz"), **out)
    print(f"render64: voxels={len(vox)} nodes={len(pre)} hits={np.mean(leaf != 0xFFFFFFFF):.3f} "
          f"size={os.path.getsize(os.path.join(OUT, 'render64.npz'))}")
    ref.vox_destroy_tree(tree)


def edit_ops(rng, n, lo, hi, voxel, start, p_insert=0.55, p_fraction=0.15):
    """A seeded sequence of (kind, x, y, z): kind 0 insert, 1 delete; deletions
    mostly of voxels present (tracked on the grid), some of random places;
    some coordinates off the grid (the call snaps them)."""
    v = np.asarray(voxel, np.float64)
    present = {tuple(p) for p in np.round(np.asarray(start, np.float64) / v).astype(np.int64)}
    ops = []
    for _ in range(n):
        if rng.random() < p_insert or not present:
            g = rng.integers(lo, hi, 3)
            off = rng.random(3) * 0.9 if rng.random() < p_fraction else np.zeros(3)
            ops.append((0, *((g + off) * v)))
            present.add(tuple(g))
        else:
            if rng.random() < 0.75:
                keys = list(present)
                g = np.asarray(keys[int(rng.integers(len(keys)))])
                present.discard(tuple(g))
            else:
                g = rng.integers(lo, hi, 3)
                present.discard(tuple(g))
            ops.append((1, *(g * v)))
    return np.asarray(ops, np.float64)


def edit_case(name, voxel, start, ops, every=50):
    """Replays `ops` on the reference's tree built from `start` with its
    vox_insert_voxel / vox_delete_voxel; stores the return values and the
    tree's dump every `every` operations and at the end."""
    set_voxel(voxel)
    t = vp(ref_tree_from_voxels(start) if len(start) else None)
    rets = np.zeros(len(ops), np.int32)
    out = dict(voxel=np.asarray(voxel, np.float32), start=np.asarray(start, np.float32).reshape(-1, 3),
               ops=ops.astype(np.float32))
    snaps = []
    for i, (k, x, y, z) in enumerate(ops):
        a = np.asarray([x, y, z], np.float32)
        rets[i] = (ref.vox_insert_voxel if k == 0 else ref.vox_delete_voxel)(C.byref(t), P(a))
        if (i + 1) % every == 0 or i + 1 == len(ops):
            d = orc.dump_tree(t.value) if t.value else None
            snaps.append(i)
            pre = f"s{len(snaps) - 1}_"
            if d is None:
                out[pre + "empty"] = np.ones(1, np.uint8)
            else:
                for key in ("flags", "dots_num", "boxes", "centers", "child_mask", "dots"):
                    out[pre + key] = d[key]
    out["returns"] = rets
    out["snap_after"] = np.asarray(snaps, np.int32)
    path = os.path.join(OUT, f"{name}.npz")
    np.savez_compressed(path, **out)
    print(f"{name}: ops={len(ops)} inserted={int(rets[ops[:, 0] == 0].sum())} "
          f"deleted={int(rets[ops[:, 0] == 1].sum())} size={os.path.getsize(path)}")
    if t.value:
        ref.vox_destroy_tree(t.value)
    set_voxel((1.0, 1.0, 1.0))


def edit_cases():
    """Tree editing (tree.c:425-866) by the reference's own code."""
    # A: a blob volume, random insertions and deletions around it
    rng = np.random.default_rng(80)
    vol = wl.blobs_volume(20, 6, 80, 0.30)
    start = wl.voxels_from_mask(vol)
    edit_case("edit_blobs", (1, 1, 1), start, edit_ops(rng, 700, -3, 23, (1, 1, 1), start))
    # B: dense leaves: a cube and a stripe, edited around their voxels
    rng = np.random.default_rng(81)
    cube = np.mgrid[0:6, 0:6, 0:6].reshape(3, -1).T
    stripe = np.stack([np.arange(10, 19), np.full(9, 2), np.full(9, 3)], 1)
    start = np.concatenate([cube, stripe]).astype(np.float32)
    ops = []
    present = [tuple(p) for p in start.astype(np.int64)]
    for _ in range(500):
        if rng.random() < 0.6 and present:
            ops.append((1, *present.pop(int(rng.integers(len(present))))))
        else:
            g = tuple(int(x) for x in rng.integers(-1, 20, 3)) if rng.random() < 0.3 else \
                tuple(int(x) for x in rng.integers(0, 7, 3))
            ops.append((0, *g))
            present.append(g)
    edit_case("edit_dense", (1, 1, 1), start, np.asarray(ops, np.float64), every=25)
    # C: from an empty tree: insert 300 voxels, then delete them all
    rng = np.random.default_rng(82)
    pts = np.unique(rng.integers(0, 12, (300, 3)), axis=0)
    rng.shuffle(pts)
    order = rng.permutation(len(pts))
    ops = [(0, *p) for p in pts] + [(1, *pts[i]) for i in order]
    edit_case("edit_empty", (1, 1, 1), np.zeros((0, 3), np.float32), np.asarray(ops, np.float64))
    # D: non-unit voxels
    rng = np.random.default_rng(83)
    v = (0.5, 1.0, 2.0)
    g = np.mgrid[0:10, 0:10, 0:10].reshape(3, -1).T
    sel = g[((g - 5) ** 2).sum(1) < 20]
    start = (sel * np.asarray(v)).astype(np.float32)
    edit_case("edit_voxsize", v, start, edit_ops(rng, 500, -2, 12, v, start))


# ---------------------------------------------------------------- SSE layout

class Node16(C.Structure):
    """struct vox_node of a voxvision built with SSE_INTRIN (tree.h:28-38 with
    the 16-byte aligned float[4] vox_dot of voxvision.h.in:45-57): box 32
    bytes, flags and dots_num, 8 bytes of padding, the union at byte 48
    (a dots pointer, or the centre and 8 children): 128 bytes."""
    _fields_ = [("bmin", C.c_float * 4), ("bmax", C.c_float * 4), ("flags", C.c_uint), ("dots_num", C.c_uint),
                ("pad", C.c_uint * 2), ("u", C.c_float * 4), ("children", vp * 8)]


assert C.sizeof(Node16) == 128


def f4(a):
    """(n, 3) floats as (n, 4) rows of a 16-byte aligned array (vox_dot of the SSE build)."""
    a = np.asarray(a, np.float32).reshape(-1, 3)
    buf = np.zeros(a.shape[0] * 4 + 4, np.float32)
    off = (-buf.ctypes.data % 16) // 4
    out = buf[off: off + a.shape[0] * 4].reshape(-1, 4)
    out[:, :3] = a
    assert out.ctypes.data % 16 == 0
    return out


def dump16(root):
    """Pre-order dump (the oracle's dump fields) of an SSE-layout tree, and
    the node pointers in that order."""
    flags, dnum, boxes, centers, mask, doff, dots, ptrs = [], [], [], [], [], [], [], []
    stack = [root] if root else []
    nd = 0
    while stack:
        p = stack.pop()
        n = Node16.from_address(p)
        ptrs.append(p)
        flags.append(n.flags); dnum.append(n.dots_num)
        boxes.append(list(n.bmin[:3]) + list(n.bmax[:3]))
        doff.append(nd)
        c, m = [0.0, 0.0, 0.0], 0
        if n.flags & 2:
            pass
        elif n.flags & 1:
            base = C.c_void_p.from_address(p + 48).value
            arr = (C.c_float * (4 * n.dots_num)).from_address(base)
            d = np.frombuffer(arr, np.float32).reshape(-1, 4)[:, :3]
            dots.append(d.copy())
            nd += n.dots_num
        else:
            c = list(n.u[:3])
            for o in range(7, -1, -1):
                if n.children[o]:
                    m |= 1 << o
                    stack.append(n.children[o])
        centers.append(c); mask.append(m)
    d = dict(flags=np.asarray(flags, np.uint32), dots_num=np.asarray(dnum, np.uint32),
             boxes=np.asarray(boxes, np.float32).reshape(-1, 6), centers=np.asarray(centers, np.float32).reshape(-1, 3),
             child_mask=np.asarray(mask, np.uint8), dot_offset=np.asarray(doff, np.uint64),
             dots=np.concatenate(dots).astype(np.float32) if dots else np.zeros((0, 3), np.float32))
    return d, ptrs


def sse_layout_case():
    """Trees built by the reference compiled with SSE_INTRIN on (the 16-byte
    vox_dot and 128-byte struct vox_node of its default x86 build), dumped in
    pre-order with their SSE build's own ray and ball answers: the fixture of
    the SSE-layout upload (tests/test_sse_layout.py).  Needs an x86 host
    (make -C oracle ref-sse)."""
    sse = C.CDLL(os.path.join(REF, "libvoxtrees_ref_sse.so"))
    sse.vox_make_tree.argtypes = [vp, C.c_size_t]; sse.vox_make_tree.restype = vp
    sse.vox_destroy_tree.argtypes = [vp]
    sse.vox_ray_tree_intersection.argtypes = [vp, vp, vp, vp]; sse.vox_ray_tree_intersection.restype = vp
    sse.vox_tree_ball_collidep.argtypes = [vp, vp, C.c_float]; sse.vox_tree_ball_collidep.restype = C.c_int
    sse.vox_set_voxel_size.argtypes = [C.c_float] * 3
    g = np.mgrid[-12:12, -12:12, -12:12].reshape(3, -1).T
    ball = g[(g ** 2).sum(1) < 144].astype(np.float32)
    rng = np.random.default_rng(71)
    cloud = np.unique(rng.integers(0, 48, (3000, 3)), axis=0).astype(np.float32)
    rng.shuffle(cloud)
    dup = np.concatenate([np.tile([[3, 3, 3]], (12, 1)), np.mgrid[0:3, 0:3, 0:2].reshape(3, -1).T,
                          [[9, 1, 4], [9, 2, 4], [10, 2, 4]]]).astype(np.float32)
    v = (0.5, 1.0, 2.0)
    gg = np.mgrid[-8:8, -8:8, -8:8].reshape(3, -1).T
    vv = (gg[((gg ** 2).sum(1) < 64) & ((gg[:, 0] + gg[:, 1]) % 3 != 0)] * np.asarray(v)).astype(np.float32)
    blob = wl.voxels_from_mask(wl.blobs_volume(64, 20, 1, 0.20))
    cases = [("ball", ball, (1.0, 1.0, 1.0)), ("cloud", cloud, (1.0, 1.0, 1.0)), ("overflow", dup, (1.0, 1.0, 1.0)),
             ("voxsize", vv, v), ("blob64", blob, (1.0, 1.0, 1.0))]
    out = {"cases": np.array([c[0] for c in cases])}
    for k, (name, vox, voxel) in enumerate(cases):
        sse.vox_set_voxel_size(*voxel)
        s4 = f4(vox)
        t = sse.vox_make_tree(P(s4), s4.shape[0])
        d, ptrs = dump16(t)
        pmap = {p: i for i, p in enumerate(ptrs)}
        bmin, bmax = d["boxes"][0][:3], d["boxes"][0][3:]
        o, dr = edge_rays(bmin, bmax, 3000, 80 + k, np.asarray(voxel, np.float64))
        leaf = np.full(len(o), 0xFFFFFFFF, np.uint32)
        pts = np.zeros((len(o), 3), np.float32)
        o4, d4, r4 = f4(o), f4(dr), f4(np.zeros((1, 3)))
        for i in range(len(o)):
            r = sse.vox_ray_tree_intersection(t, o4[i].ctypes.data, d4[i].ctypes.data, r4[0].ctypes.data)
            if r:
                leaf[i] = pmap[int(r)]
                pts[i] = r4[0, :3]
        c, rad = edge_balls(bmin, bmax, 1500, 90 + k)
        c4 = f4(c)
        hit = np.array([sse.vox_tree_ball_collidep(t, c4[i].ctypes.data, C.c_float(float(rad[i])))
                        for i in range(len(c))], np.uint8)
        out.update({f"{name}_voxel": np.asarray(voxel, np.float32), f"{name}_voxels": np.asarray(vox, np.float32),
                    f"{name}_ray_origins": o, f"{name}_ray_dirs": dr, f"{name}_ray_leaf": leaf,
                    f"{name}_ray_points": pts, f"{name}_ball_centres": c, f"{name}_ball_radii": rad,
                    f"{name}_ball_hit": hit})
        out.update({f"{name}_tree_{key}": val for key, val in d.items()})
        print(f"sse {name}: nodes={len(ptrs)} rays hit={np.mean(leaf != 0xFFFFFFFF):.3f}")
        sse.vox_destroy_tree(t)
    sse.vox_set_voxel_size(1.0, 1.0, 1.0)
    path = os.path.join(OUT, "sse_layout.npz")
    np.savez_compressed(path, **out)
    print(f"sse_layout: {os.path.getsize(path)} B")


# ---------------------------------------------------------------- lights

from tests.helpers import mtree_walk  # noqa: E402


def light_ops(seed, n, kind):
    """A random call sequence for a light manager: insertions (valid and
    invalid colours, radii <= 0, duplicates of live lights), removals (of
    live lights and of missing ones) and ambient changes."""
    rng = np.random.default_rng(seed)
    ops, live = [], []
    for _ in range(n):
        u = rng.random()
        if u < 0.62:
            if kind == "overlap":          # tests.c:856-882: many large overlapping spheres
                c = np.floor(rng.uniform(0, 100, 3)); r = float(70 + np.floor(rng.uniform(0, 30)))
            elif kind == "float":
                c = rng.uniform(-40, 40, 3); r = float(rng.uniform(-1, 25))
            else:
                c = np.floor(rng.uniform(0, 64, 3)); r = float(np.floor(rng.uniform(-2, 20)))
            col = rng.uniform(-0.05, 1.05, 3)
            if live and rng.random() < 0.08:
                c, r = live[int(rng.integers(len(live)))]
            ops.append(("insert", np.asarray(c, np.float32), np.float32(r), np.asarray(col, np.float32)))
            live.append((np.asarray(c, np.float32), np.float32(r)))
        elif u < 0.96:
            if live and rng.random() < 0.85:
                c, r = live.pop(int(rng.integers(len(live))))
            else:
                c, r = np.floor(rng.uniform(0, 64, 3)).astype(np.float32), np.float32(5)
            ops.append(("delete", c, r, None))
        else:
            ops.append(("ambient", None, None, rng.uniform(-0.05, 1.05, 3).astype(np.float32)))
    return ops


def lights_case():
    """The reference's own light manager and M-tree (lights.c, mtree.c with
    the block-typed search cut out: make -C oracle ref-lights) driven through
    three call sequences; every 20 calls the whole M-tree (pre-order walk,
    float bits), the light count and vox_get_light at sample points (lights.c:
    104-116, the sum the renderer colours a hit with) are recorded."""
    L = C.CDLL(os.path.join(REF, "liblights_ref.so"))
    L.vox_make_light_manager.restype = vp
    L.vox_destroy_light_manager.argtypes = [vp]
    L.vox_insert_shadowless_light.argtypes = [vp, vp, C.c_float, vp]; L.vox_insert_shadowless_light.restype = C.c_int
    L.vox_delete_shadowless_light.argtypes = [vp, vp, C.c_float]; L.vox_delete_shadowless_light.restype = C.c_int
    L.vox_set_ambient_light.argtypes = [vp, vp]; L.vox_set_ambient_light.restype = C.c_int
    L.vox_shadowless_lights_number.argtypes = [vp]; L.vox_shadowless_lights_number.restype = C.c_int
    L.vox_get_light.argtypes = [vp, vp, vp]
    out = {}
    seqs = [("int", 11, 400), ("float", 12, 400), ("overlap", 13, 300)]
    out["sequences"] = np.array([s[0] for s in seqs])
    for kind, seed, n in seqs:
        ops = light_ops(seed, n, kind)
        lm = L.vox_make_light_manager()
        rng = np.random.default_rng(seed + 100)
        codes, args = [], []
        snaps = {"at": [], "count": [], "nodes": [], "node_split": [], "spheres": [], "sphere_split": [],
                 "points": [], "light": []}
        for i, (op, c, r, col) in enumerate(ops):
            if op == "insert":
                rc = L.vox_insert_shadowless_light(lm, P(c), C.c_float(r), P(col))
                codes.append(0); args.append(np.concatenate([c, [r], col]))
            elif op == "delete":
                rc = L.vox_delete_shadowless_light(lm, P(c), C.c_float(r))
                codes.append(1); args.append(np.concatenate([c, [r], [0, 0, 0]]))
            else:
                rc = L.vox_set_ambient_light(lm, P(col))
                codes.append(2); args.append(np.concatenate([[0, 0, 0, 0], col]))
            args[-1] = np.concatenate([args[-1], [rc]]).astype(np.float32)
            if (i + 1) % 20 == 0 or i + 1 == len(ops):
                root = C.c_void_p.from_address(lm + 16).value      # lights.c:11-14: ambient, then the tree
                nodes, spheres = mtree_walk(root)
                live = [a for code, a in zip(codes, args) if code == 0]
                pts = np.asarray([a[:3] for a in live[-24:]] if live else [[0, 0, 0]], np.float32)
                pts = np.concatenate([pts, pts + rng.normal(0, 4, pts.shape), rng.uniform(-40, 100, (40, 3))])
                pts = np.ascontiguousarray(pts.astype(np.float32))
                light = np.zeros_like(pts)
                for k in range(len(pts)):
                    L.vox_get_light(lm, P(pts[k]), P(light[k]))
                snaps["at"].append(i + 1); snaps["count"].append(L.vox_shadowless_lights_number(lm))
                snaps["nodes"].append(nodes); snaps["node_split"].append(len(nodes))
                snaps["spheres"].append(spheres); snaps["sphere_split"].append(len(spheres))
                snaps["points"].append(pts); snaps["light"].append(light)
        L.vox_destroy_light_manager(lm)
        out[f"{kind}_op"] = np.array(codes, np.uint8)
        out[f"{kind}_args"] = np.array(args, np.float32)
        out[f"{kind}_snap_at"] = np.array(snaps["at"], np.int32)
        out[f"{kind}_snap_count"] = np.array(snaps["count"], np.int32)
        out[f"{kind}_nodes"] = np.concatenate(snaps["nodes"]).astype(np.uint32)
        out[f"{kind}_node_split"] = np.array(snaps["node_split"], np.int64)
        out[f"{kind}_spheres"] = np.concatenate(snaps["spheres"]).astype(np.uint32)
        out[f"{kind}_sphere_split"] = np.array(snaps["sphere_split"], np.int64)
        out[f"{kind}_point_split"] = np.array([len(p) for p in snaps["points"]], np.int64)
        out[f"{kind}_points"] = np.concatenate(snaps["points"]).astype(np.float32)
        out[f"{kind}_light"] = np.concatenate(snaps["light"]).astype(np.float32)
        print(f"lights {kind}: {len(ops)} calls, {len(snaps['at'])} snapshots, final count {snaps['count'][-1]}, "
              f"nodes {snaps['node_split'][-1]}")
    path = os.path.join(OUT, "lights.npz")
    np.savez_compressed(path, **out)
    print(f"lights: {os.path.getsize(path)} B")


def main():
    # 1. ball of radius 12 (the reference's own tree fixture, tests.c:214-237, scaled down)
    set_voxel((1.0, 1.0, 1.0))
    g = np.mgrid[-12:12, -12:12, -12:12].reshape(3, -1).T
    ball = g[(g ** 2).sum(1) < 144].astype(np.float32)
    t = ref_tree_from_voxels(ball)
    save_case("ball12", t, (1, 1, 1), ball, seed=10)
    ref.vox_destroy_tree(t)

    # 2. the regression tree of tests.c:600-659, built by insertion
    t = vp(None)
    pts = [(0, 0, 0), (0, 0, -1), (0, 0, -2), (0, 0, 1), (0, 0, 2)]
    pts += [(-i, 0, 0) for i in range(1, 5)] + [(i, 0, 0) for i in range(1, 5)]
    pts += [(0, -i, 0) for i in range(1, 5)] + [(0, i, 0) for i in range(1, 5)]
    for p in pts:
        a = np.asarray(p, np.float32)
        ref.vox_insert_voxel(C.byref(t), P(a))
    pmap, pre = preorder_map(t.value)
    o = np.asarray([[-2, -2, 0]], np.float32); d = np.asarray([[1, 1, -1]], np.float32)
    l, p = ref_rays(t.value, None, o, d, pmap)
    assert l[0] != 0xFFFFFFFF, "regression ray of tests.c:655-658 must hit"
    save_case("g676d50c", t.value, (1, 1, 1), None, nrays=4000, nballs=2000, seed=20,
              extra=dict(regress_origin=o, regress_dir=d, regress_leaf=l, regress_point=p), leaf_roots=200)

    # 3. duplicates -> overflowed leaf (tree.c:281-305); plus a small blob around it
    dup = np.concatenate([np.tile([[3, 3, 3]], (12, 1)), np.mgrid[0:3, 0:3, 0:2].reshape(3, -1).T,
                          [[9, 1, 4], [9, 2, 4], [10, 2, 4]]]).astype(np.float32)
    t = ref_tree_from_voxels(dup)
    save_case("overflow", t, (1, 1, 1), dup, nrays=4000, nballs=2000, seed=30, leaf_roots=200)
    ref.vox_destroy_tree(t)

    # 4. non-unit voxel size
    v = (0.5, 1.0, 2.0)
    set_voxel(v)
    g = np.mgrid[-8:8, -8:8, -8:8].reshape(3, -1).T
    sel = g[((g ** 2).sum(1) < 64) & ((g[:, 0] + g[:, 1]) % 3 != 0)]
    vv = (sel * np.asarray(v)).astype(np.float32)
    t = ref_tree_from_voxels(vv)
    save_case("voxsize", t, v, vv, nrays=6000, nballs=3000, seed=40)
    ref.vox_destroy_tree(t)
    set_voxel((1.0, 1.0, 1.0))

    # 5. a full cube (one dense leaf) and a cube with holes (dense sub-leaves)
    cube = np.mgrid[0:8, 0:8, 0:8].reshape(3, -1).T.astype(np.float32)
    t = ref_tree_from_voxels(cube)
    save_case("dense", t, (1, 1, 1), cube, nrays=3000, nballs=1500, seed=50, leaf_roots=50)
    ref.vox_destroy_tree(t)
    holes = cube[(cube.sum(1) % 5) != 0]
    t = ref_tree_from_voxels(holes)
    save_case("holes", t, (1, 1, 1), holes, nrays=4000, nballs=2000, seed=60)
    ref.vox_destroy_tree(t)

    # 6. random sparse cloud in a 48^3 box
    rng = np.random.default_rng(70)
    cloud = np.unique(rng.integers(0, 48, (3000, 3)), axis=0).astype(np.float32)
    rng.shuffle(cloud)
    t = ref_tree_from_voxels(cloud)
    save_case("cloud48", t, (1, 1, 1), cloud, nrays=8000, nballs=4000, seed=70)
    ref.vox_destroy_tree(t)

    camera_cases()
    render_case()
    vectops_case()
    geom_case()


if __name__ == "__main__":
    parts = {"edits": edit_cases, "vectops": vectops_case, "geom": geom_case, "sse": sse_layout_case,
             "lights": lights_case}
    if sys.argv[1:] and sys.argv[1] not in parts:
        sys.exit(f"unknown fixture set {sys.argv[1]!r}; one of {sorted(parts)} or none for everything")
    if sys.argv[1:]:
        parts[sys.argv[1]]()
    else:
        main()
        edit_cases()
