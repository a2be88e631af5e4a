"""geom.h's exported metrics and subspace index, and the debugging dumps of
trees (tree.h:130) and M-trees (mtree.h:98): the metrics bit for bit the
reference's geom.c on 3000 random and special input pairs (signed zeros,
infinities, NaN, subnormals, ties), the tree dump the reference's own text
for the same tree (tests/golden/geom.npz, made by the reference's compiled
code; pointers other than NULL masked).  No GPU is used."""
import ctypes as C
import re

import numpy as np

from tests.helpers import load
from voxvision_gb300 import lib, set_voxel_size


def _L():
    L = lib()
    for name in ("vox_abs_metric", "vox_sqr_metric"):
        getattr(L, name).argtypes = [C.c_void_p, C.c_void_p]
        getattr(L, name).restype = C.c_float
    L.vox_sqr_norm.argtypes = [C.c_void_p]
    L.vox_sqr_norm.restype = C.c_float
    L.get_subspace_idx.argtypes = [C.c_void_p, C.c_void_p]
    L.get_subspace_idx.restype = C.c_int
    L.vox_dump_tree.argtypes = [C.c_void_p]
    L.vox_dump_tree.restype = None
    L.vox_mtree_dump.argtypes = [C.c_void_p]
    L.vox_mtree_dump.restype = None
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _flush():
    libc = C.CDLL(None)
    libc.fflush.argtypes = [C.c_void_p]
    libc.fflush(None)


def test_metrics_match_reference_bit_for_bit():
    L, g = _L(), load("geom")
    a, b = g["a"], g["b"]
    n = a.shape[0]
    got = {"abs_metric": np.array([L.vox_abs_metric(_p(a[i]), _p(b[i])) for i in range(n)], np.float32),
           "sqr_metric": np.array([L.vox_sqr_metric(_p(a[i]), _p(b[i])) for i in range(n)], np.float32),
           "sqr_norm": np.array([L.vox_sqr_norm(_p(a[i])) for i in range(n)], np.float32)}
    for k, v in got.items():
        ref = g[k]
        same = (v.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(v) & np.isnan(ref))
        assert same.all(), (k, int((~same).sum()))
    sub = np.array([L.get_subspace_idx(_p(a[i]), _p(b[i])) for i in range(n)], np.int32)
    assert np.array_equal(sub, g["subspace"])


def test_tree_dump_is_the_reference_text(capfd):
    L, g = _L(), load("geom")
    set_voxel_size((1, 1, 1))
    vox = np.ascontiguousarray(g["dump_voxels"], np.float32).copy()
    t = lib().vox_make_tree(_p(vox), vox.shape[0])
    capfd.readouterr()
    L.vox_dump_tree(t)
    _flush()
    out = capfd.readouterr().out
    lib().vox_destroy_tree(C.c_void_p(t))
    assert re.sub(r"0x[0-9a-f]+", "PTR", out) == str(g["dump_text"])


def test_mtree_dump_lists_every_node_and_sphere(capfd):
    L = _L()

    class Sphere(C.Structure):
        _fields_ = [("center", C.c_float * 3), ("color", C.c_float * 3), ("radius", C.c_float),
                    ("sqr_radius", C.c_float)]

    root = C.c_void_p(None)
    rng = np.random.default_rng(3)
    for _ in range(40):
        s = Sphere()
        s.center[:] = [float(x) for x in rng.uniform(-50, 50, 3)]
        s.color[:] = [1.0, 1.0, 1.0]
        s.radius = float(rng.uniform(1, 10))
        assert lib().vox_mtree_add_sphere(C.byref(root), C.byref(s))
    capfd.readouterr()
    L.vox_mtree_dump(root)
    _flush()
    out = capfd.readouterr().out
    lines = out.splitlines()
    assert lines[0].startswith("Node 0x") and "parent=(nil)" in lines[0]
    spheres = sum(1 for ln in lines if re.fullmatch(r"<[ -]?\d+\.\d{4}, +-?\d+\.\d{4}, +-?\d+\.\d{4}>, +\d+\.\d{4}",
                                                    ln.strip()))
    assert spheres == lib().vox_mtree_items(root) == 40
    assert sum(ln.startswith("Leaf content (") for ln in lines) >= 2
    lib().vox_mtree_destroy(root)
    capfd.readouterr()
    L.vox_mtree_dump(None)
    _flush()
    assert capfd.readouterr().out == "Node (nil) empty node\n"
