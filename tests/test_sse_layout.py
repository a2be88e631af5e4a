"""Trees of the SSE vox_dot layout at the upload boundary (no GPU needed).

A voxvision built with SSE_INTRIN -- its default on x86 -- has a 16-byte
vox_dot and a 128-byte struct vox_node (voxvision.h.in:45-57,
tree.h:22-38).  tests/golden/sse_layout.npz holds trees built by the
reference compiled that way (make -C oracle ref-sse; make_golden.py sse),
dumped in pre-order with that build's own ray and ball answers.  Here each
tree is rebuilt in memory in the SSE layout and flattened by the library's
SSE reading; the image must equal the scalar layout's image of the same
voxels built by the library's vox_make_tree, byte for byte.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import MISS, dumps_equal, load, same_points, sse_tree_from_dump
from voxvision_gb300 import HostTree, lib, set_voxel_size

G = load("sse_layout")
CASES = [str(c) for c in G["cases"]]
LAYOUT_SCALAR, LAYOUT_SSE = 0, 1


def _case(name):
    pre = f"{name}_"
    d = {k[len(pre):]: v for k, v in G.items() if k.startswith(pre)}
    tree = {k[5:]: v for k, v in d.items() if k.startswith("tree_")}
    return d, tree


def _image(root, layout, voxel):
    L = lib()
    nu, ni = C.c_size_t(), C.c_size_t()
    v = np.ascontiguousarray(voxel, np.float32)
    vp = v.ctypes.data_as(C.c_void_p)
    assert L.vox_cuda_tree_flatten_host_layout(root, layout, vp, None, 0, None, 0, C.byref(nu), C.byref(ni)) == 0
    units = np.zeros((max(nu.value, 1), 4), np.uint32)
    ids = np.zeros(max(ni.value, 1), np.uint32)
    assert L.vox_cuda_tree_flatten_host_layout(root, layout, vp, units.ctypes.data_as(C.c_void_p), nu.value,
                                               ids.ctypes.data_as(C.c_void_p), ni.value, None, None) == 0
    return units[:nu.value], ids[:ni.value]


@pytest.mark.parametrize("name", CASES)
def test_sse_built_tree_is_the_scalar_built_tree(name):
    """The SSE build of vox_make_tree (its vector find_center and bounding
    box, tree.c:31-121) makes the tree the scalar build makes, node for node."""
    d, tree = _case(name)
    set_voxel_size(tuple(d["voxel"]))
    try:
        t = HostTree.from_voxels(d["voxels"])
        ok, key = dumps_equal(orc.dump_tree(t.ptr), tree)
    finally:
        set_voxel_size((1, 1, 1))
    assert ok, key


@pytest.mark.parametrize("name", CASES)
def test_sse_layout_image_equals_scalar_layout_image(name):
    d, tree = _case(name)
    root, keep = sse_tree_from_dump(tree)
    a_units, a_ids = _image(C.c_void_p(root), LAYOUT_SSE, d["voxel"])
    set_voxel_size(tuple(d["voxel"]))
    try:
        t = HostTree.from_voxels(d["voxels"])
        b_units, b_ids = _image(C.c_void_p(t.ptr), LAYOUT_SCALAR, d["voxel"])
    finally:
        set_voxel_size((1, 1, 1))
    assert np.array_equal(a_units, b_units) and np.array_equal(a_ids, b_ids)
    assert lib().vox_cuda_image_check(a_units.ctypes.data_as(C.c_void_p), len(a_units), len(a_ids)) == 0
    del keep


@pytest.mark.parametrize("name", CASES)
def test_scalar_arithmetic_answers_the_sse_build(name):
    """The searches the kernels restate (the scalar geom.c) give the SSE
    build's own answers on its trees -- the same leaf, the same point bits,
    the same ball booleans -- for every ray with a non-zero direction
    (random, axis-aligned, one or two zero components, signed zeros).  The
    two builds of the reference differ on one degenerate input only: a ray
    whose direction is all zeros.  The scalar hit_box divides by zero
    (geom.c:79) and reports a hit with a NaN point; the SSE one blends
    those quotients to 0 (geom-sse.c:96-98) and misses.  The library follows
    the scalar build (the only one on aarch64) there."""
    d, tree = _case(name)
    orc.set_voxel(tuple(d["voxel"]))
    try:
        t = orc.OracleTree.from_dump(tree)
        leaf, _, pts, _ = t.rays(d["ray_origins"], d["ray_dirs"], nthreads=2)
        hit, _ = t.balls(d["ball_centres"], d["ball_radii"], nthreads=2)
    finally:
        orc.set_voxel((1, 1, 1))
    zero = (d["ray_dirs"] == 0).all(axis=1)
    assert zero.any()
    ok = ~zero
    assert np.array_equal(leaf[ok], d["ray_leaf"][ok])
    assert same_points(pts[ok], d["ray_points"][ok], leaf[ok] != MISS)[0]
    differ = leaf != d["ray_leaf"]
    assert (d["ray_leaf"][differ] == MISS).all() and np.isnan(pts[differ]).all()
    assert np.array_equal(hit, d["ball_hit"])


def test_unknown_layout_is_refused():
    d, tree = _case(CASES[0])
    root, keep = sse_tree_from_dump(tree)
    nu = C.c_size_t()
    assert lib().vox_cuda_tree_flatten_host_layout(C.c_void_p(root), 7, None, None, 0, None, 0, C.byref(nu),
                                                   None) == -1
