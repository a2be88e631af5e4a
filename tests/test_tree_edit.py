"""Tree editing on the host (vox_insert_voxel, vox_delete_voxel): replayed
sequences of insertions and deletions give the reference's return values and,
at every checkpoint, the reference's tree node for node (flags, counts,
boxes, centres, children, voxels) -- golden fixtures recorded from the
reference's own compiled tree.c (tests/golden/make_golden.py edits).  No GPU."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from tests.helpers import load
import voxvision_gb300 as vg

CASES = ["edit_blobs", "edit_dense", "edit_empty", "edit_voxsize"]
KEYS = ("flags", "dots_num", "boxes", "centers", "child_mask", "dots")


@pytest.mark.parametrize("case", CASES)
def test_edits_match_the_reference(case):
    g = load(case)
    L = vg.lib()
    v = tuple(float(x) for x in g["voxel"])
    vg.set_voxel_size(v)
    orc.set_voxel(v)
    try:
        start = np.ascontiguousarray(g["start"], np.float32).copy()
        root = C.c_void_p(L.vox_make_tree(start.ctypes.data_as(C.c_void_p), start.shape[0]) if len(start) else None)
        snaps = list(g["snap_after"])
        k = 0
        for i, (kind, x, y, z) in enumerate(g["ops"]):
            a = np.asarray([x, y, z], np.float32)
            fn = L.vox_insert_voxel if kind == 0 else L.vox_delete_voxel
            rc = fn(C.byref(root), a.ctypes.data_as(C.c_void_p))
            assert rc == g["returns"][i], f"op {i}: returned {rc}, the reference {g['returns'][i]}"
            if k < len(snaps) and i == snaps[k]:
                pre = f"s{k}_"
                if pre + "empty" in g:
                    assert root.value is None, f"op {i}: the reference's tree is empty"
                else:
                    d = orc.dump_tree(root.value)
                    for key in KEYS:
                        assert np.array_equal(d[key], g[pre + key]), f"op {i}: {key} differs"
                k += 1
        assert k == len(snaps)
        if root.value:
            L.vox_destroy_tree(root)
    finally:
        vg.set_voxel_size((1, 1, 1))
        orc.set_voxel((1, 1, 1))


def test_edit_helpers():
    """Coordinates are snapped to the grid; the _coord forms; rebuilding."""
    L = vg.lib()
    vg.set_voxel_size((1, 1, 1))
    root = C.c_void_p(None)
    assert L.vox_insert_voxel_coord(C.byref(root), 2.7, 3.2, -0.5) == 1
    assert L.vox_insert_voxel_coord(C.byref(root), 2.0, 3.0, -1.0) == 0          # the same voxel
    p = np.asarray([2.9, 3.9, -0.1], np.float32)
    assert L.vox_delete_voxel(C.byref(root), p.ctypes.data_as(C.c_void_p)) == 1
    assert p.tolist() == [2.0, 3.0, -1.0]                                         # snapped in place
    assert root.value is None
    for x in range(12):
        for y in range(3):
            L.vox_insert_voxel_coord(C.byref(root), float(x), float(y), float((x * y) % 4))
    assert L.vox_voxels_in_tree(root) == 36
    rebuilt = L.vox_rebuild_tree(root)
    assert L.vox_voxels_in_tree(rebuilt) == 36
    pts = np.zeros((36, 3), np.float32)
    k = 0
    for x in range(12):
        for y in range(3):
            pts[k] = (x, y, (x * y) % 4)
            k += 1
    fresh = L.vox_make_tree(pts.ctypes.data_as(C.c_void_p), 36)
    a, b = orc.dump_tree(rebuilt), orc.dump_tree(fresh)
    assert a["flags"].shape == b["flags"].shape
    L.vox_destroy_tree(C.c_void_p(fresh))
    L.vox_destroy_tree(C.c_void_p(rebuilt))
    L.vox_destroy_tree(root)
