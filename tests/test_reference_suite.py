"""The reference's own `voxtrees` tree tests (tests/tests.c:214-598), restated
over the library's host trees: construction of the radius-50 ball, the
insertion cases (a repeated voxel refused, a dense-leaf root grown, sparse and
dense 3x3x3 blocks), the deletion cases (dense leaves kept or split), and the
dense-leaf transitions on insertion and deletion -- each followed by the
reference's `check_tree` invariants (tests.c:239-300), restated here over a
pre-order dump of the tree.  No GPU is used."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from voxvision_gb300 import lib, set_voxel_size

LEAF, DENSE, LEAF_MASK = 1, 2, 3
MAX_DOTS = 7   # params.h:29


@pytest.fixture(autouse=True)
def unit_voxel():
    set_voxel_size((1, 1, 1))
    yield
    set_voxel_size((1, 1, 1))


def _dot(*x):
    return np.array(x, np.float32)


class Tree:
    """A tree edited through vox_insert_voxel / vox_delete_voxel (tree.h:88-122)."""

    def __init__(self, ptr=None):
        self.p = C.c_void_p(ptr)

    def insert(self, *x):
        d = _dot(*x)
        return lib().vox_insert_voxel(C.byref(self.p), d.ctypes.data_as(C.c_void_p))

    def delete(self, *x):
        d = _dot(*x)
        return lib().vox_delete_voxel(C.byref(self.p), d.ctypes.data_as(C.c_void_p))

    def count(self):
        return int(lib().vox_voxels_in_tree(self.p)) if self.p.value else 0

    def root_flags(self):
        return int(orc.dump_tree(self.p.value)["flags"][0]) if self.p.value else None

    def destroy(self):
        if self.p.value:
            lib().vox_destroy_tree(self.p)
        self.p = C.c_void_p(None)


def check_tree(ptr, voxel=(1.0, 1.0, 1.0)):
    """tests.c:239-300 on a pre-order dump: dense leaves hold their box's
    volume in voxels; leaf voxels lie in their leaf's box; an inner node's
    children lie in its box, in the octant of their index, and hold all its
    voxels."""
    if ptr:
        check_dump(orc.dump_tree(ptr), voxel)


def check_dump(d, voxel=(1.0, 1.0, 1.0)):
    flags, num, boxes, centers = d["flags"], d["dots_num"], d["boxes"], d["centers"]
    mask, doff, dots = d["child_mask"], d["dot_offset"], d["dots"]
    v = np.asarray(voxel, np.float32)
    half = (v / np.float32(2)).astype(np.float32)

    def between(box, p):
        return bool(np.all(p >= box[:3]) and np.all(p <= box[3:]))

    def subspace(center, p):      # geom.c:44-51
        return sum(int(center[k] > p[k]) << k for k in range(3))

    def walk(i):
        f = int(flags[i])
        if f & DENSE:
            size = (boxes[i, 3:] - boxes[i, :3]).astype(np.float32)
            vol = np.float32(np.float32(size[0] * size[1]) * size[2]) / np.float32(v[0] * v[1] * v[2])
            assert int(num[i]) == int(vol)
            return i + 1
        if f & LEAF:
            for p in dots[int(doff[i]):int(doff[i]) + int(num[i])]:
                assert between(boxes[i], p) and between(boxes[i], (p + v).astype(np.float32))
            return i + 1
        j, total = i + 1, 0
        for o in range(8):
            if (int(mask[i]) >> o) & 1:
                cb = boxes[j]
                assert between(boxes[i], cb[:3]) and between(boxes[i], cb[3:])
                assert subspace(centers[i], (cb[:3] + half).astype(np.float32)) == o
                assert subspace(centers[i], (cb[3:] - half).astype(np.float32)) == o
                total += int(num[j])
                j = walk(j)
        assert total == int(num[i])
        return j

    assert walk(0) == len(flags)


def test_tree_cons():                                                     # tests.c:214-237, 360-365
    g = np.mgrid[-50:50, -50:50, -50:50].reshape(3, -1).T
    ball = np.ascontiguousarray(g[(g ** 2).sum(1) < 2500], np.float32)
    n = ball.shape[0]
    t = lib().vox_make_tree(ball.ctypes.data_as(C.c_void_p), n)
    assert t and int(lib().vox_voxels_in_tree(C.c_void_p(t))) == n
    check_tree(t)
    lib().vox_destroy_tree(C.c_void_p(t))


def test_tree_ins():                                                      # tests.c:367-438
    t = Tree()
    assert t.insert(0, 0, 0) and t.count() == 1
    assert not t.insert(0.5, 0.1, 0.8) and t.count() == 1                 # the same voxel again
    assert t.insert(6, 6, 6) and t.count() == 2
    check_tree(t.p.value)
    t.destroy()

    box = np.array([5, 5, 5, 10, 10, 10], np.float32)                    # a dense leaf as the root
    t = Tree(lib().vox_make_dense_leaf(box.ctypes.data_as(C.c_void_p)))
    assert t.count() == 125 and t.root_flags() & DENSE
    assert not t.insert(6, 6, 6)
    assert t.insert(0, 0, 0) and t.count() == 126
    check_tree(t.p.value)
    t.destroy()

    for step in (2, 1):                                                   # sparse, then dense 3x3x3
        t = Tree()
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    assert t.insert(step * i, step * j, step * k)
        assert t.count() == 27
        check_tree(t.p.value)
        t.destroy()


@pytest.mark.parametrize("axis,start,step,dense_after", [(1, 0, 1, True), (2, MAX_DOTS + 9, -1, True),
                                                         (0, 1, 1, False)])
def test_tree_del_stripes(axis, start, step, dense_after):               # tests.c:441-505 (del1-del3)
    t = Tree()
    d = [0, 0, 0]
    for _ in range(MAX_DOTS + 10):
        t.insert(*d)
        d[axis] += 1
    assert t.root_flags() & DENSE
    d = [0, 0, 0]
    d[axis] = start
    for _ in range(10):
        t.delete(*d)
        d[axis] += step
        if dense_after:
            assert t.root_flags() & DENSE
        else:
            assert not (t.root_flags() & LEAF_MASK)
        check_tree(t.p.value)
    t.destroy()


@pytest.mark.parametrize("hole", [(0, 0, 0), (1, 1, 1)])
def test_tree_del_from_dense_block(hole):                                 # tests.c:507-557 (del4, del5)
    t = Tree()
    for i in range(3):
        for j in range(3):
            for k in range(3):
                t.insert(i, j, k)
    assert t.root_flags() & DENSE
    t.delete(*hole)
    assert not (t.root_flags() & LEAF_MASK)
    check_tree(t.p.value)
    t.destroy()


def test_tree_transitions():                                              # tests.c:559-598
    t = Tree()
    d = [0, 0, 0]
    for _ in range(MAX_DOTS + 4):
        d[0] += 1
        t.insert(*d)
        assert t.root_flags() & DENSE
    t.destroy()

    t = Tree()
    d = [0, 0, 0]
    for _ in range(MAX_DOTS + 4):
        d[0] += 1
        t.insert(*d)
    d = [0, 0, 0]
    for _ in range(MAX_DOTS + 4):
        assert t.root_flags() & DENSE
        d[0] += 1
        t.delete(*d)
    assert not t.p.value                                                  # deleted down to nothing


def test_check_tree_sees_planted_mistakes():
    """The invariants fail on dumps with a mistake planted on the host: a
    child box moved out of its octant, a count that does not add up, a leaf
    voxel outside its leaf."""
    g = np.mgrid[0:12, 0:12, 0:12].reshape(3, -1).T
    vox = np.ascontiguousarray(g[(g.sum(1) % 4) != 0], np.float32)
    t = lib().vox_make_tree(vox.ctypes.data_as(C.c_void_p), vox.shape[0])
    d = orc.dump_tree(t)
    lib().vox_destroy_tree(C.c_void_p(t))
    check_dump(d)
    inner = int(np.flatnonzero((d["flags"] & LEAF_MASK) == 0)[0])
    child = inner + 1
    bad = {k: v.copy() for k, v in d.items()}
    bad["boxes"][child, :3] -= 100.0                      # leaves the parent's box
    with pytest.raises(AssertionError):
        check_dump(bad)
    bad = {k: v.copy() for k, v in d.items()}
    bad["dots_num"][inner] += 1                           # children no longer add up
    with pytest.raises(AssertionError):
        check_dump(bad)
    leaf = int(np.flatnonzero((d["flags"] & LEAF) != 0)[0])
    bad = {k: v.copy() for k, v in d.items()}
    bad["dots"][int(bad["dot_offset"][leaf])] += 50.0     # a voxel outside its leaf
    with pytest.raises(AssertionError):
        check_dump(bad)
