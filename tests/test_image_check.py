"""The host check every upload makes before a tree image reaches the GPU
(vox_flatten_validate behind vox_cuda_image_check), on images made on the host
(vox_cuda_tree_flatten_host).  Sound images pass; every planted damage -- a
child block or voxel run past the image's end, an unknown node kind, a leaf
id past the node count, a voxel count that disagrees with the leaf record, a
cycle back to an ancestor, a node count that does not match -- is refused.
The damage is planted in host memory; no GPU is used."""
import ctypes as C

import numpy as np
import pytest

from tests.helpers import load
from voxvision_gb300 import HostTree, lib, set_voxel_size
from voxvision_gb300 import workloads as wl

KIND_INNER, KIND_LEAF, KIND_DENSE = 0, 1, 2


def _image(tree):
    L = lib()
    nu, ni = C.c_size_t(), C.c_size_t()
    assert L.vox_cuda_tree_flatten_host(tree.ptr, None, 0, None, 0, C.byref(nu), C.byref(ni)) == 0
    units = np.zeros((nu.value, 4), np.uint32)
    recs = np.zeros(ni.value, np.uint32)
    assert L.vox_cuda_tree_flatten_host(tree.ptr, units.ctypes.data, nu.value, recs.ctypes.data, ni.value,
                                        C.byref(nu), C.byref(ni)) == 0
    return units, recs


def _check(units, n_nodes):
    u = np.ascontiguousarray(units, np.uint32)
    return lib().vox_cuda_image_check(u.ctypes.data if u.size else None, u.shape[0], n_nodes)


@pytest.fixture(scope="module")
def image():
    set_voxel_size((1, 1, 1))
    t = HostTree.from_voxels(wl.voxels_from_mask(wl.noise_volume(64, 10, 0.10)))
    units, recs = _image(t)
    kinds = units[recs + 1, 2] & 3
    return t, units, recs, kinds


def test_sound_images_pass():
    set_voxel_size((1, 1, 1))
    for case in ("ball12", "overflow", "dense", "holes", "cloud48"):
        g = load(case)
        set_voxel_size(tuple(g["voxel"]))
        t = HostTree.from_voxels(g["voxels"])
        units, recs = _image(t)
        assert _check(units, len(recs)) == 0, case
    set_voxel_size((1, 1, 1))
    assert _check(np.zeros((0, 4), np.uint32), 0) == 0            # the empty tree


def _first(kinds, recs, kind):
    i = int(np.flatnonzero(kinds == kind)[0])
    return int(recs[i])


def test_links_past_the_end_are_refused(image):
    t, units, recs, kinds = image
    n = units.shape[0]
    inner = _first(kinds, recs, KIND_INNER)
    bad = units.copy()
    bad[inner + 1, 3] = n - 1                 # child block would run past the end
    assert _check(bad, len(recs)) != 0
    leaf = _first(kinds, recs, KIND_LEAF)
    bad = units.copy()
    bad[leaf + 1, 3] = n - 1                  # voxel run past the end
    assert _check(bad, len(recs)) != 0
    bad = units.copy()
    bad[leaf + 1, 2] = (bad[leaf + 1, 2] & 3) | (0x3FFFFFFF << 2)   # a huge voxel count
    assert _check(bad, len(recs)) != 0


def test_unknown_kinds_and_ids_are_refused(image):
    t, units, recs, kinds = image
    leaf = _first(kinds, recs, KIND_LEAF)
    bad = units.copy()
    bad[leaf + 1, 2] |= 3                     # kind 3 does not exist
    assert _check(bad, len(recs)) != 0
    bad = units.copy()
    bad[leaf + 2, 0] = len(recs)              # leaf id past the node count
    assert _check(bad, len(recs)) != 0
    bad = units.copy()
    bad[leaf + 2, 1] += 1                     # count in the id record disagrees
    assert _check(bad, len(recs)) != 0
    dense = _first(kinds, recs, KIND_DENSE)
    bad = units.copy()
    bad[dense + 1, 3] = len(recs) + 5         # dense leaf id past the node count
    assert _check(bad, len(recs)) != 0


def test_cycles_and_wrong_counts_are_refused(image):
    t, units, recs, kinds = image
    deep = [int(r) for r, k in zip(recs, kinds) if k == KIND_INNER][-1]   # an inner node near the bottom
    bad = units.copy()
    bad[deep + 1, 3] = 0                      # its child block is the root record: a cycle
    bad[deep + 1, 2] = (bad[deep + 1, 2] & ~np.uint32(0xFF00)) | np.uint32(1 << 8)
    assert _check(bad, len(recs)) != 0
    assert _check(units, len(recs) + 1) != 0  # a node the walk never reaches
    assert _check(units, len(recs) - 1) != 0  # more nodes reached than declared
    assert _check(units[: units.shape[0] - 1], len(recs)) != 0   # image cut short
    assert _check(units, len(recs)) == 0      # the untouched image still passes


def test_random_damage_never_passes_unnoticed(image):
    """Random bits flipped in the meta and link words of random records: any
    image the check accepts must still be walkable in bounds, reaching each
    declared node once (a Python walk of the same rules)."""
    t, units, recs, kinds = image
    rng = np.random.default_rng(5)
    n = units.shape[0]
    refused = 0
    for _ in range(300):
        bad = units.copy()
        for _ in range(int(rng.integers(1, 4))):
            r = int(recs[int(rng.integers(len(recs)))])
            word = int(rng.integers(2, 4))
            bad[r + 1, word] ^= np.uint32(1 << int(rng.integers(32)))
        if _check(bad, len(recs)) != 0:
            refused += 1
            continue
        seen, work = 0, [0]
        while work:
            r = work.pop()
            assert r + 3 <= n
            seen += 1
            assert seen <= len(recs)
            meta, link = int(bad[r + 1, 2]), int(bad[r + 1, 3])
            kind = meta & 3
            assert kind != 3
            if kind == KIND_LEAF:
                assert link + (meta >> 2) <= n
            elif kind == KIND_INNER:
                k = bin((meta >> 8) & 0xFF).count("1")
                assert link + 3 * k <= n
                work.extend(link + 3 * i for i in range(k))
        assert seen == len(recs)
    assert refused > 100
