"""The light manager and its M-tree (host side, no GPU): the oracle's
restatement satisfies the reference's own M-tree tests (tests/tests.c:
779-900: invariants after every insertion and removal, duplicates refused,
search counts equal to brute force), the library's independent restatement
answers every call of a random sequence exactly as the oracle does, and both
are pinned to the reference's own compiled lights.c and mtree.c: the
library's M-tree node for node, the oracle's light sums bit for bit."""
import os

import numpy as np
import pytest

from oracle import oracle as orc
import voxvision_gb300 as vg


def _sphere_stream(seed, n, lo=0.0, hi=100.0, r0=1.0, r1=15.0):
    """Integer centres in [lo, hi), radii r0 + floor(U * r1), colours in [0, 1]:
    the shape of the reference's test_mtree data."""
    rng = np.random.default_rng(seed)
    for _ in range(n):
        yield (np.floor(rng.uniform(lo, hi, 3)).astype(np.float32), float(r0 + np.floor(rng.uniform(0, r1))),
               rng.uniform(0, 1, 3).astype(np.float32))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_oracle_mtree_keeps_the_reference_invariants(seed):
    L = orc.OracleLights()
    spheres = list(_sphere_stream(seed, 140))
    added = []
    for c, r, col in spheres:
        ok = L.insert(c, r, col)
        assert ok == all(not (np.array_equal(c, c2) and r == r2) for c2, r2 in added)
        if ok:
            added.append((c, r))
        assert L.verify() == 0
        assert L.count() == len(added)
    c, r, col = spheres[-1]
    assert not L.insert(c, r, col)                     # already in the tree
    for i, (c, r) in enumerate(added):
        assert L.delete(c, r)
        assert not L.delete(c, r)
        assert L.verify() == 0
        assert L.count() == len(added) - i - 1


def test_oracle_search_counts_match_brute_force():
    """tests/tests.c:856-882: 500 spheres of radius 70..100 around [0, 100)^3;
    the spheres found at the origin are exactly those containing it."""
    L = orc.OracleLights()
    rng = np.random.default_rng(4)
    count = 0
    for _ in range(500):
        c = np.floor(rng.uniform(0, 100, 3)).astype(np.float32)
        r = float(70 + np.floor(rng.uniform(0, 30)))
        if L.insert(c, r, (0.5, 0.5, 0.5)) and np.sqrt(np.float32((c.astype(np.float32) ** 2).sum())) < r:
            count += 1
    assert L.verify() == 0
    _, found = L.light((0, 0, 0))
    assert found == count


def test_library_answers_like_the_oracle():
    """Insertions (some invalid: colour outside [0, 1], radius <= 0,
    duplicates), removals (some of missing lights), ambient changes: the
    library's return values and light counts equal the oracle's."""
    rng = np.random.default_rng(9)
    L, M = orc.OracleLights(), vg.LightManager()
    live = []
    for step in range(1500):
        op = rng.random()
        if op < 0.6:
            c = np.floor(rng.uniform(0, 64, 3)).astype(np.float32)
            r = float(np.floor(rng.uniform(-2, 20)))
            col = rng.uniform(-0.1, 1.1, 3).astype(np.float32)
            if live and rng.random() < 0.1:
                c, r = live[int(rng.integers(len(live)))]
            a, b = L.insert(c, r, col), M.insert(c, r, col)
            assert a == b, step
            if a:
                live.append((c, r))
        elif op < 0.95:
            if live and rng.random() < 0.8:
                c, r = live.pop(int(rng.integers(len(live))))
            else:
                c, r = np.floor(rng.uniform(0, 64, 3)).astype(np.float32), float(rng.integers(1, 20))
            assert L.delete(c, r) == M.delete(c, r), step
        else:
            col = rng.uniform(-0.2, 1.2, 3).astype(np.float32)
            assert L.ambient(col) == M.ambient(col)
        assert L.count() == M.count() == len(live)
        assert L.verify() == 0
    M.clear()
    assert M.count() == 0


# ---- pinned to the reference's own light manager and M-tree ---------------
#
# tests/golden/lights.npz: three call sequences run through the reference's
# lights.c and mtree.c compiled here (make -C oracle ref-lights), with the
# whole M-tree, the light count and vox_get_light at sample points recorded
# every 20 calls (make_golden.py lights).

LG = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "lights.npz"))
SEQUENCES = [str(s) for s in LG["sequences"]]


def _replay(kind, manager, at_snapshot):
    ops, args = LG[f"{kind}_op"], LG[f"{kind}_args"]
    snaps = list(LG[f"{kind}_snap_at"])
    k = 0
    for i, (op, a) in enumerate(zip(ops, args)):
        if op == 0:
            rc = manager.insert(a[:3], a[3], a[4:7])
        elif op == 1:
            rc = manager.delete(a[:3], a[3])
        else:
            rc = manager.ambient(a[4:7])
        assert int(rc) == int(a[7]), (kind, i, int(op))
        if k < len(snaps) and i + 1 == snaps[k]:
            at_snapshot(k)
            k += 1
    assert k == len(snaps)


def _split(kind, name, k):
    cut = np.concatenate([[0], np.cumsum(LG[f"{kind}_{name}_split"])])
    return LG[f"{kind}_{name}s" if name != "point" else f"{kind}_points"][cut[k]:cut[k + 1]]


@pytest.mark.parametrize("kind", SEQUENCES)
def test_library_mtree_is_the_references(kind):
    """The library's light manager returns what the reference's does for
    every call, and its M-tree is the reference's node for node -- shape,
    order, bounding spheres and stored spheres to the bit -- after every 20
    calls (insertions with splits, removals with merges, refusals)."""
    import ctypes as C
    from tests.helpers import mtree_walk
    M = vg.LightManager()

    def check(k):
        nodes, spheres = mtree_walk(C.c_void_p.from_address(M.ptr + 16).value)
        assert np.array_equal(nodes, _split(kind, "node", k)), (kind, k)
        assert np.array_equal(spheres, _split(kind, "sphere", k)), (kind, k)
        assert M.count() == LG[f"{kind}_snap_count"][k]

    _replay(kind, M, check)
    M.close()


@pytest.mark.parametrize("kind", SEQUENCES)
def test_oracle_light_sums_are_the_references(kind):
    """The oracle's light at every sample point -- ambient plus each
    containing sphere's share, summed in M-tree order -- has the bits of the
    reference's vox_get_light (lights.c:104-116) after every 20 calls."""
    L = orc.OracleLights()
    cut = np.concatenate([[0], np.cumsum(LG[f"{kind}_point_split"])])

    def check(k):
        pts = LG[f"{kind}_points"][cut[k]:cut[k + 1]]
        ref = LG[f"{kind}_light"][cut[k]:cut[k + 1]]
        got = np.array([L.light(p)[0] for p in pts], np.float32)
        assert np.array_equal(got.view(np.uint32), ref.view(np.uint32)), (kind, k)
        assert L.count() == LG[f"{kind}_snap_count"][k]

    _replay(kind, L, check)
