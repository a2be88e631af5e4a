"""The light manager and its M-tree (host side, no GPU): the oracle's
restatement satisfies the reference's own M-tree tests (tests/tests.c:
779-900: invariants after every insertion and removal, duplicates refused,
search counts equal to brute force), and the library's independent
restatement answers every call of a random sequence exactly as the oracle
does."""
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
