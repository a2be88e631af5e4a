"""Shared helpers for the parity tests."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TREE_CASES = ["ball12", "g676d50c", "overflow", "voxsize", "dense", "holes", "cloud48"]
MISS = 0xFFFFFFFF


def load(name):
    return dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))


def tree_dump(g):
    return {k[5:]: v for k, v in g.items() if k.startswith("tree_")}


def same_points(a, b, hit):
    """Bit-exact float compare on hit rows, with every NaN counted equal
    (NaN payloads differ between x86, aarch64 and the GPU)."""
    a = np.asarray(a, np.float32)[hit]
    b = np.asarray(b, np.float32)[hit]
    both_nan = np.isnan(a) & np.isnan(b)
    eq = (a.view(np.uint32) == b.view(np.uint32)) | both_nan
    return bool(eq.all()), int((~eq.all(axis=1)).sum()) if a.ndim == 2 else int((~eq).sum())


def close_points(a, b, hit, rel=1e-5):
    a = np.asarray(a, np.float64)[hit]
    b = np.asarray(b, np.float64)[hit]
    both_nan = np.isnan(a) & np.isnan(b)
    ok = both_nan | (np.abs(a - b) <= rel * np.maximum(1.0, np.abs(b)))
    return bool(ok.all())


def dumps_equal(d1, d2):
    for k in ("flags", "dots_num", "child_mask", "dot_offset"):
        if not np.array_equal(d1[k], d2[k]):
            return False, k
    for k in ("boxes", "centers", "dots"):
        if not np.array_equal(np.asarray(d1[k], np.float32).view(np.uint32),
                              np.asarray(d2[k], np.float32).view(np.uint32)):
            return False, k
    return True, None


def image_dump(units, rec_of_id, voxel):
    """The device image of a tree (pool_layout.h) decoded into the pre-order
    dump format of the oracle (flags with the overflow bit for leaves of more
    than VOX_MAX_DOTS voxels, dots_num, boxes, centers, child_mask, dot_offset,
    dots): device-built trees compare directly with the reference's dumps."""
    n = len(rec_of_id)
    recs = rec_of_id.astype(np.int64)
    r0, r1, r2 = units[recs], units[recs + 1], units[recs + 2]
    boxes = np.concatenate([r0, r1[:, :2]], axis=1).astype(np.uint32).view(np.float32)
    meta, link = r1[:, 2], r1[:, 3]
    kind = meta & 3
    flags = np.zeros(n, np.uint32)
    dots_num = np.zeros(n, np.uint64)
    centers = np.zeros((n, 3), np.float32)
    mask = np.zeros(n, np.uint8)
    doff = np.zeros(n, np.uint64)
    dots = []
    nd = 0
    id_of_rec = {int(r): i for i, r in enumerate(recs)}
    children = {}
    v = np.asarray(voxel, np.float64)
    for i in range(n):
        doff[i] = nd
        if kind[i] == 2:
            flags[i] = 2
            ext = (boxes[i, 3:].astype(np.float64) - boxes[i, :3]) / v
            dots_num[i] = int(np.prod(np.rint(ext)))
        elif kind[i] == 1:
            cnt = int(meta[i] >> 2)
            flags[i] = 1 | (4 if cnt > 7 else 0)
            dots_num[i] = cnt
            dots.append(units[link[i]:link[i] + cnt, :3])
            nd += cnt
        else:
            m = int((meta[i] >> 8) & 0xFF)
            mask[i] = m
            centers[i] = r2[i, :3].astype(np.uint32).view(np.float32)
            children[i] = [id_of_rec[int(link[i]) + 3 * j] for j in range(bin(m).count("1"))]
    for i in range(n - 1, -1, -1):
        if i in children:
            dots_num[i] = sum(int(dots_num[c]) for c in children[i])
    d = np.concatenate(dots).astype(np.uint32).view(np.float32) if dots else np.zeros((0, 3), np.float32)
    return dict(flags=flags, dots_num=dots_num.astype(np.uint32), boxes=boxes, centers=centers,
                child_mask=mask, dot_offset=doff, dots=d)
