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


def sse_tree_from_dump(d):
    """A tree in the SSE layout of the reference (16-byte aligned float[4]
    vox_dot, 128-byte struct vox_node: box at 0, flags and dots_num at 32, the
    union at 48 -- a dots pointer, or the centre and 8 children) built in
    memory from a pre-order dump.  Returns the root's address (0 for the
    empty tree) and the buffers that hold the nodes and voxels."""
    import ctypes as C
    n = len(d["flags"])
    if n == 0:
        return 0, None

    def aligned(nbytes):
        raw = np.zeros(nbytes + 16, np.uint8)
        off = (-raw.ctypes.data) % 16
        return raw, raw.ctypes.data + off

    nodes_raw, base = aligned(128 * n)
    nd = len(d["dots"])
    dots_raw, dbase = aligned(16 * max(nd, 1))
    dots4 = np.frombuffer((C.c_float * (4 * max(nd, 1))).from_address(dbase), np.float32).reshape(-1, 4)
    dots4[:nd, :3] = d["dots"]
    addr = [base + 128 * i for i in range(n)]
    # children from the pre-order numbering: node i, then the subtrees of its
    # children in octant order
    size = np.ones(n, np.int64)
    kids = [[] for _ in range(n)]
    stack = []
    for i in range(n - 1, -1, -1):
        m = int(d["child_mask"][i])
        if not (int(d["flags"][i]) & 3) and m:
            k = bin(m).count("1")
            for _ in range(k):
                c = stack.pop()
                kids[i].append(c)
                size[i] += size[c]
        stack.append(i)
    for i in range(n):
        p = addr[i]
        box = np.frombuffer((C.c_float * 8).from_address(p), np.float32)
        box[:3] = d["boxes"][i][:3]
        box[4:7] = d["boxes"][i][3:]
        C.c_uint.from_address(p + 32).value = int(d["flags"][i])
        C.c_uint.from_address(p + 36).value = int(d["dots_num"][i])
        f = int(d["flags"][i])
        if f & 2:
            continue
        if f & 1:
            C.c_void_p.from_address(p + 48).value = dbase + 16 * int(d["dot_offset"][i])
            continue
        ctr = np.frombuffer((C.c_float * 4).from_address(p + 48), np.float32)
        ctr[:3] = d["centers"][i]
        m = int(d["child_mask"][i])
        ks = iter(kids[i])
        for o in range(8):
            C.c_void_p.from_address(p + 64 + 8 * o).value = addr[next(ks)] if (m >> o) & 1 else None
    return addr[0], (nodes_raw, dots_raw)


def mtree_walk(root):
    """An M-tree (struct vox_mtree_node, mtree.h:46-56: bounding sphere,
    parent, leaf flag, count, then 10 child pointers or a spheres pointer;
    128 bytes) in pre-order -- node, then its children in order: per node
    its leaf flag, item count, parent's pre-order index (0xFFFFFFFF for the
    root) and bounding sphere (centre, colour, radius, squared radius as
    float bits); the leaves' spheres in order, as float bits.  The
    reference's and the library's trees share this layout."""
    import ctypes as C

    class Sphere(C.Structure):         # mtree.h:17-40
        _fields_ = [("center", C.c_float * 3), ("color", C.c_float * 3), ("radius", C.c_float),
                    ("sqr_radius", C.c_float)]

    class MNode(C.Structure):
        _fields_ = [("bs", Sphere), ("parent", C.c_void_p), ("leaf", C.c_uint), ("num", C.c_uint),
                    ("data", C.c_void_p * 10)]

    assert C.sizeof(MNode) == 128

    def bits(sp):
        return np.array(list(sp.center) + list(sp.color) + [sp.radius, sp.sqr_radius], np.float32).view(np.uint32)

    nodes, spheres = [], []
    stack = [(root, -1)] if root else []
    while stack:
        p, parent = stack.pop()
        n = MNode.from_address(p)
        k = len(nodes)
        nodes.append(np.concatenate([[n.leaf, n.num, parent & 0xFFFFFFFF], bits(n.bs)]).astype(np.uint32))
        if n.leaf:
            base = n.data[0]
            for i in range(n.num):
                spheres.append(bits(Sphere.from_address(base + i * C.sizeof(Sphere))))
        else:
            for i in range(n.num - 1, -1, -1):
                stack.append((n.data[i], k))
    return np.array(nodes, np.uint32).reshape(-1, 11), np.array(spheres, np.uint32).reshape(-1, 8)
