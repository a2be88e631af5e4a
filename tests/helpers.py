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
