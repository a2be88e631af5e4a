"""Argument and file checks of the raw-volume reader (vox_cuda_read_raw_data,
datareader.c:11-85): they happen on the host before any device work, with the
reference's error strings."""
import ctypes as C

import numpy as np

import voxvision_gb300 as vg
from voxvision_gb300._lib import RawTest

EINVAL, ETOOBIG = -1, -6


def _read(path, dim, ss, test):
    d = (C.c_uint * 3)(*dim)
    h = C.c_void_p()
    err = C.c_char_p()
    rc = vg.lib().vox_cuda_read_raw_data(str(path).encode(), C.byref(d), ss, C.byref(test), C.byref(h), C.byref(err))
    return rc, (err.value.decode() if err.value else None), h


def test_missing_file(tmp_path):
    rc, err, h = _read(tmp_path / "none.raw", (4, 4, 4), 1, RawTest(1, 255, None))
    assert rc == EINVAL and err == "No such file or directory" and not h.value


def test_wrong_size(tmp_path):
    p = tmp_path / "v.raw"
    p.write_bytes(bytes(4 * 4 * 4 * 2))
    rc, err, _ = _read(p, (4, 4, 4), 1, RawTest(1, 255, None))   # datareader.c:40-43
    assert rc == EINVAL and err == "Wrong size of dataset"
    rc, err, _ = _read(p, (4, 4, 5), 2, RawTest(1, 255, None))
    assert rc == EINVAL and err == "Wrong size of dataset"


def test_bad_arguments(tmp_path):
    p = tmp_path / "v.raw"
    p.write_bytes(bytes(8))
    mask = np.zeros(1 << 21, np.uint8)
    assert _read(p, (2, 2, 2), 5, RawTest(0, 1, None))[0] == EINVAL            # samples of 1..4 bytes
    assert _read(p, (2, 2, 2), 3, RawTest(0, 0, mask.ctypes.data))[0] == EINVAL  # tables for 1-2 bytes only
    assert _read(p, (65536, 65536, 2), 1, RawTest(0, 1, None))[0] == ETOOBIG  # 2^33 samples


def test_predicate_table():
    from voxvision_gb300 import _raw_test
    t, mask = _raw_test(1, None, None, test=lambda v: v % 3 == 0)
    bits = np.unpackbits(mask, bitorder="little")
    assert bits.size == 256 and all(bits[v] == (v % 3 == 0) for v in range(256))
    t, mask = _raw_test(2, 10, 20)
    assert mask is None and (t.lo, t.hi) == (10, 20)
