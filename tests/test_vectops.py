"""The vector helpers exported for camera modules (vect-ops.h:13-64): bit for
bit the reference's vect-ops.c on 2000 random and special inputs
(tests/golden/vectops.npz, made by the reference's compiled code), and the
reference's own `vectops` suite (tests/tests.c:79-358: identity, rotation
around its own axis, axis changes, anticommutativity, composition, norm
preservation, the quaternion multiplication table) at its precise_check
tolerance.  No GPU is used."""
import ctypes as C
import math

import numpy as np
import pytest

from tests.helpers import load
from voxvision_gb300 import lib

PRECISE = 1e-5   # tests.c:957-959


@pytest.fixture(scope="module")
def L():
    L = lib()
    for name in ("vox_quat_mul", "vox_rotate_vector", "vox_rotate_vector_q"):
        getattr(L, name).argtypes = [C.c_void_p] * 3
        getattr(L, name).restype = None
    for name in ("vox_quat_normalize", "vox_dot_normalize", "vox_quat_set_identity"):
        getattr(L, name).argtypes = [C.c_void_p]
        getattr(L, name).restype = None
    return L


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _f(*x):
    return np.array(x, np.float32)


def _bits_equal(a, b):
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    same = a.view(np.uint32) == b.view(np.uint32)
    return bool(np.all(same | (np.isnan(a) & np.isnan(b))))


def test_matches_reference_bit_for_bit(L):
    g = load("vectops")
    n = g["q1"].shape[0]
    prod = np.zeros_like(g["q1"]); rot = np.zeros_like(g["v"]); rotq = np.full_like(g["q1"], 7.0)
    qn = g["q1"].copy(); dn = g["v"].copy()
    for i in range(n):
        L.vox_quat_mul(_p(g["q1"][i]), _p(g["q2"][i]), _p(prod[i]))
        L.vox_rotate_vector(_p(g["unit"][i]), _p(g["v"][i]), _p(rot[i]))
        L.vox_rotate_vector_q(_p(g["unit"][i]), _p(g["q2"][i]), _p(rotq[i]))
        L.vox_quat_normalize(_p(qn[i]))
        L.vox_dot_normalize(_p(dn[i]))
    for name, got in (("prod", prod), ("rot", rot), ("rotq", rotq), ("qn", qn), ("dn", dn)):
        assert _bits_equal(got, g[name]), name
    ident = np.full(4, 9.0, np.float32)
    L.vox_quat_set_identity(_p(ident))
    assert _bits_equal(ident, g["identity"])


def _rot(L, q, v):
    r = np.zeros(3, np.float32)
    L.vox_rotate_vector(_p(np.asarray(q, np.float32)), _p(np.asarray(v, np.float32)), _p(r))
    return r


def _close(a, b):
    return float(np.max(np.abs(np.asarray(a, np.float32) - np.asarray(b, np.float32)))) <= PRECISE


def test_reference_suite_rotations(L):
    ident = np.zeros(4, np.float32)
    L.vox_quat_set_identity(_p(ident))
    for d in (_f(1, 2, 4), _f(-321, 22, 124), _f(-321, 22, -124)):               # tests.c:79-96
        assert _close(_rot(L, ident, d), d)
    c, s = math.cos(0.1), math.sin(0.1)                                             # tests.c:98-120
    for q, v in ((_f(c, s, 0, 0), _f(1, 0, 0)), (_f(c, 0, s, 0), _f(0, 1, 0)), (_f(c, 0, 0, s), _f(0, 0, 1))):
        assert _close(_rot(L, q, v), v)
    sc = np.float32(math.sqrt(2.0) / 2.0)                                           # tests.c:122-146
    for q, v, e in ((_f(sc, 0, sc, 0), _f(1, 0, 0), _f(0, 0, -1)),
                    (_f(sc, 0, 0, sc), _f(0, 1, 0), _f(-1, 0, 0)),
                    (_f(sc, sc, 0, 0), _f(0, 0, 1), _f(0, -1, 0))):
        v = v.copy()
        L.vox_rotate_vector(_p(q), _p(v), _p(v))                                   # in place, as there
        assert _close(v, e)
    r1 = _rot(L, _f(sc, sc, 0, 0), _f(0, 1, 0))                                     # tests.c:155-170
    r2 = _rot(L, _f(sc, 0, sc, 0), _f(1, 0, 0))
    assert _close(r1, -r2)
    phi, psi = np.float32(0.1), np.float32(0.2)                                     # tests.c:172-201
    b1 = _f(math.cos(phi), math.sin(phi), 0, 0)
    b2 = _f(math.cos(psi), 0, math.sin(psi), 0)
    br = _f(math.cos(phi) * math.cos(psi), math.sin(phi) * math.cos(psi), math.sin(psi) * math.cos(phi),
            math.sin(psi) * math.sin(phi))
    v = _f(132, 2, 35)
    assert _close(_rot(L, b1, _rot(L, b2, v)), _rot(L, br, v))
    v = _f(1, 5, 2)                                                                 # tests.c:203-212
    r = _rot(L, _f(0.5, 0.5, 0.5, 0.5), v)
    assert abs(float(v @ v) - float(r @ r)) < PRECISE


def test_reference_suite_quat_mul(L):                                              # tests.c:302-358
    def mul(a, b):
        r = np.zeros(4, np.float32)
        L.vox_quat_mul(_p(_f(*a)), _p(_f(*b)), _p(r))
        return r
    table = [((0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1)), ((0, 0, 1, 0), (0, 0, 0, 1), (0, 1, 0, 0)),
             ((0, 0, 0, 1), (0, 1, 0, 0), (0, 0, 1, 0)), ((0, 0, 1, 0), (0, 1, 0, 0), (0, 0, 0, -1)),
             ((0, 0, 0, 1), (0, 0, 1, 0), (0, -1, 0, 0)), ((0, 1, 0, 0), (0, 0, 0, 1), (0, 0, -1, 0)),
             ((4, 3, 2, 1), (1, 0, 0, 0), (4, 3, 2, 1)), ((1, 0, 0, 0), (4, 3, 2, 1), (4, 3, 2, 1)),
             ((4, 1, 2, 3), (2, 0, 2, 0), (4, -4, 12, 8))]
    for a, b, e in table:
        assert _close(mul(a, b), _f(*e)), (a, b)


def test_rotate_vector_q_leaves_the_scalar(L):
    res = _f(42, 0, 0, 0)
    L.vox_rotate_vector_q(_p(_f(1, 0, 0, 0)), _p(_f(3, 1, 2, 3)), _p(res))
    assert res[0] == 42 and _close(res[1:], _f(1, 2, 3))
