"""The module loader (modules.c:1-69) and the data-file search
(datareader.c:88-125): a camera class built as a module the way the
reference's camera plugins are (`<name>.so` with module_init(), compiled here
against include/voxrnd.h) is found through $VOXVISION_MODULES and used
through vox_camera_methods like a built-in class; modules that are missing,
of another class or without module_init are refused; data files are found as
given, then in $VOXVISION_DATA, then in $HOME/.voxvision.  No GPU is used."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from voxvision_gb300 import lib
from voxvision_gb300.cameras import CONS, DESTROY, DOTM, S2W, WS

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")

CAMERA_MODULE_SRC = r"""
#include <stdlib.h>
#include <string.h>
#include "voxrnd.h"

/* A panorama-like test class: the ray of pixel (sx, sy) is
 * (sx / w - 0.5, 1, 0.5 - sy / h) before any rotation. */
struct test_camera {
    struct vox_camera_interface *iface;
    float pos[3];
    int w, h;
};

static void set_number(struct vox_camera *c, const char *name, float v) {}
static void set_dot(struct vox_camera *c, const char *name, const vox_dot v)
{
    if (strcmp(name, "position") == 0) memcpy(((struct test_camera *)c)->pos, v, sizeof(vox_dot));
}
static void screen2world(const struct vox_camera *c, vox_dot ray, int sx, int sy)
{
    const struct test_camera *t = (const struct test_camera *)c;
    ray[0] = (float)sx / (float)t->w - 0.5f;
    ray[1] = 1.0f;
    ray[2] = 0.5f - (float)sy / (float)t->h;
}
static void rotate(struct vox_camera *c, const vox_dot d) {}
static void move(struct vox_camera *c, const vox_dot d)
{
    for (int i = 0; i < 3; i++) ((struct test_camera *)c)->pos[i] += d[i];
}
static void look_at(struct vox_camera *c, const vox_dot d) {}
static void get_position(const struct vox_camera *c, vox_dot r)
{
    memcpy(r, ((const struct test_camera *)c)->pos, sizeof(vox_dot));
}
static void window_size(struct vox_camera *c, int w, int h)
{
    ((struct test_camera *)c)->w = w;
    ((struct test_camera *)c)->h = h;
}
static struct vox_camera *construct(const struct vox_camera *old);
static void destroy(struct vox_camera *c) { free(c); }

static struct vox_camera_interface methods = {set_number, set_dot, screen2world, rotate, move, look_at,
                                              get_position, window_size, construct, destroy};

static struct vox_camera *construct(const struct vox_camera *old)
{
    struct test_camera *c = calloc(1, sizeof *c);
    if (old) memcpy(c, old, sizeof *c);
    else c->w = c->h = 1;
    c->iface = &methods;
    return (struct vox_camera *)c;
}

static struct vox_module module = {MODULE_TYPE, (struct vox_module_methods *)&methods};
struct vox_module *module_init(void) { return &module; }
"""


def _build(tmp_path, name, src, defines=()):
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    c = tmp_path / f"{name}.c"
    c.write_text(src)
    subprocess.run(["gcc", "-shared", "-fPIC", "-O1", "-I", INCLUDE, *defines, "-o", str(tmp_path / f"{name}.so"),
                    str(c)], check=True)


@pytest.fixture
def modules(tmp_path, monkeypatch):
    _build(tmp_path, "test-camera", CAMERA_MODULE_SRC, ["-DMODULE_TYPE=CAMERA_MODULE"])
    _build(tmp_path, "other-kind", CAMERA_MODULE_SRC, ["-DMODULE_TYPE=7"])
    _build(tmp_path, "no-init", "int nothing_here(void) { return 0; }\n")
    monkeypatch.setenv("VOXVISION_MODULES", str(tmp_path))
    L = lib()
    L.vox_camera_methods.restype = C.c_void_p
    L.vox_camera_methods.argtypes = [C.c_char_p]
    L.vox_load_module.restype = C.c_void_p
    L.vox_load_module.argtypes = [C.c_char_p, C.c_int]
    return L


def test_camera_module_is_used_like_a_builtin_class(modules):
    L = modules
    builtin = L.vox_camera_methods(b"simple-camera")
    m = L.vox_camera_methods(b"test-camera")
    assert m and m != builtin
    assert L.vox_load_module(b"test-camera", 0) == m                     # the same methods again
    tbl = C.cast(m, C.POINTER(C.c_void_p * 10)).contents
    cam = CONS(tbl[8])(None)
    WS(tbl[7])(cam, 200, 100)
    ray = np.zeros(3, np.float32)
    S2W(tbl[2])(cam, ray.ctypes.data_as(C.c_void_p), 50, 25)
    assert np.array_equal(ray, np.array([50 / 200 - 0.5, 1, 0.5 - 25 / 100], np.float32))
    pos = np.array([1, 2, 3], np.float32)
    DOTM(tbl[4])(cam, pos.ctypes.data_as(C.c_void_p))                     # move by (1, 2, 3)
    got = np.zeros(3, np.float32)
    DOTM(tbl[6])(cam, got.ctypes.data_as(C.c_void_p))
    assert np.array_equal(got, pos)
    DESTROY(tbl[9])(cam)
    assert L.vox_camera_methods(b"simple-camera") == builtin              # built-ins answered first


def test_refused_modules(modules):
    L = modules
    assert not L.vox_camera_methods(b"no-such-camera")
    assert not L.vox_camera_methods(b"other-kind")                         # module of another class
    assert L.vox_load_module(b"other-kind", 7)                             # ... which loads as its own
    assert not L.vox_load_module(b"no-init", 0)                            # no module_init
    assert not L.vox_camera_methods(None)


def test_find_data_file(tmp_path, monkeypatch):
    L = lib()
    L.vox_find_data_file.argtypes = [C.c_char_p, C.c_char_p]
    L.vox_find_data_file.restype = C.c_int
    out = C.create_string_buffer(4096)
    data = tmp_path / "data"
    data.mkdir()
    (data / "skull.dat").write_bytes(b"\0" * 8)
    assert L.vox_find_data_file(str(data / "skull.dat").encode(), out) == 1          # as given
    assert out.value.decode() == str(data / "skull.dat")
    monkeypatch.setenv("VOXVISION_DATA", str(data))
    assert L.vox_find_data_file(b"skull.dat", out) == 1                              # $VOXVISION_DATA
    assert out.value.decode() == os.path.join(str(data), "skull.dat")
    assert L.vox_find_data_file(b"bonsai.dat", out) == 0
    home = tmp_path / "home"
    (home / ".voxvision").mkdir(parents=True)
    (home / ".voxvision" / "bonsai.dat").write_bytes(b"\0")
    monkeypatch.delenv("VOXVISION_DATA")
    monkeypatch.setenv("HOME", str(home))
    assert L.vox_find_data_file(b"bonsai.dat", out) == 1                             # $HOME/.voxvision
    assert out.value.decode() == os.path.join(str(home), ".voxvision", "bonsai.dat")
    assert L.vox_find_data_file(str(data).encode(), out) == 0                        # a directory is no file
