"""The C ABI library: builds, loads, exports what include/*.h declares, and
keeps the reference's struct layouts (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import pytest

from voxvision_gb300 import _lib
from voxvision_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        src = open(os.path.join(INCLUDE, f)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"\{[^{}]*\}", "{}", src)          # struct bodies
        for m in re.finditer(r"\b(vox_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def libpath():
    return build()


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert "vox_voxel" in exported


def test_library_loads_with_signatures(libpath):
    L = _lib.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.vox_cuda_version().startswith(b"voxtrees_cuda")
    assert L.vox_cuda_strerror(-4) == b"tree deeper than the traversal stack supports"


class VoxNode(C.Structure):
    """struct vox_node of the reference, scalar build (tree.h:28-38)."""
    class _Data(C.Union):
        class _Inner(C.Structure):
            _fields_ = [("center", C.c_float * 3), ("children", C.c_void_p * 8)]
        _fields_ = [("dots", C.c_void_p), ("inner", _Inner)]
    _fields_ = [("box", C.c_float * 6), ("flags", C.c_uint), ("dots_num", C.c_uint), ("data", _Data)]


def test_node_layout_matches_reference(tmp_path):
    """sizeof/offsetof of the library's struct vox_node equal the reference's
    scalar layout (112 bytes; data at 32; children at 48)."""
    assert C.sizeof(VoxNode) == 112
    src = tmp_path / "l.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "voxtrees.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu", sizeof(struct vox_node),'
                   ' offsetof(struct vox_node, data), offsetof(struct vox_node, data.inner.children),'
                   ' offsetof(struct vox_node, flags));return 0;}\n')
    exe = tmp_path / "l"
    subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    assert subprocess.run([str(exe)], capture_output=True, text=True).stdout == "112 32 48 24"


def test_headers_compile_as_c_and_cpp(tmp_path):
    for lang, comp in (("c", "gcc"), ("cpp", "g++")):
        src = tmp_path / f"h.{lang}"
        src.write_text('#include "voxtrees_cuda.h"\n#include "voxtrees.h"\n#include "voxrnd.h"\n'
                       'int main(void){return 0;}\n')
        subprocess.run([comp, "-Wall", "-Werror", "-I", INCLUDE, "-c", str(src), "-o",
                        str(tmp_path / f"h_{lang}.o")], check=True)
