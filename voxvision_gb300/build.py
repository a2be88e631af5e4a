"""Build libvoxtrees_cuda.so in-tree (nvcc for sm_103a, gcc/g++ for the host C/C++).

    python -m voxvision_gb300.build        # or voxvision_gb300.build.build()
    python -m voxvision_gb300.build --checked

Translation units compile in parallel; the result is
voxvision_gb300/libvoxtrees_cuda.so (git-ignored).  `--checked` (build(checked=True))
makes libvoxtrees_cuda_checked.so beside it with -DVOX_CUDA_CHECKED: searches
that check every load's index against the uploaded arrays (selected at run
time with VOXTREES_CUDA_LIB).  The host C of the tree
builder is compiled with -ffp-contract=off so its float arithmetic matches the
reference's own build; the CUDA code uses explicitly rounded intrinsics and is
additionally compiled with --fmad=false.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libvoxtrees_cuda.so")
CHECKED_OUT_DIR = os.path.join(HERE, "_build_checked")
CHECKED_LIB = os.path.join(HERE, "libvoxtrees_cuda_checked.so")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = ["-O3", ARCH, "-lineinfo", "-std=c++17", "--fmad=false", "-Xptxas", "-v",
              "-Xcompiler", "-fPIC,-fvisibility=hidden"]
CC_FLAGS = ["-O2", "-std=gnu11", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall",
            "-Wno-unused-parameter"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-Wall"]

CUDA_SOURCES = ["voxtrees_cuda.cu", "batch.cu", "server.cu", "build.cu", "raysort.cu", "make_tree.cu"]
C_SOURCES = ["host_tree.c", "cameras.c", "lights.c", "modules.c"]
CXX_SOURCES = ["flatten.cpp", "dropin_search.cpp", "renderer.cpp"]


def _nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _stale(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(os.path.dirname(HERE), "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build(verbose: bool = False, force: bool = False, checked: bool = False) -> str:
    out_dir, lib = (CHECKED_OUT_DIR, CHECKED_LIB) if checked else (OUT_DIR, LIB)
    nvcc_flags = NVCC_FLAGS + (["-DVOX_CUDA_CHECKED"] if checked else [])
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    hdrs = _headers()
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append((src, [nvcc, *nvcc_flags, "-c", s, "-o", o]))
    for src in C_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append((src, ["gcc", *CC_FLAGS, "-c", s, "-o", o]))
    for src in CXX_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(out_dir, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append((src, ["g++", *CXX_FLAGS, "-I", cuda_inc, "-c", s, "-o", o]))
    procs = [(name, cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
             for name, cmd in jobs]
    failed = []
    for name, cmd, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stdout.write(f"--- {name}\n{out}")
        if p.returncode:
            failed.append(name)
    if failed:
        raise RuntimeError(f"compilation failed: {failed}")
    if jobs or not os.path.exists(lib):
        tmp = lib + ".tmp"
        cmd = [nvcc, ARCH, "-shared", "-o", tmp, *objs, "-Xlinker", "-Bsymbolic", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode:
            sys.stdout.write(r.stdout)
            raise RuntimeError("link failed")
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv, checked="--checked" in sys.argv))
