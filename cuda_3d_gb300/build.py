"""Build recipe of the native library (nvcc only, no cmake).

Compiles every translation unit under csrc/ for sm_103a in parallel and links
them into cuda_3d_gb300/_lib/libgca3d.so (CUDA runtime linked statically, so the
library is self-contained for C and C++ callers).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libgca3d.so")
OBJDIR = os.path.join(LIBDIR, "obj")
# the checked build: device-side index checks compiled in (GCA3D_CHECKED), each failure
# a status (an error bit of the context), never a fault or a trap; same entry points
LIB_CHECKED = os.path.join(LIBDIR, "libgca3d_checked.so")
OBJDIR_CHECKED = os.path.join(LIBDIR, "obj_checked")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include"),
              "-I", CSRC]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgca3d")
    return exe


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src, extra, objdir=OBJDIR):
    obj = os.path.join(objdir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}")
    return obj


def _stale(lib=LIB):
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = sources() + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(ROOT, "include", "gca3d.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, extra=(), verbose=False, checked=False):
    """libgca3d.so, or with checked=True libgca3d_checked.so (index checks compiled in)"""
    lib, objdir = (LIB_CHECKED, OBJDIR_CHECKED) if checked else (LIB, OBJDIR)
    extra = list(extra) + (["-DGCA3D_CHECKED"] if checked else [])
    if not force and not _stale(lib):
        return lib
    os.makedirs(objdir, exist_ok=True)
    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra, objdir), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-ldl", "-lpthread", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
