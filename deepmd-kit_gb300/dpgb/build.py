"""In-tree build of the CUDA library ``libdpgb.so`` for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel and the
objects are linked into ``dpgb/libdpgb.so`` (next to this file).  Rebuilds
only when a source or header is newer than the library.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)               # deepmd-kit_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(PKG, "libdpgb.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the dpgb CUDA library cannot be built")


def _sources():
    """CUDA translation units (nvcc) and host-only C++ ones (g++)."""
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cc")))


def _deps():
    return (_sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
            + [os.path.join(ROOT, "plugin", "deeppot_backend.cc")])


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++"), shutil.which("c++")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("no C++ compiler found")


def needs_build() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(PLUGIN):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    flags = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC] + ARCH
    if verbose:
        flags += ["-Xptxas", "-v"]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src).rsplit(".", 1)[0] + ".o")
        if src.endswith(".cc"):
            cmd = [cxx(), "-std=c++17", "-O2", "-fPIC", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        else:
            cmd = [cc] + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compilation failed on {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, _sources()))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_plugin(cc)
    return LIB


PLUGIN_SRC = os.path.join(ROOT, "plugin", "deeppot_backend.cc")
# the file name a reference host looks for when it loads the backend of .pth
# models (lib + deepmd_backend_pt + .so, in DP_BACKEND_PLUGIN_PATH)
PLUGIN = os.path.join(PKG, "libdeepmd_backend_pt.so")


def build_plugin(cc: str) -> str:
    """The DeepPot backend plugin library, linked to libdpgb.so next to it."""
    tmp = PLUGIN + ".tmp"
    cmd = [cc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-shared", "-I", INCLUDE, PLUGIN_SRC, "-o", tmp,
           "-L", PKG, "-ldpgb", "-lcudart", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"plugin build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, PLUGIN)
    return PLUGIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
