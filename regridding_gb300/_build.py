"""In-tree build of ``libregrid_gb300.so`` (CUDA, sm_103a) with nvcc.

Each ``csrc/*.cu`` translation unit is compiled in parallel into
``_build/*.o`` and linked into one shared library with the CUDA runtime
linked statically, so the library only needs the NVIDIA driver at run time.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libregrid_gb300.so")
# the debug library (-DRG_DEBUG: bounds-checked grid reads in the builds,
# reported as errors); regridding_gb300 loads it when RG_DEBUG=1
BUILD_DEBUG = os.path.join(HERE, "_build_debug")
LIB_DEBUG = os.path.join(BUILD_DEBUG, "libregrid_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE]


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build regridding_gb300")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, debug: bool = False) -> str:
    """Compile the CUDA sources if needed and return the path of the library
    (with ``debug``, the bounds-checked variant in ``_build_debug``)."""
    BUILD = BUILD_DEBUG if debug else globals()["BUILD"]
    LIB = LIB_DEBUG if debug else globals()["LIB"]
    flags = NVCC_FLAGS + (["-DRG_DEBUG"] if debug else [])
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    headers.append(os.path.join(INCLUDE, "regrid_gb300.h"))
    exe = nvcc()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        if force or _stale(obj, [src] + headers):
            cmd = [exe, *ARCH, *flags, "-c", src, "-o", obj]
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
            if verbose:
                print(res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread", "-ldl"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB
