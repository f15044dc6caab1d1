"""In-tree build of libcbk_cuda.so (the CUDA kernels and the C ABI).

Every translation unit under csrc/ is compiled for sm_103a only, in parallel,
into csrc/../_build/, and linked into cbk_gb300/libcbk_cuda.so with the static
CUDA runtime (the library then loads without a CUDA runtime on the library
path). A unit is rebuilt when it or any header under csrc/ or include/ is
newer than its object.

Floating-point contraction is off (--fmad=false): the kernels write every
fused multiply-add they want as fma(), so each arithmetic result is fixed by
the source and identical between the register, shared-memory and
global-memory variants of a routine.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcbk_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-O2", "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libcbk_cuda.so")


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _stale(src: str, obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in [src] + deps)


LIB_CHECKED = os.path.join(PKG, "libcbk_cuda_checked.so")


def build(verbose: bool = False, jobs: int | None = None, checked: bool = False) -> str:
    """Compile and link; returns the library path. checked=True builds the
    bounds-checked variant (CBK_CUDA_CHECKED; libcbk_cuda_checked.so, objects
    in _build/checked): every matrix-view access tested against its extent,
    for the tests, not for speed."""
    build_dir = os.path.join(BUILD, "checked") if checked else BUILD
    lib_path = LIB_CHECKED if checked else LIB
    flags = NVCC_FLAGS + (["-DCBK_CUDA_CHECKED"] if checked else [])
    os.makedirs(build_dir, exist_ok=True)
    cc = nvcc()
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    deps = _headers()
    objs = []
    todo = []
    for src in sources:
        obj = os.path.join(build_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(src, obj, deps):
            lang = [] if src.endswith(".cu") else ["-x", "cu"]
            todo.append([cc, "-c"] + lang + flags + [src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for msg in ex.map(run, todo):
            if verbose and msg:
                print(msg)
    if todo or not os.path.exists(lib_path) or any(
            os.path.getmtime(o) > os.path.getmtime(lib_path) for o in objs):
        tmp = lib_path + ".tmp"
        run([cc, "-shared"] + ARCH + ["-cudart", "static", "-o", tmp] + objs)
        os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
