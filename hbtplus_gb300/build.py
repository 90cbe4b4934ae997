"""In-tree build of the CUDA library (hbtplus_gb300/_build/libhbtu.so).

Each .cu translation unit is compiled for sm_103a only, in parallel, and the
objects are linked into one shared library with the CUDA runtime linked
statically, so the library loads on a host without a GPU (for the symbol
checks) and needs nothing but the driver on a GPU host.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libhbtu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["prims.cu", "tree.cu", "walk.cu", "loop.cu", "small.cu", "capi.cu", "noalloc.cu",
           "direct.cu", "index.cu", "props.cu", "merge.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
                     "-I" + INCLUDE]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build hbtplus_gb300")


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra_flags=()) -> str:
    """Compile and link the library if any source changed; return its path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    headers = _headers()
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        if force or _stale(o, [s] + headers):
            jobs.append([cc] + NVCC_FLAGS + list(extra_flags) + ["-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if force or jobs or _stale(LIB, objs):
        run([cc] + ARCH + ["-shared", "--cudart", "static", "-o", LIB] + objs)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
