"""Build recipe for the engine's shared library (no CMake).

``build()`` compiles the host C++ (CObjects buffer, lattice compiler) with
g++ and the CUDA sources for sm_103a with nvcc, in parallel, and links
``sixtracklib_gb300/lib/libsixtracklib_gb300.so`` in the source tree.  The
tracking kernel's translation unit is compiled with ``-fmad=false``: the
exact arithmetic policy relies on it, the fast one uses explicit fma().
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OUT_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(OUT_DIR, "libsixtracklib_gb300.so")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

HOST_SOURCES = ["buffer.cpp", "lattice.cpp", "output_buffer.cpp", "aliases.cpp"]
CUDA_SOURCES = {
    "track_kernel.cu": ["-fmad=false"],
    "engine.cu": [],
    "probe.cu": [],
    "compact.cu": [],
    "noalloc.cu": [],
    "adjoint.cu": [],
    "batch.cu": [],
    "tricub.cu": ["-fmad=false"],
}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the engine")
    return cand


def _sources():
    return [os.path.join(CSRC, f) for f in HOST_SOURCES + list(CUDA_SOURCES)] + [
        os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))
    ] + [os.path.join(INCLUDE, "sixtracklib_gb300.h")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def _compile(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the engine library if any source is newer; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    common = ["-O3", "-I" + INCLUDE, "-I" + CSRC]
    jobs = []
    objs = []
    for f in HOST_SOURCES:
        o = os.path.join(OBJ_DIR, f + ".o")
        objs.append(o)
        # no FMA contraction: the lattice compiler's element constants are the
        # reference's expressions, rounded as it rounds them
        jobs.append(["g++", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", *common, "-c",
                     os.path.join(CSRC, f), "-o", o])
    for f, extra in CUDA_SOURCES.items():
        o = os.path.join(OBJ_DIR, f + ".o")
        objs.append(o)
        jobs.append([nvcc, "-std=c++17", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xptxas", "-v" if verbose else "-O3", *extra, *common, "-c",
                     os.path.join(CSRC, f), "-o", o])
    with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        outs = list(ex.map(_compile, jobs))
    if verbose:
        for o in outs:
            print(o)
    tmp = LIB + f".tmp{os.getpid()}"
    _compile([nvcc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
