"""Build the CUDA extension libmrsph_relax.so for sm_103a (in-tree, no cmake).

Each translation unit is compiled by nvcc in parallel, then linked as a
shared library exporting the C ABI of include/mrsph_relax.h.  The FP64 engine
and the level-set build are compiled with -fmad=false so that FP64 results
follow the reference's operation order.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # sph-mesh-generation_gb300/
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "_build")
LIB = os.path.join(ROOT, "libmrsph_relax.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "mrsph_api.cu": [],
    "mrsph_sort.cu": [],
    "mrsph_levelset.cu": ["-fmad=false"],
    "mrsph_fp64.cu": ["-fmad=false"],
    "mrsph_fp32.cu": [],
    "mrsph_noalloc.cu": [],
    "mrsph_cvp.cu": ["-fmad=false"],
    "mrsph_tri.cu": ["-fmad=false"],
    "mrsph_batch.cu": [],
}


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "mrsph_relax.h"))
    base = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
            "--expt-relaxed-constexpr", "-I", CSRC]
    # tuning macros of the neighbour passes (e.g. "-DMRSPH_DENSITY_MIN_BLOCKS=4")
    base += os.environ.get("MRSPH_NVCC_DEFINES", "").split()
    jobs = []
    objs = []
    for src, extra in SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            jobs.append(base + extra + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed:\n" + " ".join(j) + "\n" + r.stdout + r.stderr)
                if verbose:
                    print(r.stdout + r.stderr)
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


HOST = os.path.join(ROOT, "host")
HOST_LIB = os.path.join(ROOT, "libmrsph_host.so")
HOST_BIN = os.path.join(ROOT, "mrsph_relax")


def gxx() -> str:
    for c in (shutil.which("g++"), "/usr/bin/g++"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("g++ not found")


def build_host(force: bool = False) -> str:
    """The C++ host layer (host/*.cpp, the reference's SPH_mesh_generation and
    Solver entry points over the C ABI) as libmrsph_host.so, and its
    command-line driver mrsph_relax, both linked against libmrsph_relax.so."""
    lib = build(force=force)
    srcs = [os.path.join(HOST, "sph_mesh_generation.cpp")]
    deps = srcs + [os.path.join(HOST, "sph_mesh_generation.hpp"),
                   os.path.join(os.path.dirname(ROOT), "include", "mrsph_relax.h"), lib]
    flags = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-I", HOST]
    link = ["-L", ROOT, "-lmrsph_relax", "-Wl,-rpath,$ORIGIN"]
    if force or _stale(HOST_LIB, deps):
        r = subprocess.run([gxx(), *flags, "-shared", "-o", HOST_LIB + ".tmp", *srcs, *link],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed (host library):\n" + r.stdout + r.stderr)
        os.replace(HOST_LIB + ".tmp", HOST_LIB)
    main = os.path.join(HOST, "mrsph_relax_main.cpp")
    if force or _stale(HOST_BIN, deps + [main, HOST_LIB]):
        r = subprocess.run([gxx(), *flags, "-o", HOST_BIN + ".tmp", main, "-L", ROOT, "-lmrsph_host",
                            *link], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed (mrsph_relax):\n" + r.stdout + r.stderr)
        os.replace(HOST_BIN + ".tmp", HOST_BIN)
    return HOST_BIN


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
