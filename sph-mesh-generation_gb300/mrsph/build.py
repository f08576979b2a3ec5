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
    "mrsph_tet.cu": ["-fmad=false"],
    "mrsph_batch.cu": [],
    "mrsph_persist.cu": [],
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


TUNED = os.path.join(PKG, "tuned.json")


def tuned_defines() -> list:
    """Tuning macros of the neighbour passes: MRSPH_NVCC_DEFINES when set
    (e.g. "-DMRSPH_DENSITY_MIN_BLOCKS=4"), else those an autotuner run wrote
    to mrsph/tuned.json (mrsph/autotune.py), else none (the engine's
    defaults, tuned on a GB300 for the 3D torus)."""
    env = os.environ.get("MRSPH_NVCC_DEFINES")
    if env is not None:
        return env.split()
    if os.path.exists(TUNED):
        import json
        with open(TUNED) as f:
            return ["-DMRSPH_%s=%d" % (k, int(v)) for k, v in sorted(json.load(f)["defines"].items())]
    return []


def build(force: bool = False, verbose: bool = False, defines: list = None, build_dir: str = None,
          lib_path: str = None) -> str:
    """Compile the library; defines / build_dir / lib_path override the tuning
    macros and the output locations (the autotuner builds its candidates
    side by side)."""
    bdir = build_dir or BUILD
    out_lib = lib_path or LIB
    os.makedirs(bdir, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(os.path.dirname(ROOT), "include", "mrsph_relax.h"))
    base = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
            "--expt-relaxed-constexpr", "-I", CSRC]
    base += tuned_defines() if defines is None else list(defines)
    jobs = []
    objs = []
    for src, extra in SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(bdir, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *headers] + ([TUNED] if os.path.exists(TUNED) else [])):
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
    if force or jobs or _stale(out_lib, objs):
        tmp = out_lib + ".tmp"
        r = subprocess.run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, out_lib)
    return out_lib


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
