"""Compile parts of the reference's own code into oracle/_ref/ (checker only).

TEST INFRASTRUCTURE ONLY.  Three pieces of the reference's relaxation path are
compiled from its sources, where they lie, with C-ABI shims of this project:

* geometry_tools/polygonise.cpp (+ polygonise.h): needs nothing but the C++
  standard library; pins the oracle's marching-cubes surface area.
* geometry_tools/AABB_calculator.cpp (+ its header): needs nothing but the
  C++ standard library; pins the oracle's segment-in-cell length (the
  SEGMENT cells' term of the cut-cell pass).
* base_cls_particle/particle.cpp: the smoothing kernels and their gradients
  (Kernel_function*, Derivative_kernel_function*) and Set_particle_scale.  Its
  global headers include TBB, Boost (MPI, serialization, graph) and the
  solver classes; the stand-in headers of oracle/ref_stubs/ (empty TBB/Boost
  headers, a two-member SPH class) take their place, so the file compiles as
  it is.  GCC's -I- makes the stand-ins shadow the headers that sit next to
  particle.cpp (sph.h, level_infor.h, Mypool.h); the reference's glbparam.h,
  glbcls.h, glbfunc.h and particle.h are used unchanged.  One library per
  dimension and kernel macro (the reference selects both at compile time).

The reference's source root comes from MRSPH_REFERENCE_SRC (default: the
reference checkout's src/ directory of this container); nothing is built when
it is absent (the GPU machines).  Outputs go to oracle/_ref/ only.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = os.environ.get("MRSPH_REFERENCE_SRC", "/root/reference/src")
OUT_DIR = os.path.join(HERE, "_ref")
OUT = os.path.join(OUT_DIR, "libref_polygonise.so")
SHIM = os.path.join(HERE, "ref_polygonise_shim.cpp")
KSHIM = os.path.join(HERE, "ref_kernels_shim.cpp")
ASHIM = os.path.join(HERE, "ref_aabb_shim.cpp")
AABB_OUT = os.path.join(OUT_DIR, "libref_aabb.so")
STUBS = os.path.join(HERE, "ref_stubs")
# kernel ids of the C ABI (hyperbolic, cubic, Wendland, Gaussian, quintic) ->
# the reference's compile-time kernel macros (Makefile.in:36-40)
KERNEL_MACROS = {0: "_HYPERBOLIC_KERNEL_", 1: "_CUBIC_SPLINE_", 2: "_WINDLAND_C4_", 3: "_GAUSSIAN_",
                 4: "_QUINTIC_SPLINE_"}
KERNEL_NAMES = {0: "hyperbolic", 1: "cubic", 2: "wendland", 3: "gaussian", 4: "quintic"}


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "geometry_tools", "polygonise.cpp"))


def aabb_available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "geometry_tools", "AABB_calculator.cpp"))


def build_aabb(force: bool = False):
    srcs = [ASHIM, os.path.join(REF_SRC, "geometry_tools", "AABB_calculator.cpp")]
    if not force and _fresh(AABB_OUT, srcs):
        return AABB_OUT
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
           os.path.join(REF_SRC, "geometry_tools")] + srcs + ["-o", AABB_OUT + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(AABB_OUT + ".tmp", AABB_OUT)
    return AABB_OUT


def kernels_available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "base_cls_particle", "particle.cpp"))


def kernel_lib(dim: int, kernel: int) -> str:
    return os.path.join(OUT_DIR, f"libref_kernels_{dim}d_{KERNEL_NAMES[kernel]}.so")


def _fresh(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def build_polygonise(force: bool = False):
    srcs = [SHIM, os.path.join(REF_SRC, "geometry_tools", "polygonise.cpp")]
    if not force and _fresh(OUT, srcs):
        return OUT
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I",
           os.path.join(REF_SRC, "geometry_tools")] + srcs + ["-o", OUT + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


def build_kernels(force: bool = False):
    """The ten particle.cpp libraries (2D/3D x five kernels); returns their paths."""
    part = os.path.join(REF_SRC, "base_cls_particle", "particle.cpp")
    stubs = [os.path.join(dp, f) for dp, _, fs in os.walk(STUBS) for f in fs]
    srcs = [KSHIM, part] + stubs
    jobs, outs = [], []
    for dim in (2, 3):
        for k, macro in KERNEL_MACROS.items():
            out = kernel_lib(dim, k)
            outs.append(out)
            if not force and _fresh(out, srcs):
                continue
            cmd = ["g++", "-O2", "-std=c++11", "-w", "-ffp-contract=off", "-fPIC", "-shared",
                   "-D_DOUBLE_", "-D_MESH_GENERATION_", f"-D_DIM{dim}_", f"-D{macro}",
                   "-I", STUBS, "-I", REF_SRC, "-I", os.path.join(REF_SRC, "base_cls_particle"), "-I-",
                   "-I", STUBS, KSHIM, part, "-o", out + ".tmp"]
            jobs.append((cmd, out))
    procs = [(subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), o) for c, o in jobs]
    for p, o in procs:
        log = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            raise RuntimeError("reference kernel build failed:\n" + log)
        os.replace(o + ".tmp", o)
    return outs


def build(force: bool = False):
    """Returns the polygoniser library path, or None when the reference is absent."""
    if not available():
        return OUT if os.path.exists(OUT) else None
    os.makedirs(OUT_DIR, exist_ok=True)
    build_polygonise(force)
    if aabb_available():
        build_aabb(force)
    if kernels_available():
        build_kernels(force)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
