"""Compile the reference's own marching-cubes polygoniser into oracle/_ref/.

TEST INFRASTRUCTURE ONLY.  The one part of the reference's relaxation path
that compiles from its own sources without TBB, Boost or voro++ is
geometry_tools/polygonise.cpp (+ polygonise.h); it is built here, where the
reference sources lie, with a C-ABI shim (oracle/ref_polygonise_shim.cpp) and
pins the oracle's surface-area restatement.  Outputs go to oracle/_ref/ only.
Does nothing when the reference sources are absent.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SRC = "/root/reference/src/geometry_tools"
OUT = os.path.join(HERE, "_ref", "libref_polygonise.so")
SHIM = os.path.join(HERE, "ref_polygonise_shim.cpp")


def available() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "polygonise.cpp"))


def build(force: bool = False):
    """Returns the library path, or None when the reference is absent."""
    if not available():
        return OUT if os.path.exists(OUT) else None
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    srcs = [SHIM, os.path.join(REF_SRC, "polygonise.cpp")]
    if not force and os.path.exists(OUT) and all(os.path.getmtime(OUT) >= os.path.getmtime(s) for s in srcs):
        return OUT
    cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-I", REF_SRC] + srcs + \
          ["-o", OUT + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
