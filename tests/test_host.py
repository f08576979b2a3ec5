"""The C++ host layer (host/*.cpp: SPH_mesh_generation, Solver and the
mrsph_relax driver over the C ABI) on the CPU: it builds, its workloads
count the same particles as the Python workloads, and without a GPU it
fails with the engine's message and status 2.  The GPU runs are in
test_gpu_host.py."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sph-mesh-generation_gb300"))
from mrsph import build, cases  # noqa: E402


@pytest.fixture(scope="module")
def binary():
    return build.build_host()


def run(binary, *args):
    return subprocess.run([binary, *args], capture_output=True, text=True, timeout=300)


def test_help(binary):
    r = run(binary, "--help")
    assert r.returncode == 0 and "--case" in r.stdout
    assert run(binary, "--bogus").returncode == 1


def test_counts_match_python_workloads(binary):
    d = json.loads(run(binary, "--case", "disc_hole_2d", "--count-only").stdout)
    assert d["n_particles"] == cases.disc_hole_2d(spacing=0.02, grid=64).n_particles
    t = json.loads(run(binary, "--case", "torus_3d", "--count-only").stdout)
    assert t["n_particles"] == cases.torus_3d().n_particles


def test_engine_error_without_gpu(binary):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    r = run(binary, "--case", "disc_hole_2d", "--steps", "1")
    assert r.returncode == 2 and "mrsph_create" in r.stderr


def test_cpp_particle_vtu_matches_python_writer(binary, tmp_path):
    """The C++ Particle_binary_writer writes the same bytes as the Python
    writer (mrsph/io.py) for the same particle arrays."""
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_particle_vtu
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_longlong] + [ctypes.c_void_p] * 5
    rng = np.random.default_rng(4)
    n = 1000
    xyz = rng.random((n, 3))
    typ = rng.integers(0, 2, n).astype(np.int32)
    h = rng.random(n)
    nn = rng.integers(1, 90, n).astype(np.int32)
    nrm = rng.normal(size=(n, 3))
    p = tmp_path / "c.vtu"
    size = f(str(p).encode(), n, xyz.ctypes.data, typ.ctypes.data, h.ctypes.data, nn.ctypes.data, nrm.ctypes.data)
    pd = [("id", np.arange(n, dtype="<i4")), ("local_id", np.arange(n, dtype="<i4")), ("type", typ),
          ("h", h.astype("<f4")), ("NN", nn), ("color", np.zeros(n, dtype="<i4")), ("norm", nrm.astype("<f4"))]
    ref = io.vtu_bytes(xyz, np.arange(n, dtype="<i4"), 1, pd)
    got = p.read_bytes()
    assert size == len(ref) and got == ref
    back = io.read_vtu(str(p))
    assert np.array_equal(back["NN"], nn) and np.array_equal(back["Position"], xyz.astype(np.float32))
