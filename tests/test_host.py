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
