"""The C++ host layer on the GPU: mrsph_relax (SPH_mesh_generation + Solver
over the C ABI, workloads built in C++) relaxes the same particles as the
Python mirror, and its .pst restarts and list.csv read back with the Python
reader."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sph-mesh-generation_gb300"))
from mrsph import SPHMeshGeneration, build, cases, io  # noqa: E402

pytestmark = pytest.mark.gpu


def test_cpp_driver_matches_python(tmp_path):
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "disc_hole_2d", "--precision", "fp64", "--steps", "6",
                        "--output-every", "3", "--out", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    assert d["n_particles"] == case.n_particles and d["step"] == 6 and d["flags"] == 0
    assert io.read_particle_list(str(tmp_path)) == (1, [(3, case.n_particles), (6, case.n_particles)])
    cpp = io.read_pst(str(tmp_path / "rstfile_particles" / "step_6_rank_0.pst"))
    g = SPHMeshGeneration(case, precision="fp64")
    g.Initialize_case()
    g.SPH_run_mesh_generation(6)
    py = g.particles(("xyz",))["xyz"]
    dt = g.stats()["dt"]
    g.close()
    assert np.max(np.abs(cpp - py)) < 1e-12
    assert abs(d["dt"] - dt) <= 1e-12 * abs(dt)


def test_cpp_driver_torus_fp32():
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "torus_3d", "--steps", "3"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    assert d["n_particles"] == 2410164 and d["step"] == 3 and d["particle_steps_per_s"] > 0


def test_cpp_driver_cut_cell_count():
    """--cut-cell-count seeds the reference's particle count (Get_num_particles
    over the cut-cell volume pass), the count the Python mirror reports."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "disc_hole_2d", "--precision", "fp64", "--steps", "2", "--cut-cell-count"],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    g = SPHMeshGeneration(case, precision="fp64")
    n = g.volume_mass(-1)["num_particle"]
    g.close()
    assert d["n_particles"] == n and d["step"] == 2 and d["flags"] == 0


def test_cpp_driver_writes_particle_vtu(tmp_path):
    """--vtu writes the reference's particle VTU series at every output; the
    pieces read back with the Python reader and carry the restart's positions."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "disc_hole_2d", "--precision", "fp64", "--steps", "6",
                        "--output-every", "3", "--out", str(tmp_path), "--vtu"], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    out = tmp_path / "outdata"
    assert (out / "particle.pvd").read_text().count("<DataSet") == 2
    v = io.read_vtu(str(out / "particle_rank_0_step_1.vtu"))
    pst = io.read_pst(str(tmp_path / "rstfile_particles" / "step_6_rank_0.pst"))
    assert np.array_equal(v["Position"], pst.astype(np.float32))
    assert np.array_equal(v["id"], np.arange(len(pst))) and v["NN"].min() >= 1
    assert (out / "particle_step_1.pvtu").exists()


def test_cpp_driver_writes_levelset_image(tmp_path):
    """--lset writes the level-set image; it equals the Python writer's for the
    same workload (header bytes and every field; the spacing field within
    FP32 rounding of the two tanh implementations)."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "disc_hole_2d", "--precision", "fp64", "--steps", "1", "--out",
                        str(tmp_path / "c"), "--lset"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    cpp = tmp_path / "c" / "outdata" / "mesh_lset_rank_0_step_0.vti"
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    g = SPHMeshGeneration(case, precision="fp64")
    py = io.LevelSetWriter(str(tmp_path / "p")).Output_lset(0, g, level=0, run_time=0)
    g.close()
    a, b = io.read_vtu(str(cpp)), io.read_vtu(py)
    head = lambda p: open(p, "rb").read().split(b"<AppendedData")[0]  # noqa: E731
    assert head(cpp) == head(py)
    for k in ("interface", "char"):
        assert np.array_equal(a[k], b[k]), k
    for k in ("phi", "curv", "vol", "area", "scale"):
        assert np.allclose(a[k], b[k], rtol=1e-6, atol=1e-30), k


@pytest.mark.parametrize("dim", [2, 3])
def test_cpp_driver_box_characteristics(tmp_path, dim):
    """A box with corners (and edges in 3D): the C++ driver passes the
    singularity points and segments to the engine; its level-set image
    ('char' = tag_characteristic) and level-set restart equal the Python
    writers' for the same workload, and its particles after relaxation match
    the Python mirror's (SINGULARITY and SEGMENT particles included)."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", f"box_{dim}d", "--precision", "fp64", "--steps", "300",
                        "--output-every", "300", "--out", str(tmp_path / "c"), "--lset", "--lset-restart"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    kw = dict(spacing=0.04, grid=32) if dim == 3 else dict(spacing=0.02, grid=64)
    case = cases.box_with_corners(dim=dim, kernel="hyperbolic", h_over_dx=1.0, **kw)
    g = SPHMeshGeneration(case, precision="fp64")
    py_vti = io.LevelSetWriter(str(tmp_path / "p")).Output_lset(0, g, level=0, run_time=0)
    py_rst = io.save_lset_restart(g, str(tmp_path / "p" / "levelset.rst"))
    ctag = io.characteristic_fields(g.characteristic_tags(0))[0]
    assert np.count_nonzero(ctag == 1) == len(case.extra["singularities"])
    cpp_vti = tmp_path / "c" / "outdata" / "mesh_lset_rank_0_step_0.vti"
    a, b = io.read_vtu(str(cpp_vti)), io.read_vtu(py_vti)
    assert np.array_equal(a["char"], b["char"]) and np.count_nonzero(a["char"] == 1) == len(ctag[ctag == 1])
    if dim == 3:
        assert np.count_nonzero(a["char"] == 2) > 0
    cpp_rst = (tmp_path / "c" / "rstfile" / "levelset.rst").read_bytes()
    rc, rp = io.load_lset_restart(str(tmp_path / "c" / "rstfile" / "levelset.rst")), io.load_lset_restart(py_rst)
    for k in ("singularities", "segments", "tag_characteristic", "idx_characteristic", "tag_interface", "phi"):
        assert np.array_equal(rc[k], rp[k]), k
    # the spacing fields differ by the two tanh implementations only
    assert len(cpp_rst) == len(open(py_rst, "rb").read())
    g.Initialize_case()
    g.SPH_run_mesh_generation(300)
    gp = g.particles(("xyz", "type"))
    g.close()
    cpp = io.read_pst(str(tmp_path / "c" / "rstfile_particles" / "step_300_rank_0.pst"))
    assert d["step"] == 300 and d["flags"] & ~8 == 0
    assert np.max(np.abs(cpp - gp["xyz"])) < 1e-12
    assert (gp["type"] == 2).any()


def test_cpp_driver_partitioning_matches_python():
    """--cvp K: SPH_mesh_generation::Partitioning (Voronoi::Partitioning over
    the C ABI) of the relaxed particles gives the VPs the Python API gives
    for the same particles and initial VPs, bit for bit."""
    binary = build.build_host()
    K, iters = 8, 100
    r = subprocess.run([binary, "--case", "disc_hole_2d", "--precision", "fp64", "--steps", "20", "--cvp", str(K),
                        "--cvp-iter", str(iters)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    g = SPHMeshGeneration(case, precision="fp64")
    g.Initialize_case()
    g.SPH_run_mesh_generation(20)
    x = g.particles(("xyz",))["xyz"]
    n = len(x)
    vp0 = np.array([x[k * n // K] for k in range(K)])
    vp, labels, mass, res = g.Partitioning(vp0, max_iter=iters)
    g.close()
    assert d["cvp"]["iterations"] == res["iterations"]
    assert np.array_equal(np.array(d["cvp"]["vp"]).reshape(K, 3), vp)


def test_cpp_driver_restart_run_matches_python(tmp_path):
    """The reference's two-run workflow: a level-set restart written by the
    C++ driver (--lset-restart) is relaxed by the C++ restart run
    (--load-lset-restart, Load_rst_case) and by the Python mirror
    (cases.from_lset_restart) to the same particles, SINGULARITY particles
    included (the first appear after about 250 steps); the driver seeds the
    reference's restart count."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "box_2d", "--precision", "fp64", "--steps", "1", "--out",
                        str(tmp_path / "a"), "--lset-restart"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rst = str(tmp_path / "a" / "rstfile" / "levelset.rst")
    r = subprocess.run([binary, "--load-lset-restart", rst, "--kernel", "hyperbolic", "--h-over-dx", "1.0",
                        "--precision", "fp64", "--steps", "300", "--output-every", "300", "--out",
                        str(tmp_path / "b")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    case = cases.from_lset_restart(rst, kernel="hyperbolic", h_over_dx=1.0, precision="fp64")
    assert d["n_particles"] == case.n_particles and d["step"] == 300 and d["flags"] & ~8 == 0
    g = SPHMeshGeneration(case, precision="fp64")
    g.Initialize_case()
    g.SPH_run_mesh_generation(300)
    gp = g.particles(("xyz", "type"))
    g.close()
    cpp = io.read_pst(str(tmp_path / "b" / "rstfile_particles" / "step_300_rank_0.pst"))
    assert np.max(np.abs(cpp - gp["xyz"])) < 1e-12
    assert (gp["type"] == 2).any()


def test_cpp_driver_writes_tet_mesh(tmp_path):
    """--mesh in 3D: Mesh_binary_writer's tet branch writes
    outdata/mesh_tets_rank_0_step_0.vtu (VTK_TETRA cells with 'vol',
    'aspect', 'radius_ratio', 'mindihedangle') and the JSON line carries the
    tet count and quality of SPH_mesh_generation::Reconstruct_tets."""
    binary = build.build_host()
    r = subprocess.run([binary, "--case", "box_3d", "--precision", "fp64", "--steps", "50", "--out", str(tmp_path),
                        "--mesh"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout)
    t = d["tets"]
    assert t["ntet"] > 3 * d["n_particles"] and t["total_volume"] > 0 and t["max_aspect"] >= t["avg_aspect"] > 1
    v = io.read_vtu(str(tmp_path / "outdata" / "mesh_tets_rank_0_step_0.vtu"))
    assert len(v["types"]) == t["ntet"] and set(np.unique(v["types"])) == {10}
    assert len(v["connectivity"]) == 4 * t["ntet"] and v["connectivity"].max() < d["n_particles"]
    for k in ("vol", "aspect", "radius_ratio", "mindihedangle"):
        assert np.all(np.isfinite(v[k])) and len(v[k]) == t["ntet"], k
    assert abs(float(v["vol"].astype(np.float64).sum()) - t["total_volume"]) < 1e-5 * t["total_volume"]
    assert (tmp_path / "outdata" / "mesh_tets.pvd").exists()
