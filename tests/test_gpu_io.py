"""Writers and restarts through a live GPU handle: the particle VTU, the
triangle-mesh VTU, the level-set VTI and the .pst restart read back equal to
the engine's state, and a restart loaded into a new handle reproduces the
positions."""
import numpy as np
import pytest

from mrsph import SPHMeshGeneration, cases, io

pytestmark = pytest.mark.gpu


def test_writers_and_restart_round_trip(tmp_path):
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    g = SPHMeshGeneration(case, precision="fp64")
    g.Initialize_case()
    g.SPH_run_mesh_generation(10)
    p = g.particles(("xyz", "type", "h", "norm"))
    off, _ = g.neighbors()
    f = io.ParticleWriter(str(tmp_path / "outdata")).Output_particle(0, g)
    r = io.read_vtu(f)
    assert np.array_equal(r["Position"], p["xyz"].astype(np.float32))
    assert np.array_equal(r["type"], p["type"])
    assert np.array_equal(r["h"], p["h"].astype(np.float32))
    assert np.array_equal(r["NN"], np.diff(off))
    assert np.array_equal(r["norm"], p["norm"].astype(np.float32))
    tris, q = g.Reconstruct_tris()
    m = io.read_vtu(io.MeshWriter(str(tmp_path / "outdata")).Output_mesh(0, g, tris=tris))
    assert np.array_equal(m["connectivity"].reshape(-1, 3), np.asarray(tris))
    assert len(m["vol"]) == len(tris) and np.all(m["aspect"] >= 1.0)
    lf = io.read_vtu(io.LevelSetWriter(str(tmp_path / "outdata")).Output_lset(0, g))
    f0 = g.levelset_fields(0)
    mm = 4 * case.levels[0].margin
    assert lf["interface"].sum() == (f0["tag"][0, mm:-mm, mm:-mm] == 1).sum() > 0
    assert np.allclose(lf["curv"], io.corner_average(f0["curv"], mm, 2).ravel().astype(np.float32))
    vm = g.volume_mass(0, cells=True)
    assert np.array_equal(lf["vol"], vm["vol"][0, mm:-mm, mm:-mm].ravel().astype(np.float32))
    assert np.array_equal(lf["area"], vm["area"][0, mm:-mm, mm:-mm].ravel().astype(np.float32))
    assert abs(float(lf["vol"].astype(np.float64).sum()) - vm["total_volume"]) < 1e-5 * vm["total_volume"]
    pst = io.save_particle_post_file(g, str(tmp_path), first=True)
    assert np.array_equal(io.read_pst(pst), p["xyz"])
    g.close()
    g2 = SPHMeshGeneration(case, precision="fp64")
    assert io.load_data_for_post(g2, pst, pre_run=False) == len(p["xyz"])
    assert np.array_equal(g2.particles(("xyz",))["xyz"], p["xyz"])
    g2.close()


def test_case_from_lset_restart_relaxes_like_its_writer(tmp_path):
    """A level-set restart written from a live handle and loaded back as a
    case (cases.from_lset_restart) relaxes the same particles, bit for bit,
    as the case that wrote it."""
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=1)
    g = SPHMeshGeneration(case, precision="fp32")
    path = io.save_lset_restart(g, str(tmp_path / "levelset.rst"))
    kern = {v: k for k, v in cases.KERNELS.items()}[case.params["kernel"]]
    c2 = cases.from_lset_restart(path, kernel=kern, h_over_dx=case.params["cell_ratio"] / 2,
                                 precision="fp32", scale_law=case.params.get("scale_law", 0))
    g2 = SPHMeshGeneration(c2, precision="fp32")
    out = []
    assert c2.n_particles == g.volume_mass(0)["num_particle"]
    for s in (g, g2):
        s.Initialize_case(case.n_particles)
        s.SPH_run_mesh_generation(20)
        out.append(s.particles(("xyz", "type", "h")))
        s.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
