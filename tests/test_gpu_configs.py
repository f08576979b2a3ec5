"""The benchmark configurations at their own sizes against the FP64 oracle.

* The 2D disc-hole configuration exactly (8,745 particles, 256^2 level set,
  dx 0.01, Wendland C2, FP64, 200 steps): every step the oracle's state is
  injected, one GPU step runs, and binning and neighbour sets (bit-exact),
  kernel sums, both force stages, time steps and velocities (1e-12) are
  compared with the oracle's on the GPU's post-map state; then both relax
  200 steps from one seed and their spacing statistics agree within 1%.
* CVP with 256 cells and 50 iterations (the sphere union's partition) on a
  relaxed 182,785-particle sphere union: labels, VP positions and masses
  bit-exact.
* The triangulation of the full 64-ellipse workload (312,897 particles) after
  its 400 FP32-split steps: triangle list bit-exact.
* FP32-split against the oracle over 100 steps from one seed on a
  37,658-particle torus: spacing percentiles and histogram, minimum pair
  distance, surface count and surface deviation within 1%.
"""
import numpy as np
import pytest

import oracle
from mrsph import SPHMeshGeneration, cases
from mrsph import _lib as L
from paritylib import gpu_post_map_to_oracle, make_gpu, oracle_state_to_gpu, rel_err

pytestmark = pytest.mark.gpu


def _spacing(xyz, h, hdx, dim, type_=None, phi=None):
    from scipy.spatial import cKDTree
    pts = xyz[:, :dim]
    d, _ = cKDTree(pts).query(pts, k=2)
    r = d[:, 1] / (h / hdx)
    out = {"median": float(np.median(r)), "p05": float(np.percentile(r, 5)), "p95": float(np.percentile(r, 95)),
           "min_distance": float(d[:, 1].min()), "hist": np.histogram(r, bins=40, range=(0.0, 2.0))[0]}
    if type_ is not None:
        surf = type_ == 1
        out["surface_count"] = int(surf.sum())
        out["surface_dev_mean"] = float(np.mean(np.abs(phi[surf]) / (h[surf] / hdx))) if surf.any() else 0.0
    return out


def test_disc_hole_2d_config_stepwise():
    case = cases.disc_hole_2d()
    assert case.n_particles == 8745
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    seed_state = orc.get_state()
    gpu = make_gpu(case, "fp64")
    o2 = oracle.Oracle(case)
    for step in range(200):
        st = orc.get_state()
        gpu.set_state(oracle_state_to_gpu(st))
        gpu.run_phase(L.PHASE_FORCE2)
        gp = gpu.particles()
        lc, _ = gpu.cells()
        off, nb = gpu.neighbors()
        stats = gpu.stats()
        gpu_post_map_to_oracle(o2, gp, st)
        assert np.array_equal(lc, o2.cells()), f"binning differs at step {step}"
        ooff, onb = o2.neighbors()
        assert np.array_equal(off, ooff) and np.array_equal(nb, onb), f"neighbour sets differ at step {step}"
        o2.density(ooff, onb)
        s0 = o2.get_state()
        assert rel_err(gp["sum"], s0["sum"]) < 1e-12, step
        o2.force(ooff, onb, 1)
        s1 = o2.get_state()
        assert rel_err(gp["a1"], np.stack([s1["ax"], s1["ay"], s1["az"]], 1)) < 1e-12, step
        assert abs(stats["dt_stage1"] - s1["dt"]) <= 1e-12 * s1["dt"], step
        o2.force(ooff, onb, 2)
        s2 = o2.get_state()
        assert rel_err(gp["a2"], np.stack([s2["ax"], s2["ay"], s2["az"]], 1), floor=1e-300) < 1e-12, step
        assert abs(stats["dt"] - s2["dt"]) <= 1e-12 * s2["dt"], step
        assert rel_err(gp["v"], np.stack([s2["vx"], s2["vy"], s2["vz"]], 1), floor=1e-300) < 1e-12, step
        orc.steps(1)
    # 200 free-running steps from the seed on both sides
    gpu.set_state(oracle_state_to_gpu(seed_state))
    gpu.SPH_run_mesh_generation(200)
    gpu.sync()
    g = gpu.particles(("xyz", "h", "type", "phi"))
    assert gpu.stats()["flags"] & ~L.FLAG_NEIGHBOR_SPILL == 0
    gpu.close()
    ref = oracle.Oracle(case)
    ref.set_state(seed_state)
    ref.steps(200)
    o = ref.get_state()
    hdx = case.params["cell_ratio"] / case.params["cutoff"]
    gs = _spacing(g["xyz"], g["h"], hdx, 2, g["type"], g["phi"])
    os_ = _spacing(np.stack([o["x"], o["y"], o["z"]], 1), o["h"], hdx, 2, o["type"], o["phi"])
    for k in ("median", "p05", "p95", "min_distance", "surface_count"):
        assert abs(gs[k] - os_[k]) <= 0.01 * abs(os_[k]), (k, gs[k], os_[k])
    assert np.abs(gs["hist"] - os_["hist"]).sum() <= 0.01 * case.n_particles


def test_cvp_256_cells_50_iterations_sphere_union():
    case = cases.spheres_3d(fine_pkg=32, nlevels=2, dx_min=0.006, middle_dl=0.01, dx_max=0.03)
    gpu = SPHMeshGeneration(case, precision="fp32")
    gpu.Initialize_case()
    gpu.SPH_run_mesh_generation(20)
    xyz = gpu.particles(("xyz",))["xyz"]
    assert len(xyz) >= 100000
    rng = np.random.default_rng(7)
    vp = xyz[rng.choice(len(xyz), 256, replace=False)].copy()
    gv, gl, gm, gr = gpu.Partitioning(vp, max_iter=50)
    p = case.params
    ov, ol, om, orr = oracle.cvp(3, p["box_l"], p["box_r"], xyz, vp, max_iter=50)
    assert np.array_equal(gl, ol), f"labels differ at {np.count_nonzero(gl != ol)} points"
    assert np.array_equal(gv, ov)
    assert np.array_equal(gm, om)
    assert gr["iterations"] == orr["iterations"]
    gpu.close()


def test_triangulation_full_ellipses_after_400_steps():
    case = cases.ellipses_2d()
    assert case.n_particles == 312897
    gpu = make_gpu(case, "fp32", cap=256)
    gpu.Initialize_case()
    gpu.SPH_run_mesh_generation(400)
    gt, gq = gpu.Reconstruct_tris()
    p = gpu.particles(("xyz", "type", "phi"))
    off, nb = gpu.neighbors()
    ot, oq = oracle.Oracle(case).triangulate(p["xyz"], p["type"], p["phi"], off, nb)
    assert gt.shape == ot.shape
    assert np.array_equal(gt, ot)
    for k in ("ntri", "nedge", "nedge_first", "ndeleted", "nerror"):
        assert gq[k] == oq[k], k
    assert list(gq["hist"]) == list(oq["hist"])
    assert gq["ntri"] > gpu.n
    gpu.close()


def test_fp32_relaxation_statistics_against_oracle_torus():
    case = cases.torus_3d(dx_min=0.02, dx_max=0.08)
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    seed_state = orc.get_state()
    orc.steps(100)
    o = orc.get_state()
    gpu = SPHMeshGeneration(case, precision="fp32", neighbor_cap=1024)
    gpu.set_state(oracle_state_to_gpu(seed_state))
    gpu.SPH_run_mesh_generation(100)
    gpu.sync()
    g = gpu.particles(("xyz", "h", "type", "phi"))
    assert gpu.stats()["flags"] & ~L.FLAG_NEIGHBOR_SPILL == 0
    gpu.close()
    hdx = case.params["cell_ratio"] / case.params["cutoff"]
    gs = _spacing(g["xyz"], g["h"], hdx, 3, g["type"], g["phi"])
    os_ = _spacing(np.stack([o["x"], o["y"], o["z"]], 1), o["h"], hdx, 3, o["type"], o["phi"])
    for k in ("median", "p05", "p95", "min_distance", "surface_count", "surface_dev_mean"):
        assert abs(gs[k] - os_[k]) <= 0.01 * abs(os_[k]), (k, gs[k], os_[k])
    assert np.abs(gs["hist"] - os_["hist"]).sum() <= 0.01 * case.n_particles
