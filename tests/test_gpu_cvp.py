"""GPU CVP partitioning (row A13) against the FP64 oracle: assignment labels,
VP positions and VP masses bit-exact after every iteration count tested,
given identical points and initial VPs."""
import numpy as np
import pytest

import oracle
from mrsph import SPHMeshGeneration, cases
from paritylib import warm_oracle

pytestmark = pytest.mark.gpu


def _compare(gpu, dim, box_l, box_r, xyz, vp, iters, mass=None):
    gv, gl, gm, gr = gpu.partition_points(xyz, vp, mass=mass, max_iter=iters)
    ov, ol, om, orr = oracle.cvp(dim, box_l, box_r, xyz, vp, mass=mass, max_iter=iters)
    assert np.array_equal(gl, ol), f"labels differ at {np.count_nonzero(gl != ol)} points"
    assert np.array_equal(gv, ov), f"VP positions differ by {np.max(np.abs(gv - ov))}"
    assert np.array_equal(gm, om)
    assert gr["iterations"] == orr["iterations"] and gr["converged"] == orr["converged"]
    assert gr["error_max"] == orr["error_max"]
    return gv, gl, gm, gr


def test_cvp_square_quadrants():
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    gpu = SPHMeshGeneration(case, precision="fp64")
    g = (np.arange(100) + 0.5) / 100
    X, Y = np.meshgrid(g, g, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), 0 * X.ravel()], 1)
    rng = np.random.default_rng(0)
    vp = np.zeros((4, 3))
    vp[:, :2] = 0.3 + 0.4 * rng.random((4, 2))
    p = case.params  # mrsph_cvp_points partitions inside the handle's domain
    gv, gl, gm, gr = _compare(gpu, 2, p["box_l"], p["box_r"], xyz, vp, 400)
    assert gr["converged"] == 1
    assert gm.min() > 0.9 * 2500
    gpu.close()


def test_cvp_weighted_3d():
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    gpu = SPHMeshGeneration(case, precision="fp32")
    p = case.params
    rng = np.random.default_rng(3)
    lo, hi = np.array(p["box_l"]), np.array(p["box_r"])
    xyz = lo + rng.random((30000, 3)) * (hi - lo)
    mass = 0.5 + rng.random(30000)
    vp = lo + rng.random((24, 3)) * (hi - lo)
    _compare(gpu, 3, p["box_l"], p["box_r"], xyz, vp, 30, mass=mass)
    gpu.close()


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_cvp_of_relaxed_particles(prec):
    """mrsph_cvp on the handle's own particles == the oracle on the same positions."""
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    gpu = SPHMeshGeneration(case, precision=prec)
    gpu.Initialize_case()
    gpu.SPH_run_mesh_generation(5)
    xyz = gpu.particles(("xyz",))["xyz"]
    rng = np.random.default_rng(7)
    vp = xyz[rng.choice(len(xyz), 32, replace=False)].copy()
    gv, gl, gm, gr = gpu.Partitioning(vp, max_iter=50)
    p = case.params
    ov, ol, om, orr = oracle.cvp(3, p["box_l"], p["box_r"], xyz, vp, max_iter=50)
    assert np.array_equal(gl, ol)
    assert np.array_equal(gv, ov)
    assert gm.sum() == len(xyz)
    gpu.close()


def test_cvp_disconnected_points_with_empty_cells():
    """Points on a union of separated spheres: some cells lose all their
    points.  Labels, VP positions and masses still match the oracle bit for
    bit, and the partition does not collapse (an empty cell keeps its
    position instead of dividing by its zero mass)."""
    case = cases.spheres_3d(fine_pkg=16, nlevels=2, dx_min=0.012, middle_dl=0.03, dx_max=0.08)
    orc = warm_oracle(case, max_steps=5, need_surface=False)
    st = orc.get_state()
    xyz = np.stack([st["x"], st["y"], st["z"]], 1)
    rng = np.random.default_rng(0)
    vp = xyz[rng.choice(len(xyz), 64, replace=False)].copy()
    gpu = SPHMeshGeneration(case, precision="fp64")
    p = case.params
    gv, gl, gm, gr = _compare(gpu, 3, p["box_l"], p["box_r"], xyz, vp, 49)
    assert (gm == 0).any()
    assert np.isfinite(gv).all()
    assert gr["error_max"] < 5.0
    gpu.close()
