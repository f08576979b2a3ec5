"""GPU parity: the CUDA engine (through the C ABI) against the FP64 oracle.

Bars (from the project's correctness contract):
  * FP64-plain: cell binning and neighbour sets bit-exact given identical
    positions; level-set fields bit-exact; single-step densities, forces and
    time steps within 1e-12 relative.
  * FP32-split: cell binning and neighbour sets bit-exact given identical
    positions (the FP32 decisions are re-made in FP64 inside their error
    bands); kernel sums of REAL and SURFACE particles, both force stages and
    both time steps within 1e-5, each normalised by the largest magnitude of
    its field over the particles compared (max |gpu - oracle| / max |oracle|);
    positions within 1e-5 of the local spacing after the map phase.
"""
import numpy as np
import pytest

import oracle
from mrsph import _lib as L
from paritylib import (gpu_post_map_to_oracle, make_gpu, neighbor_sets, oracle_state_to_gpu, rel_err,
                       small_cases, warm_oracle)

pytestmark = pytest.mark.gpu

CASES = small_cases()


@pytest.fixture(scope="module", params=sorted(CASES))
def warmed(request):
    case = CASES[request.param]()
    orc = warm_oracle(case)
    return request.param, case, orc.get_state()


@pytest.mark.parametrize("name", sorted(CASES))
def test_levelset_build_matches_oracle(name):
    case = CASES[name]()
    orc = oracle.Oracle(case)
    gpu = make_gpu(case, "fp64")
    for l in range(len(case.levels)):
        g = gpu.levelset_fields(l)
        f = orc.fields[l]
        shp = g["nx"].shape
        for k in ("nx", "ny", "nz"):
            assert np.array_equal(g[k].ravel(), f[k]), f"{k} level {l}"
        assert np.array_equal(g["tag"].ravel().astype(np.int32), f["tag"]), f"tag level {l}"
        assert rel_err(g["curv"].ravel(), f["curv"]) < 1e-12
        assert shp == case.levels[l].phi.shape
    assert g["max_phi"] == orc.ctx.max_phi
    gpu.close()


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_levelset_sampling(name, prec):
    case = CASES[name]()
    orc = oracle.Oracle(case)
    gpu = make_gpu(case, prec)
    rng = np.random.default_rng(5)
    p = case.params
    lo = np.array(p["box_l"])
    hi = np.array(p["box_r"])
    pts = lo + rng.random((4000, 3)) * (hi - lo)
    if p["dim"] == 2:
        pts[:, 2] = 0.0
    phi, nrm, curv, tag = gpu.sample_levelset(pts)
    rphi, rnrm, rcurv, rtag = orc.sample(pts)
    tol = 1e-13 if prec == "fp64" else 1e-5 * orc.ctx.max_phi
    assert np.max(np.abs(phi - rphi)) <= tol
    assert np.max(np.abs(nrm - rnrm)) <= (1e-13 if prec == "fp64" else 1e-5)
    assert np.array_equal(tag, rtag)
    gpu.close()


def _gpu_step_taps(case, prec, st, cap=0):
    gpu = make_gpu(case, prec, cap)
    gpu.set_state(oracle_state_to_gpu(st))
    gpu.run_phase(L.PHASE_FORCE2)
    gp = gpu.particles()
    lc, ids = gpu.cells()
    off, nb = gpu.neighbors()
    stats = gpu.stats()
    gpu.close()
    return gp, lc, ids, off, nb, stats


def test_fp64_step_phase_parity(warmed):
    name, case, st = warmed
    gp, lc, ids, off, nb, stats = _gpu_step_taps(case, "fp64", st)
    # map phase from the same injected state
    orc = oracle.Oracle(case)
    orc.set_state(st)
    orc.phase_map(advect=True)
    ost = orc.get_state()
    oxyz = np.stack([ost["x"], ost["y"], ost["z"]], axis=1)
    assert np.array_equal(gp["type"], ost["type"])
    assert np.array_equal(gp["level"], ost["level"])
    assert np.max(np.abs(gp["xyz"] - oxyz)) < 1e-12
    assert rel_err(gp["h"], ost["h"]) < 1e-12
    assert rel_err(gp["phi"], ost["phi"]) < 1e-12
    assert np.max(np.abs(gp["norm"] - np.stack([ost["nx"], ost["ny"], ost["nz"]], 1))) < 1e-12
    # binning + neighbours bit-exact from the GPU's own post-map state
    o2 = oracle.Oracle(case)
    gpu_post_map_to_oracle(o2, gp, st)
    oc = o2.cells()
    assert np.array_equal(lc, oc), "cell binning differs"
    # storage order: levels, then half cells (dcell / 2) row-major, ids ascending
    # inside a half cell; half-cell keys recomputed on the host from the GPU
    # positions exactly as the engine bins them
    lv = o2.levels()
    dim = case.params["dim"]
    box_l = np.array(case.params["box_l"])
    hoff = [0]
    for L in range(lv["ncl"]):
        hoff.append(hoff[-1] + int(np.prod([2 * lv["ncell"][L][d] for d in range(dim)])))
    key = np.zeros(len(ids), dtype=np.int64)
    for a, i in enumerate(ids):
        L = int(lc[i][0])
        k = 0
        for d in (2, 1, 0):
            hn = 2 * lv["ncell"][L][d] if d < dim else 1
            hq = 0
            if d < dim:
                hq = int(np.floor((gp["xyz"][i][d] - box_l[d]) / (0.5 * lv["dcell"][L][d])))
                hq = min(max(hq, 0), hn - 1)
                assert hq >> 1 == lc[i][1 + d]
            k = k * hn + hq
        key[a] = hoff[L] + k
    assert np.all(np.diff(key) >= 0), "storage order is not grouped by half cell"
    same = np.diff(key) == 0
    assert np.all(np.diff(ids)[same] > 0), "ids not ascending inside a half cell"
    ooff, onb = o2.neighbors()
    assert np.array_equal(off, ooff), "neighbour counts differ"
    assert np.array_equal(nb, onb), "neighbour sets differ"
    assert stats["pairs"] == len(onb) - len(off) + 1
    # density and the two force stages on identical inputs
    o2.density(ooff, onb)
    s = o2.get_state()
    assert rel_err(gp["sum"], s["sum"]) < 1e-12
    o2.force(ooff, onb, 1)
    s1 = o2.get_state()
    a1 = np.stack([s1["ax"], s1["ay"], s1["az"]], 1)
    assert rel_err(gp["a1"], a1) < 1e-12
    assert abs(stats["dt_stage1"] - s1["dt"]) <= 1e-12 * s1["dt"]
    o2.force(ooff, onb, 2)
    s2 = o2.get_state()
    a2 = np.stack([s2["ax"], s2["ay"], s2["az"]], 1)
    assert rel_err(gp["a2"], a2, floor=1e-300) < 1e-12
    assert abs(stats["dt"] - s2["dt"]) <= 1e-12 * s2["dt"]
    assert abs(stats["max_v"] - s2["max_v"]) <= 1e-12 * max(s2["max_v"], 1e-300)
    assert rel_err(gp["nu"], s2["nu"]) < 1e-12
    v = np.stack([s2["vx"], s2["vy"], s2["vz"]], 1)
    assert rel_err(gp["v"], v) < 1e-12


def check_fp32_single_step(case, st, cap=0):
    """One FP32-split step from the injected state st; the oracle redoes
    binning, neighbour search, density and both force stages on the GPU's own
    post-map state.  Returns the errors."""
    gp, lc, ids, off, nb, stats = _gpu_step_taps(case, "fp32", st, cap)
    o2 = oracle.Oracle(case)
    gpu_post_map_to_oracle(o2, gp, st)
    assert np.array_equal(lc, o2.cells()), "FP32-split cell binning differs"
    ooff, onb = o2.neighbors()
    assert np.array_equal(off, ooff), "FP32-split neighbour counts differ"
    assert np.array_equal(nb, onb), "FP32-split neighbour sets differ"
    assert stats["pairs"] == len(onb) - len(off) + 1
    o2.density(ooff, onb)
    s = o2.get_state()
    real = gp["type"] == 0
    surf = gp["type"] == 1
    err = {"sum_real": rel_err(gp["sum"][real], s["sum"][real]),
           "sum_surface": rel_err(gp["sum"][surf], s["sum"][surf]) if surf.any() else 0.0,
           "n_surface": int(surf.sum())}
    o2.force(ooff, onb, 1)
    s1 = o2.get_state()
    err["a1"] = rel_err(gp["a1"], np.stack([s1["ax"], s1["ay"], s1["az"]], 1))
    err["dt1"] = abs(stats["dt_stage1"] - s1["dt"]) / s1["dt"]
    o2.force(ooff, onb, 2)
    s2 = o2.get_state()
    err["a2"] = rel_err(gp["a2"], np.stack([s2["ax"], s2["ay"], s2["az"]], 1), floor=1e-300)
    err["dt2"] = abs(stats["dt"] - s2["dt"]) / s2["dt"]
    print("fp32 single-step errors", case.name, err)
    for k in ("sum_real", "sum_surface", "a1", "dt1", "a2", "dt2"):
        assert err[k] < 1e-5, (k, err)
    return err, gp


def test_fp32_step_phase_parity(warmed):
    name, case, st = warmed
    err, gp = check_fp32_single_step(case, st)
    dx = case.params["min_dl"]
    orc = oracle.Oracle(case)
    orc.set_state(st)
    orc.phase_map(advect=True)
    ost = orc.get_state()
    oxyz = np.stack([ost["x"], ost["y"], ost["z"]], axis=1)
    same = gp["type"] == ost["type"]
    assert same.mean() > 0.999
    assert np.max(np.abs(gp["xyz"][same] - oxyz[same])) < 1e-5 * dx


def test_fp32_surface_parity_hyperbolic_disc():
    """SURFACE particles with a non-zero surface kernel (the hyperbolic 1D
    kernel; the Wendland 1D kernel is the reference's zero): the disc after
    30 oracle steps."""
    case = CASES["disc2d_hyperbolic"]()
    orc = warm_oracle(case, max_steps=0, need_surface=False)
    orc.steps(30)
    err, gp = check_fp32_single_step(case, orc.get_state())
    assert err["n_surface"] > 20
    assert np.any(gp["sum"][gp["type"] == 1] != 0.0)


def test_fp32_surface_parity_torus():
    """A 37,658-particle torus after 100 oracle steps (thousands of SURFACE
    particles, three cell-list levels)."""
    from mrsph import cases
    case = cases.torus_3d(dx_min=0.02, dx_max=0.08)
    orc = warm_oracle(case, max_steps=0, need_surface=False)
    orc.steps(100)
    err, gp = check_fp32_single_step(case, orc.get_state(), cap=1024)
    assert err["n_surface"] > 1000


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_multistep_statistics(prec):
    """20 relaxation steps from identical seeds: median and minimum
    nearest-neighbour spacing and the surface count within 1%."""
    case = CASES["disc2d_wendland"]()
    orc = warm_oracle(case, max_steps=0, need_surface=False)
    st = orc.get_state()
    gpu = make_gpu(case, prec)
    gpu.set_state(oracle_state_to_gpu(st))
    gpu.SPH_run_mesh_generation(20)
    gpu.sync()
    orc.steps(20)
    gp = gpu.particles(("xyz", "type", "h"))
    os_ = orc.get_state()
    oxyz = np.stack([os_["x"], os_["y"], os_["z"]], 1)
    from scipy.spatial import cKDTree
    def stats(x):
        d, _ = cKDTree(x[:, :2]).query(x[:, :2], k=2)
        return d[:, 1].min(), np.median(d[:, 1])
    gmin, gmed = stats(gp["xyz"])
    omin, omed = stats(oxyz)
    assert abs(gmed - omed) <= 0.01 * omed
    assert abs(gmin - omin) <= 0.01 * omin
    assert abs((gp["type"] == 1).sum() - (os_["type"] == 1).sum()) <= 0.01 * len(gp["type"]) + 2
    s = gpu.stats()
    assert s["step"] == 20
    assert s["flags"] & ~L.FLAG_NEIGHBOR_SPILL == 0
    gpu.close()


@pytest.mark.parametrize("name", ["disc2d_hyperbolic", "spheres3d_curvature"])
def test_seed_matches_oracle_fp64(name):
    """Seeding + pre-run: the acceptance test phi > h runs the spacing law
    (the curvature law for the spheres), so positions match only if it does."""
    case = CASES[name]()
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    o = orc.get_state()
    gpu = make_gpu(case, "fp64")
    gpu.Initialize_case(case.n_particles)
    gp = gpu.particles(("xyz", "type", "h"))
    oxyz = np.stack([o["x"], o["y"], o["z"]], 1)
    assert np.max(np.abs(gp["xyz"] - oxyz)) < 1e-12
    assert np.array_equal(gp["type"], o["type"])
    gpu.close()


@pytest.mark.parametrize("kernel", ["hyperbolic", "cubic", "wendland", "gaussian", "quintic"])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_all_kernels_single_step(kernel, dim, prec):
    """Density sums and both force stages for every smoothing kernel
    (particle.cpp:31-807), 2D and 3D, from the GPU's own post-map state."""
    from mrsph import cases
    if dim == 2:
        case = cases.disc_hole_2d(spacing=0.02, grid=64, kernel=kernel)
    else:
        case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2, kernel=kernel)
    orc = warm_oracle(case, max_steps=2, need_surface=False)
    st = orc.get_state()
    if prec == "fp32":
        check_fp32_single_step(case, st, cap=2048 if dim == 3 else 0)
        return
    gp, lc, ids, off, nb, stats = _gpu_step_taps(case, prec, st, cap=2048 if dim == 3 else 0)
    o2 = oracle.Oracle(case)
    gpu_post_map_to_oracle(o2, gp, st)
    ooff, onb = o2.neighbors()
    assert np.array_equal(off, ooff) and np.array_equal(nb, onb)
    o2.density(ooff, onb)
    s = o2.get_state()
    assert rel_err(gp["sum"], s["sum"]) < 1e-12
    o2.force(ooff, onb, 1)
    s1 = o2.get_state()
    assert rel_err(gp["a1"], np.stack([s1["ax"], s1["ay"], s1["az"]], 1)) < 1e-12
    o2.force(ooff, onb, 2)
    s2 = o2.get_state()
    assert rel_err(gp["a2"], np.stack([s2["ax"], s2["ay"], s2["az"]], 1), floor=1e-300) < 1e-12


def test_map_only_phases_then_steps():
    """mrsph_run_phase(MAP) stops before the sort: the next steps still bin
    every particle once (storage order a permutation, symmetric neighbour
    sets, no device flags)."""
    case = CASES["disc2d_wendland"]()
    gpu = make_gpu(case, "fp64")
    gpu.Initialize_case()
    gpu.run_phase(L.PHASE_MAP)
    gpu.run_phase(L.PHASE_MAP)
    gpu.SPH_run_mesh_generation(3)
    gpu.sync()
    lc, ids = gpu.cells()
    assert np.array_equal(np.sort(ids), np.arange(gpu.n))
    off, nb = gpu.neighbors()
    sets = neighbor_sets(off, nb)
    for i in range(0, gpu.n, 5):
        for j in sets[i]:
            assert i in sets[j]
    assert gpu.stats()["flags"] & ~L.FLAG_NEIGHBOR_SPILL == 0
    gpu.close()
