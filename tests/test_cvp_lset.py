"""Level-set partition with ghost VPs: Voronoi_lset::
Partitioning_for_initial_VP_distribution (CVP/voronoi_lset.cpp:824-889) with
Ghost_VP_generation (:250-308).

* The oracle's first iteration against a plain restatement.  The points
  start coloured by their nearest VP.  Every VP k > 0 holding a point with
  surface mass is mirrored across the surface (x - 2 phi n at the VP), in VP
  order.  The points are then assigned among VPs and ghosts; a point nearest
  a ghost belongs to no VP.  Finally the VP masses are summed.
* The GPU (mrsph_cvp_lset) against the oracle, bit for bit: VP positions,
  labels, masses, ghosts and iteration counts, in 2D and 3D.
"""
import numpy as np
import pytest

import oracle
from mrsph import cases


def _packages(case, orc, level=0):
    """Package centres with total / surface mass (Calculate_volume_mass,
    lset_package.cpp:1283-1397) from the oracle's cut-cell pass; the same
    formulas as SPHMeshGeneration.lset_packages."""
    from mrsph.io import cell_scale
    lv = case.levels[level]
    dim = case.params["dim"]
    shp = lv.phi.shape
    vm = orc.volume_mass(level)

    class Sim:
        pass
    sim = Sim()
    sim.case = case
    sim.levelset_fields = lambda l: {"max_phi": orc.ctx.max_phi,
                                     "curv": orc.fields[l]["curv"].reshape(case.levels[l].phi.shape),
                                     "tag": orc.fields[l]["tag"].reshape(case.levels[l].phi.shape)}
    sc = cell_scale(sim, level)
    vol, area = vm["vol"].reshape(shp), vm["area"].reshape(shp)
    with np.errstate(divide="ignore", invalid="ignore"):
        cm = np.where(vol > 0, vol / sc ** dim, 0.0)
        cs = np.where(area > 0, area / sc ** (dim - 1), 0.0)
    m = lv.margin
    npk = [lv.num_pkg[d] + 2 * m if d < dim else 1 for d in range(3)]
    cz = 4 if dim == 3 else 1

    def per_pkg(a):
        return a.reshape(npk[2], cz, npk[1], 4, npk[0], 4).sum(axis=(1, 3, 5))
    sl = (slice(m, -m) if dim == 3 else slice(None), slice(m, -m), slice(m, -m))
    pm, ps = per_pkg(cm)[sl], per_pkg(cs)[sl]
    idx = np.stack(np.meshgrid(*[np.arange(pm.shape[a]) for a in range(3)], indexing="ij"), -1).reshape(-1, 3)
    cen = np.zeros((len(idx), 3))
    for d in range(dim):
        cen[:, d] = lv.box_l[d] + (idx[:, 2 - d] + 0.5) * lv.dpkg[d]
    keep = pm.ravel() > 0
    return cen[keep], pm.ravel()[keep], ps.ravel()[keep]


CASES = {
    "disc2d": (lambda: cases.disc_hole_2d(spacing=0.02, grid=64), 8, 200),
    "torus3d": (lambda: cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2), 16, 120),
}


def _dist(dim, a, b):
    s = 0.0
    s += (a[0] - b[0]) * (a[0] - b[0])
    s += (a[1] - b[1]) * (a[1] - b[1])
    if dim == 3:
        s += (a[2] - b[2]) * (a[2] - b[2])
    return np.sqrt(s)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_ghost_iteration_restated(name):
    mk, K, _ = CASES[name]
    case = mk()
    dim = case.params["dim"]
    orc = oracle.Oracle(case)
    xyz, mass, msurf = _packages(case, orc)
    rng = np.random.default_rng(11)
    vp0 = xyz[rng.choice(len(xyz), K, replace=False)].copy()
    vp, lab, vmass, res = orc.cvp_lset(xyz, mass, msurf, vp0, max_iter=0)

    def nearest(x, pts):
        best, idx = 1.e20, 0
        for k, p in enumerate(pts):
            d = _dist(dim, x, p)
            if d < best:
                best, idx = d, k
        return idx
    lab0 = [nearest(x, vp0) for x in xyz]
    flag = np.zeros(K, dtype=bool)
    for l, s in zip(lab0, msurf):
        if l > 0 and s > 0:
            flag[l] = True
    ghosts = []
    for k in range(K):
        if not flag[k]:
            continue
        phi, nrm, _, _ = orc.sample(vp0[k:k + 1])
        if phi[0] >= 1.e-6:
            ghosts.append([vp0[k, q] - 2. * phi[0] * nrm[0, q] if q < dim else vp0[k, q] for q in range(3)])
    ghosts = np.array(ghosts).reshape(-1, 3)
    assert len(ghosts) > 0
    assert np.array_equal(res["ghosts"], ghosts)
    pts = np.concatenate([vp0, ghosts])
    want = np.array([(lambda i: i if i < K else -1)(nearest(x, pts)) for x in xyz])
    assert np.array_equal(lab, want)
    assert (lab < 0).any()
    ms = np.zeros(K)
    for i in range(len(xyz)):
        if want[i] >= 0:
            ms[want[i]] += mass[i]
    assert np.allclose(vmass, ms, rtol=1e-12, atol=0.0)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_cvp_lset_matches_oracle(name):
    from paritylib import make_gpu
    mk, K, iters = CASES[name]
    case = mk()
    orc = oracle.Oracle(case)
    xyz, mass, msurf = _packages(case, orc)
    rng = np.random.default_rng(5)
    vp0 = xyz[rng.choice(len(xyz), K, replace=False)].copy()
    ov, ol, om, ores = orc.cvp_lset(xyz, mass, msurf, vp0, max_iter=iters)
    gpu = make_gpu(case, "fp64")
    gxyz, gmass, gsurf = gpu.lset_packages(0)
    assert np.array_equal(gxyz, xyz) and np.allclose(gmass, mass, rtol=1e-12) and np.array_equal(gsurf > 0, msurf > 0)
    gv, gl, gm, gres = gpu.partition_lset(xyz, mass, msurf, vp0, max_iter=iters)
    gpu.close()
    assert len(gres["ghosts"]) == len(ores["ghosts"]) > 0
    assert np.array_equal(gres["ghosts"], ores["ghosts"])
    assert np.array_equal(gl, ol), f"labels differ at {np.count_nonzero(gl != ol)} points"
    assert (gl < 0).any()
    assert np.array_equal(gv, ov)
    assert np.array_equal(gm, om)
    assert gres["iterations"] == ores["iterations"]
