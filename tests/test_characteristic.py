"""SINGULARITY and SEGMENT particles: the reference's characteristic cells.

The geometry is a box whose corners are singularity points and, in 3D,
whose 12 edges are segments (Levelset::singularity and ::segment,
level_set.h:37-41).

* Tags: Get_singularity_tag and Get_segment_tag (lset_package.cpp:515-585),
  together with is_Segment_intersec_AABB (:587-619).  The oracle's tags are
  checked against a plain-Python restatement on the CPU.  The GPU's tags are
  checked against the oracle's, bit-exact.
* Map: Find_and_map_particle (particle_mesh_generation.cpp:439-465) puts a
  particle in a SEGMENT cell onto the segment's line and a particle in a
  SINGULARITY cell onto the point.
* Kernel sums: :717-759.  A SURFACE particle also counts SEGMENT and
  SINGULARITY neighbours (no normal filter).  A SEGMENT particle in 3D counts
  SEGMENT neighbours (normal filter) and SINGULARITY neighbours with the 1D
  kernel.
* Forces: Accumulate_particle_force_seg, :769-879.  A SINGULARITY particle
  neither moves nor feels a force.
* Bars: FP64-plain on the GPU within 1e-12 of the oracle, step by step with
  the oracle's state injected every step.  FP32-split bit-exact in binning
  and neighbour sets, within 1e-5 in sums, forces and time steps.
"""
import itertools

import numpy as np
import pytest

import oracle
from mrsph import cases
from mrsph import _lib as L
from paritylib import gpu_post_map_to_oracle, make_gpu, oracle_state_to_gpu, rel_err

BOX_CASES = {
    "box2d": lambda: cases.box_with_corners(dim=2, spacing=0.02, grid=64, kernel="hyperbolic", h_over_dx=1.0),
    "box3d": lambda: cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic", h_over_dx=1.0),
}


def _restated_tags(lv, tag_flat, sing, seg, dim):
    """Characteristic tags of one level, restated in numpy from the
    reference's Get_singularity_tag / Get_segment_tag, encoded as
    mrsph_get_characteristics returns them (k + 1 on segment k, -(k + 1) at
    point k, 0 otherwise)."""
    m = lv.margin
    n = [4 * (lv.num_pkg[d] + 2 * m) if d < dim else 1 for d in range(3)]
    tag = np.asarray(tag_flat).reshape(n[2], n[1], n[0])
    out = np.zeros(tag.shape, dtype=np.int64)
    dc = [lv.dpkg[d] / 4.0 for d in range(3)]
    ks = range(4) if dim == 3 else range(1)
    pk_ranges = [range(lv.num_pkg[d]) if d < dim else range(1) for d in range(3)]

    def arr_index(pk, ce):
        g = [4 * pk[d] + ce[d] + 4 * m if d < dim else 0 for d in range(3)]
        return g[2], g[1], g[0]

    for ic, p in enumerate(sing):
        for pk in itertools.product(*pk_ranges):
            dr = [p[d] - (pk[d] * lv.dpkg[d] + lv.box_l[d]) for d in range(dim)]
            if not all(0.0 < dr[d] < lv.dpkg[d] + 1.e-10 for d in range(dim)):
                continue
            cand = []
            for ce in itertools.product(range(4), range(4), ks):
                a = arr_index(pk, ce)
                if tag[a] == 0:
                    continue
                cp = [(pk[d] * lv.dpkg[d] + (ce[d] + 0.5) * dc[d]) + lv.box_l[d] for d in range(dim)]
                cand.append((float(np.sqrt(sum((cp[d] - p[d]) ** 2 for d in range(dim)))), a))
            if cand:
                best = min(c[0] for c in cand)
                out[next(c[1] for c in cand if c[0] == best)] = -(ic + 1)
    if len(seg):
        # every interface cell that is not a singularity cell: its box
        # against each segment in order (is_Segment_intersec_AABB)
        zz, yy, xx = np.nonzero((tag != 0) & (out >= 0))
        g = [xx - 4 * m, yy - 4 * m, zz - 4 * m if dim == 3 else np.zeros_like(zz)]
        mn = np.zeros((len(xx), 3))
        for d in range(dim):
            pk, ce = np.floor_divide(g[d], 4), np.mod(g[d], 4)
            mn[:, d] = (pk * lv.dpkg[d] + ce * dc[d]) + lv.box_l[d]
        mx = mn.copy()
        for d in range(dim):
            mx[:, d] = mn[:, d] + dc[d]
        hit = np.zeros(len(xx), dtype=np.int64)
        for s_i, s in enumerate(seg):
            p1, p2 = np.asarray(s[:3]), np.asarray(s[3:])
            dd = (p2 - p1) * 0.5
            e = (mx - mn) * 0.5
            c = (p1 + dd) - (mx + mn) * 0.5
            ad = np.abs(dd)
            ok = np.all(np.abs(c) <= e + ad, axis=1)
            ok &= np.abs(dd[1] * c[:, 2] - dd[2] * c[:, 1]) <= e[:, 1] * ad[2] + e[:, 2] * ad[1] + 1.e-20
            ok &= np.abs(dd[2] * c[:, 0] - dd[0] * c[:, 2]) <= e[:, 2] * ad[0] + e[:, 0] * ad[2] + 1.e-20
            ok &= np.abs(dd[0] * c[:, 1] - dd[1] * c[:, 0]) <= e[:, 0] * ad[1] + e[:, 1] * ad[0] + 1.e-20
            new = ok & (hit == 0)
            hit[new] = s_i + 1
        out[zz, yy, xx] = hit
    return out.ravel()


def _oracle_encoded(f):
    chr_, idx = f["chr"], f["chr_idx"]
    return np.where(chr_ == 2, idx + 1, np.where(chr_ == 1, -(idx + 1), 0))


@pytest.mark.parametrize("name", sorted(BOX_CASES))
def test_oracle_characteristic_tags_restated(name):
    case = BOX_CASES[name]()
    orc = oracle.Oracle(case)
    dim = case.params["dim"]
    ch = orc.characteristics
    for l, lv in enumerate(case.levels):
        f = orc.fields[l]
        want = _restated_tags(lv, f["tag"], ch["singularities"], ch["segments"], dim)
        got = _oracle_encoded(f)
        assert np.array_equal(got, want)
        npts = len(ch["singularities"])
        assert np.count_nonzero(got < 0) == npts, "one singularity cell per point"
        if dim == 3:
            assert set(np.unique(got[got > 0])) == set(range(1, len(ch["segments"]) + 1)), "every edge tagged"


@pytest.mark.parametrize("name", sorted(BOX_CASES))
def test_oracle_characteristic_particles(name):
    """After relaxation the oracle holds SINGULARITY particles exactly at
    corners and SEGMENT particles on the edges (dispersed by 1e-5 h)."""
    case = BOX_CASES[name]()
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    orc.steps(300)
    st = orc.get_state()
    dim = case.params["dim"]
    xyz = np.stack([st["x"], st["y"], st["z"]], 1)
    corners = orc.characteristics["singularities"]
    sing = st["type"] == 2
    assert sing.any()
    for p in xyz[sing]:
        assert np.min(np.max(np.abs(corners[:, :dim] - p[:dim]), axis=1)) == 0.0
    seg = st["type"] == 3
    if dim == 3:
        assert seg.sum() > 50
        segs = orc.characteristics["segments"]
        for p, h in zip(xyz[seg], st["h"][seg]):
            d = []
            for s in segs:
                a, b = s[:3], s[3:]
                t = np.clip(np.dot(p - a, b - a) / np.dot(b - a, b - a), 0.0, 1.0)
                d.append(np.linalg.norm(a + t * (b - a) - p))
            assert min(d) <= 1.0001e-5 * h
    else:
        assert not seg.any()


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(BOX_CASES))
def test_gpu_characteristic_tags(name):
    case = BOX_CASES[name]()
    orc = oracle.Oracle(case)
    gpu = make_gpu(case, "fp64")
    for l in range(len(case.levels)):
        assert np.array_equal(gpu.characteristic_tags(l).ravel(), _oracle_encoded(orc.fields[l]))
    gpu.close()


def _compare_step(gpu, case, st, o2, o3, prec):
    """One GPU step from the oracle's state st against the oracle: the map
    phase from st (o3), then binning, neighbours, sums, forces from the
    GPU's post-map state (o2)."""
    gpu.set_state(oracle_state_to_gpu(st))
    gpu.run_phase(L.PHASE_FORCE2)
    gp = gpu.particles()
    lc, _ = gpu.cells()
    off, nb = gpu.neighbors()
    stats = gpu.stats()
    o3.set_state(st)
    o3.phase_map(advect=True)
    m = o3.get_state()
    oxyz = np.stack([m["x"], m["y"], m["z"]], 1)
    tol_x = 1e-12 if prec == "fp64" else 1e-5 * case.params["min_dl"]
    tol = 1e-12 if prec == "fp64" else 1e-5
    if prec == "fp64":
        assert np.array_equal(gp["type"], m["type"]), "types after the map phase"
        same = np.ones(len(m["type"]), dtype=bool)
    else:
        # FP32 positions after advection differ from the oracle's by about
        # 1e-7 dx, so a particle that close to a cell face may take the other
        # cell's type; the later phases run on the GPU's own post-map state
        same = gp["type"] == m["type"]
        assert same.mean() > 0.999, "types after the map phase"
    assert np.max(np.abs(gp["xyz"][same] - oxyz[same])) <= tol_x
    gpu_post_map_to_oracle(o2, gp, st)
    assert np.array_equal(lc, o2.cells()), "binning"
    ooff, onb = o2.neighbors()
    assert np.array_equal(off, ooff) and np.array_equal(nb, onb), "neighbour sets"
    o2.density(ooff, onb)
    s0 = o2.get_state()
    for t in range(4):
        sel = gp["type"] == t
        if sel.any():
            assert rel_err(gp["sum"][sel], s0["sum"][sel]) <= tol, ("sum", t)
    o2.force(ooff, onb, 1)
    s1 = o2.get_state()
    assert rel_err(gp["a1"], np.stack([s1["ax"], s1["ay"], s1["az"]], 1)) <= tol, "a1"
    assert abs(stats["dt_stage1"] - s1["dt"]) <= tol * s1["dt"]
    o2.force(ooff, onb, 2)
    s2 = o2.get_state()
    assert rel_err(gp["a2"], np.stack([s2["ax"], s2["ay"], s2["az"]], 1), floor=1e-300) <= tol, "a2"
    assert abs(stats["dt"] - s2["dt"]) <= tol * s2["dt"]
    sing = gp["type"] == 2
    assert np.all(gp["a1"][sing] == 0.0) and np.all(gp["a2"][sing] == 0.0)
    return gp


@pytest.mark.gpu
@pytest.mark.parametrize("name,nsteps", [("box2d", 300), ("box3d", 150)])
def test_gpu_characteristic_stepwise_fp64(name, nsteps):
    """Every step for nsteps steps from the seed (particles reach the
    characteristic cells from about step 30 in 3D and step 150 in 2D): the
    oracle's state injected, one FP64 GPU step, compared phase by phase."""
    case = BOX_CASES[name]()
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    gpu = make_gpu(case, "fp64")
    o2, o3 = oracle.Oracle(case), oracle.Oracle(case)
    seen = np.zeros(4, dtype=np.int64)
    for step in range(nsteps):
        gp = _compare_step(gpu, case, orc.get_state(), o2, o3, "fp64")
        seen = np.maximum(seen, np.bincount(gp["type"], minlength=4))
        orc.steps(1)
    gpu.close()
    assert seen[1] > 0 and seen[2] > 0
    if case.params["dim"] == 3:
        assert seen[3] > 50


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(BOX_CASES))
def test_gpu_characteristic_fp32(name):
    """FP32-split, one step from the oracle's state after 300 steps."""
    case = BOX_CASES[name]()
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    orc.steps(300)
    gpu = make_gpu(case, "fp32")
    gp = _compare_step(gpu, case, orc.get_state(), oracle.Oracle(case), oracle.Oracle(case), "fp32")
    gpu.close()
    assert (gp["type"] == 2).any()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_characteristic_free_run(prec):
    """300 free-running steps from one seed on the 3D box: spacing
    statistics and the particle counts of every type within 1% (+2) of the
    oracle's, SINGULARITY particles exactly at corners, SEGMENT particles on
    the edges."""
    case = BOX_CASES["box3d"]()
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    seed = orc.get_state()
    gpu = make_gpu(case, prec)
    gpu.set_state(oracle_state_to_gpu(seed))
    gpu.SPH_run_mesh_generation(300)
    gpu.sync()
    g = gpu.particles(("xyz", "type", "h"))
    assert gpu.stats()["flags"] & ~L.FLAG_NEIGHBOR_SPILL == 0
    gpu.close()
    orc.steps(300)
    o = orc.get_state()
    gc = np.bincount(g["type"], minlength=4)
    oc = np.bincount(o["type"], minlength=4)
    assert np.all(np.abs(gc - oc) <= 0.01 * oc + 2), (gc, oc)
    from scipy.spatial import cKDTree
    oxyz = np.stack([o["x"], o["y"], o["z"]], 1)
    dg, _ = cKDTree(g["xyz"]).query(g["xyz"], k=2)
    do, _ = cKDTree(oxyz).query(oxyz, k=2)
    assert abs(np.median(dg[:, 1]) - np.median(do[:, 1])) <= 0.01 * np.median(do[:, 1])
    corners = orc.characteristics["singularities"]
    tol = 0.0 if prec == "fp64" else 1e-6
    for p in g["xyz"][g["type"] == 2]:
        assert np.min(np.max(np.abs(corners - p), axis=1)) <= tol
