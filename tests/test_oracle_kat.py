"""Known-answer tests of the FP64 oracle (CPU).  The reference ships no tests
or golden vectors, so the oracle is pinned to analytic identities of the
equations it restates."""
import numpy as np
import pytest
from scipy import integrate

import oracle
from mrsph import cases

PI_REF = 3.1415926


@pytest.mark.parametrize("kind", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("dim", [2, 3])
def test_kernel_normalisation(kind, dim):
    """Integral of W over its support is 1 up to the reference's truncated PI
    and its rounded coefficients (cubic 0.4547..., quintic 7/478)."""
    h = 0.7
    r = np.linspace(0.0, 3.0 * h, 200001)
    w = oracle.kernel_W(kind, dim, r, h)
    shell = 2 * np.pi * r if dim == 2 else 4 * np.pi * r * r
    total = integrate.simpson(w * shell, x=r)
    tol = {0: 1e-6, 1: 1e-3, 2: 1e-6, 3: 1e-3, 4: 4e-3}[kind]  # Gaussian truncated at 3h; quintic 3/359 rounded
    assert abs(total - np.pi / PI_REF) < tol


@pytest.mark.parametrize("kind", [0, 1, 2, 4])
def test_kernel_gradient_matches_derivative(kind):
    h = 0.5
    r = np.linspace(0.05, 1.9 * h, 400)
    eps = 1e-6
    for dim in (2, 3):
        w1 = oracle.kernel_W(kind, dim, r + eps, h)
        w0 = oracle.kernel_W(kind, dim, r - eps, h)
        fd = (w1 - w0) / (2 * eps)
        dw = oracle.kernel_dW(kind, dim, r, h) * r  # dW returns (dW/dr)/r
        assert np.max(np.abs(fd - dw)) < 1e-4 * np.max(np.abs(dw))


def test_wendland_1d_is_zero():
    """Reference quirk Q2: the Wendland kernel has no 1D form (returns 0)."""
    r = np.linspace(0, 1, 10)
    assert np.all(oracle.kernel_W(2, 1, r, 0.3) == 0)
    assert np.all(oracle.kernel_dW(2, 1, r, 0.3) == 0)


def test_philox_known_answers():
    """Philox4x32-10 test vectors published with the algorithm (Random123)."""
    assert oracle.philox(0, 0, 0, 0, 0) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle.philox(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFFFFFFFFFF) == \
        [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def _linear_case():
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    lv = case.levels[0]
    ax = cases.cell_centres(lv.box_l, lv.dpkg, lv.num_pkg, lv.margin, 2)
    Y, X = np.meshgrid(ax[1], ax[0], indexing="ij")
    lv.phi = (0.3 * X - 0.2 * Y + 0.1)[None, :, :].copy()
    return case


def test_bilinear_interpolation_exact_for_linear_phi():
    case = _linear_case()
    orc = oracle.Oracle(case)
    rng = np.random.default_rng(1)
    pts = np.zeros((500, 3))
    pts[:, :2] = 0.05 + 0.9 * rng.random((500, 2))
    phi, nrm, curv, tag = orc.sample(pts)
    assert np.max(np.abs(phi - (0.3 * pts[:, 0] - 0.2 * pts[:, 1] + 0.1))) < 1e-14
    n = np.array([0.3, -0.2]) / np.hypot(0.3, 0.2)
    assert np.max(np.abs(nrm[:, :2] - n)) < 1e-10


def test_projection_lands_on_zero_level():
    """A REAL particle in a cut cell of a circle is projected onto phi = 0
    (Find_and_map_particle) to within the interpolation error."""
    case = cases.disc_hole_2d(spacing=0.005, grid=256)
    orc = oracle.Oracle(case)
    rng = np.random.default_rng(2)
    ang = rng.random(200) * 2 * np.pi
    rad = 0.2 + (rng.random(200) - 0.5) * 0.002
    x = np.zeros(200)
    st = {"x": 0.5 + rad * np.cos(ang), "y": 0.5 + rad * np.sin(ang), "z": x, "h": np.full(200, 0.0065),
          "type": np.zeros(200, dtype=np.int32), "step": 0, "dt": 0.0}
    orc.set_state(st)
    orc.phase_map(advect=False)
    s = orc.get_state()
    surf = s["type"] == 1
    assert surf.sum() > 150
    r = np.hypot(s["x"][surf] - 0.5, s["y"][surf] - 0.5)
    assert np.max(np.abs(r - 0.2)) < 2e-4


def test_scale_law_endpoints():
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    orc = oracle.Oracle(case)
    mp = orc.ctx.max_phi
    assert abs(orc.get_scale(0.0) - 0.03) < 1e-15
    assert abs(orc.get_scale(mp) - 0.09) < 1e-12
    assert orc.get_scale(-1.0) == 0.03


def test_lattice_gradient_sum_vanishes():
    """On a perfect lattice with uniform h the stage-1 force of an interior
    particle is zero (antisymmetric gradient sum)."""
    case = cases.disc_hole_2d(spacing=0.01, grid=256, kernel="wendland")
    orc = oracle.Oracle(case)
    g = np.arange(0.1, 0.3, 0.01)
    X, Y = np.meshgrid(g, g, indexing="ij")
    n = X.size
    st = {"x": X.ravel(), "y": Y.ravel(), "z": np.zeros(n), "h": np.full(n, 0.013),
          "rho": np.full(n, 1e4), "type": np.zeros(n, dtype=np.int32), "step": 0, "dt": 0.0,
          "level": np.zeros(n, dtype=np.int32)}
    orc.set_state(st)
    off, nb = orc.neighbors()
    orc.density(off, nb)
    orc.force(off, nb, 1)
    s = orc.get_state()
    inner = (np.abs(X.ravel() - 0.195) < 0.05) & (np.abs(Y.ravel() - 0.195) < 0.05)
    a = np.hypot(s["ax"], s["ay"])
    assert np.max(a[inner]) < 1e-9 * np.max(np.abs(s["sum"])) * 1e3


def test_level_plan_restates_define_level_infor_tight():
    case = cases.torus_3d(dx_min=0.005, dx_max=0.02)
    orc = oracle.Oracle(case)
    lv = orc.levels()
    assert lv["ncl"] == 3
    for l in range(3):
        assert abs(lv["scale"][l] - lv["max_scale"] / 2 ** l) < 1e-10
    assert lv["ncell"][2] == [244, 244, 92]


def test_neighbor_relation_symmetric_and_includes_self():
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    for _ in range(40):  # relax until surface particles (finest spacing) appear
        orc.steps(1)
        if (orc.arrays["type"] == 1).sum() > 100:
            break
    off, nb = orc.neighbors()
    n = len(off) - 1
    sets = [set(nb[off[i]:off[i + 1]].tolist()) for i in range(n)]
    assert all(i in sets[i] for i in range(n))
    for i in range(0, n, 7):
        for j in sets[i]:
            assert i in sets[j]
    lev = orc.arrays["level"]
    assert len(set(lev.tolist())) >= 2  # adaptive: more than one cell-list level


def test_cvp_converges_to_quadrant_centroids():
    """Four VPs on a uniform grid of the unit square converge to the quadrant
    centroids with mass error below the tolerance (Voronoi::Partitioning)."""
    g = (np.arange(100) + 0.5) / 100
    X, Y = np.meshgrid(g, g, indexing="ij")
    xyz = np.stack([X.ravel(), Y.ravel(), 0 * X.ravel()], 1)
    rng = np.random.default_rng(0)
    vp = np.zeros((4, 3))
    vp[:, :2] = 0.3 + 0.4 * rng.random((4, 2))
    v, lab, m, r = oracle.cvp(2, [0, 0, 0], [1, 1, 0], xyz, vp, max_iter=400)
    assert r["converged"] == 1 and r["error_max"] <= 0.05
    for c in ([0.25, 0.25], [0.25, 0.75], [0.75, 0.25], [0.75, 0.75]):
        assert np.min(np.hypot(v[:, 0] - c[0], v[:, 1] - c[1])) < 0.03
    assert np.bincount(lab, minlength=4).min() > 2300


def test_triangulation_with_full_rows_is_delaunay():
    """With every point in every neighbour row, the local-Voronoi edges of the
    oracle are the Delaunay edges of the point set (checked against qhull),
    and every Delaunay triangle is a final triangle."""
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(5)
    n = 160
    xyz = np.zeros((n, 3))
    xyz[:, :2] = 0.1 + 0.8 * rng.random((n, 2))
    off = np.arange(n + 1, dtype=np.int64) * n
    nbr = np.tile(np.arange(n, dtype=np.int32), n)
    orc = oracle.Oracle(cases.disc_hole_2d(spacing=0.02, grid=64))
    tris, q = orc.triangulate(xyz, np.zeros(n, dtype=np.int32), np.ones(n), off, nbr)
    d = spatial.Delaunay(xyz[:, :2])
    edges = set()
    for s in d.simplices:
        for a in range(3):
            for b in range(a + 1, 3):
                edges.add((min(s[a], s[b]), max(s[a], s[b])))
    assert q["nedge_first"] == len(edges)
    assert q["ndeleted"] == 0
    got = {tuple(sorted(t)) for t in tris.tolist()}
    want = {tuple(sorted(s)) for s in d.simplices.tolist()}
    assert want <= got
    assert q["ntri"] == len(got)
    assert sum(q["hist"]) == 3 * q["ntri"]
    hull_area = spatial.ConvexHull(xyz[:, :2]).volume
    sep = len(got) - len(want)  # separating 3-cycles add area
    if sep == 0:
        assert abs(q["total_area"] - hull_area) < 1e-12


def test_curvature_spacing_law():
    """Spacing law 1: min_dl at the largest cut-cell |curvature| on the
    surface, middle_dl at the smallest, max_dl at max phi, monotone in |phi|;
    below -dl the reference's minimum."""
    case = cases.spheres_3d(fine_pkg=16, nlevels=2, dx_min=0.015, middle_dl=0.035, dx_max=0.09)
    orc = oracle.Oracle(case)
    c = orc.ctx
    assert c.scale_law == 1 and c.max_curv > c.min_curv > 0
    assert orc.get_scale(0.0, c.max_curv) == pytest.approx(c.min_dl, rel=1e-12)
    assert orc.get_scale(0.0, c.min_curv) == pytest.approx(c.middle_dl, rel=1e-12)
    mid = 0.5 * (c.max_curv + c.min_curv)
    s_mid = orc.get_scale(0.0, mid)
    assert s_mid == pytest.approx(c.min_dl + 0.25 * (c.middle_dl - c.min_dl), rel=1e-9)
    assert orc.get_scale(c.max_phi, mid) == pytest.approx(c.max_dl, rel=1e-12)
    vals = [orc.get_scale(f * c.max_phi, mid) for f in np.linspace(0, 1, 11)]
    assert all(b >= a for a, b in zip(vals, vals[1:]))
    assert orc.get_scale(-1.0, mid) == c.min_dl


def test_cvp_empty_cell_does_not_collapse():
    """Two far-apart clusters and a VP between them that loses its points:
    the partition stays finite and keeps every point assigned."""
    rng = np.random.default_rng(2)
    a = rng.normal(size=(3000, 3)) * 0.03 + [0.2, 0.2, 0.2]
    b = rng.normal(size=(3000, 3)) * 0.03 + [0.8, 0.8, 0.8]
    xyz = np.concatenate([a, b])
    vp = np.array([[0.2, 0.2, 0.2], [0.8, 0.8, 0.8], [0.5, 0.5, 0.5], [0.25, 0.2, 0.2]])
    v, lab, m, r = oracle.cvp(3, [0, 0, 0], [1, 1, 1], xyz, vp, max_iter=60)
    assert np.isfinite(v).all()
    assert m.sum() == len(xyz)
    assert np.bincount(lab, minlength=4).sum() == len(xyz)
    assert (m > 0).sum() >= 2  # both clusters keep a cell
