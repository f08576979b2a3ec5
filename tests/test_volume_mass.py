"""Cut-cell volume, surface area and particle count (CPU): the oracle's
restatement of Levelset_package::Calculate_volume_mass / GeometryCalculator
(lset_package.cpp:1283-1397, geometry_calculator.cpp:12-570) and
Get_num_particles (sph_mesh_generation.cpp:900-940), pinned against the
reference's own marching-cubes polygoniser (golden vectors from
tests/golden/make_mc_golden.py; live when oracle/_ref is built) and against
analytic volumes and areas."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from mrsph import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "mc_reference.npz")


def _polygons(table_row):
    tris = [table_row[q:q + 3] for q in range(0, 15, 3) if table_row[q] >= 0]
    comps = []
    for t in tris:
        m = sum(1 << int(e) for e in t)
        hit = [c for c in comps if c & m]
        for c in hit:
            comps.remove(c)
            m |= c
        comps.append(m)
    return sorted(comps), len(tris)


def test_mc_polygons_match_reference_golden():
    """Every one of the 256 sign cases yields the reference's polygons (the
    same cut edges, joined the same way on ambiguous faces) and triangle count."""
    g = np.load(GOLDEN)
    t = oracle.mc_table()
    for ci in range(256):
        polys, ntri = _polygons(t[ci])
        ref = [int(x) for x in g["case_polygons"][ci] if x]
        assert polys == ref, ci
        assert ntri == int(g["case_ntri"][ci]), ci


def test_mc_area_matches_reference_golden():
    """Areas of plane and sphere lattices against the reference's
    get_area_MQ: planes to rounding (planar polygons), spheres within the
    polygon-split difference."""
    g = np.load(GOLDEN)
    got = np.array([oracle.mc_area(c, h, h, h) for c, h in zip(g["lattices"], g["h"])])
    ref = g["area"]
    rel = np.abs(got - ref) / ref
    plane = g["kind"] == 0
    assert rel[plane].max() < 1e-12
    assert rel[~plane].max() < 2e-3
    assert abs(got[~plane].sum() - ref[~plane].sum()) / ref[~plane].sum() < 1e-4


def _ref_lib():
    import build_ref
    path = build_ref.build()
    if path is None or not os.path.exists(path):
        pytest.skip("reference polygoniser not built (reference sources absent)")
    R = C.CDLL(path)
    R.refp_area_mq.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    R.refp_area_mq.restype = C.c_double
    return R


def test_mc_area_matches_live_reference_on_torus():
    """Live check against the compiled reference polygoniser over the cut
    cells of a torus level set: total within 1e-5."""
    R = _ref_lib()
    rng = np.random.default_rng(3)
    h = 0.02
    g = np.array([(i, j, k) for i in range(3) for j in range(3) for k in range(3)], dtype=np.float64)
    a_sum = r_sum = 0.0
    n = 0
    while n < 800:
        c = rng.uniform([-1.4, -1.4, -0.4], [1.4, 1.4, 0.4])
        x = c + (g - 1.0) * 0.5 * h
        phi = 0.35 - np.sqrt((np.hypot(x[:, 0], x[:, 1]) - 1.0) ** 2 + x[:, 2] ** 2)
        if (phi > 0).all() or (phi < 0).all():
            continue
        phi = np.ascontiguousarray(phi)
        a_sum += oracle.mc_area(phi, h, h, h)
        r_sum += R.refp_area_mq(phi.ctypes.data, h, h, h)
        n += 1
    assert abs(a_sum - r_sum) / r_sum < 1e-5


def _nbhd_of(f, h, dim):
    """3^D cell-centred phi around a cell at the origin ([x][y][z], z=0 in 2D)."""
    p = np.zeros((3, 3, 3))
    for r in range(3):
        for s in range(3):
            for t in range(3 if dim == 3 else 1):
                p[r, s, t] = f((r - 1) * h, (s - 1) * h, (t - 1) * h if dim == 3 else 0.0)
    return p


@pytest.mark.parametrize("dim", [2, 3])
def test_half_space_through_centre_is_half(dim):
    """A plane through the cell centre cuts exactly half the volume (the
    bisection is exact on a plane through lattice points)."""
    h = 0.1
    vol, area = oracle.cut_cell(dim, _nbhd_of(lambda x, y, z: x, h, dim), h, h, h)
    dv = h ** dim
    assert vol == 0.5 * dv
    assert abs(area - (h * h if dim == 3 else h)) < 1e-15


def test_tilted_plane_volume_close():
    """A tilted plane: the bisection volume fraction within 2^-6 of the cell
    of the exact fraction; the marching-cubes area of a plane is exact."""
    h = 1.0
    n = np.array([0.3, -0.5, 0.8])
    n /= np.linalg.norm(n)
    off = 0.07
    vol, area = oracle.cut_cell(3, _nbhd_of(lambda x, y, z: n[0] * x + n[1] * y + n[2] * z - off, h, 3), h, h, h)
    # Monte-Carlo free: the fraction of the unit cube with n.x > off, by fine sampling
    g = (np.arange(200) + 0.5) / 200 - 0.5
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    frac = np.mean(n[0] * X + n[1] * Y + n[2] * Z > off)
    assert abs(vol - frac) < 2 ** -6


@pytest.mark.parametrize("dim", [2, 3])
def test_level_totals_analytic(dim):
    """Whole-level totals on a disc hole (2D) and a torus (3D): volume and
    surface area within the grid error of the analytic values; the particle
    numbers follow Get_num_particles from the totals."""
    if dim == 2:
        case = cases.disc_hole_2d(spacing=0.01, grid=128)
        # the unit square's sides and the hole's circle
        exact_v, exact_a = 1.0 - np.pi * 0.2 ** 2, 4.0 + 2 * np.pi * 0.2
    else:
        case = cases.torus_3d(dx_min=0.01, dx_max=0.04, fine_pkg=24, nlevels=1)
        exact_v, exact_a = 2 * np.pi ** 2 * 1.0 * 0.35 ** 2, 4 * np.pi ** 2 * 1.0 * 0.35
    orc = oracle.Oracle(case)
    r = orc.volume_mass(-1)
    dl = min(case.levels[-1].dpkg[d] / 4.0 for d in range(dim))
    # the counted region is phi > 0 plus the cells of the band -dl < phi < 0
    # that no corner of the cut-cell test reaches, so the volume exceeds the
    # body's by less than a band of one cell
    assert -1e-3 * exact_v < r["total_volume"] - exact_v < exact_a * dl
    assert abs(r["total_area"] - exact_a) / exact_a < 0.01
    assert r["num_interface_cell"] > 0
    assert r["num_particle_surface"] == min(int(r["total_mass_surface"]), r["num_interface_cell"])
    assert r["num_particle_mesh"] == max(int(r["total_mass"] - 0.5 * r["total_mass_surface"]), 0)
    assert r["num_particle"] == r["num_particle_mesh"] + r["num_particle_surface"]
    assert np.isclose(r["vol"].sum(), r["total_volume"], rtol=1e-12)
    assert np.isclose(r["area"].sum(), r["total_area"], rtol=1e-12)
    assert dl > 0


def test_count_close_to_spacing_integral():
    """The reference's count (cut-cell volumes, minus half the surface
    particles, plus the surface particles) stays close to the spacing
    integral over phi > 0 the workloads are sized with."""
    case = cases.torus_3d(dx_min=0.01, dx_max=0.04, fine_pkg=24, nlevels=1)
    r = oracle.Oracle(case).volume_mass(-1)
    n_int = cases.particle_count(case.levels, case.params)
    assert abs(r["num_particle"] - n_int) / n_int < 0.1


def test_oracle_segment_and_singularity_terms():
    """A box [0.1, 0.9]^3 whose 8 corners are singularities and 12 edges
    segments: the SEGMENT cells' lengths add up to the edges' length outside
    the corner (SINGULARITY) cells, and Get_num_particles
    (sph_mesh_generation.cpp:909-923) counts 8 singularity particles and
    int(total_mass_segment - 4) segment particles; in 2D neither term exists
    beyond the 4 singularities."""
    import oracle
    from mrsph import cases
    case = cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic", h_over_dx=1.0)
    orc = oracle.Oracle(case)
    r = orc.volume_mass(0)
    dc = case.levels[0].dpkg[0] / 4
    assert 12 * 0.8 - 24 * dc * 1.5 < r["total_length"] <= 12 * 0.8 + 1e-12
    assert r["num_particle_singularity"] == 8
    assert r["num_particle_segment"] == max(int(r["total_mass_segment"] - 4.0), 0) > 0
    surf = max(int(r["total_mass_surface"] - 0.5 * r["total_mass_segment"]), 0)
    assert r["num_particle_surface"] == min(surf, r["num_interface_cell"])
    assert r["num_particle"] == (r["num_particle_mesh"] + r["num_particle_surface"] + r["num_particle_segment"] +
                                 r["num_particle_singularity"])
    case2 = cases.box_with_corners(dim=2, spacing=0.02, grid=64, kernel="hyperbolic", h_over_dx=1.0)
    r2 = oracle.Oracle(case2).volume_mass(0)
    assert r2["total_mass_segment"] == 0.0 and r2["num_particle_segment"] == 0
    assert r2["num_particle_singularity"] == 4
