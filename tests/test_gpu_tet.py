"""3D tetrahedralisation on the GPU (mrsph_tetrahedralize, the local
certified-Delaunay form of Graphmeshcls::Reconstruct_tets,
geometry_tools/graph_mesh.cpp:981-1100, with Tet_quality_statistics,
:1967-2400) against the oracle on the same relaxed particles and neighbour
rows: the tet list bit-exact (same order), every count and histogram equal,
the floating statistics within 1e-12; and the tets are Delaunay tets of
qhull's tetrahedralisation of the snapped positions."""
import numpy as np
import pytest

import oracle
from mrsph import cases
from paritylib import make_gpu

pytestmark = pytest.mark.gpu

CASES = {
    "box3d_fp64": (lambda: cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic", h_over_dx=1.0),
                   "fp64", 150),
    "torus3d_fp32": (lambda: cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2), "fp32", 60),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_tets_match_oracle(name):
    mk, prec, steps = CASES[name]
    case = mk()
    g = make_gpu(case, prec)
    g.Initialize_case()
    g.SPH_run_mesh_generation(steps)
    p = g.particles(("xyz", "type", "h"))
    off, nb = g.neighbors()
    tets, q = g.Reconstruct_tets()
    g.close()
    ot, oq = oracle.tetrahedralize(p["xyz"], p["type"], p["h"], off, nb, case.params["cutoff"],
                                   case.params["box_l"], case.params["box_r"])
    assert len(tets) == q["ntet"] == len(ot) > 3 * len(p["xyz"])
    assert np.array_equal(tets, ot)
    for k in ("ntet", "nopen", "ndeleted", "ntie", "ntrunc"):
        assert q[k] == oq[k], k
    for k in ("nsmall_dihedral", "aspect_hist", "radius_hist", "dihedral_hist"):
        assert list(q[k]) == list(oq[k]), k
    for k in ("grid", "min_volume", "max_volume", "min_edge", "max_edge", "min_aspect", "max_aspect",
              "min_radius_ratio", "max_radius_ratio"):
        assert q[k] == oq[k], k
    for k in ("total_volume", "avg_aspect", "avg_radius_ratio", "min_dihedral", "max_dihedral", "avg_min_dihedral"):
        assert abs(q[k] - oq[k]) <= 1e-12 * abs(oq[k]), k
    if name.startswith("box"):
        from scipy.spatial import Delaunay
        xs = oracle.snap(p["xyz"], case.params["box_l"], case.params["box_r"])
        qh = set(map(tuple, np.sort(Delaunay(xs).simplices, axis=1)))
        assert set(map(tuple, tets)) <= qh


def test_tetrahedralize_rejects_2d():
    from mrsph import _lib as L
    g = make_gpu(cases.disc_hole_2d(spacing=0.02, grid=64), "fp64")
    g.Initialize_case()
    g.SPH_run_mesh_generation(1)
    with pytest.raises(L.MrsphError):
        g.Reconstruct_tets()
    g.close()
