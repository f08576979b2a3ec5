"""Batched relaxation (mrsph_batch_*): a batch of independent 2D and 3D
geometries of uneven size, stepped together, gives every handle exactly the
state that stepping it alone gives (both precisions), across a neighbour-list
capacity check."""
import numpy as np
import pytest

from mrsph import BatchRelaxation, SPHMeshGeneration, cases

pytestmark = pytest.mark.gpu


def _geoms():
    return [cases.star_shape(2, 5, 3000), cases.star_shape(3, 6, 6000), cases.star_shape(2, 7, 12000),
            cases.star_shape(3, 8, 2500), cases.disc_hole_2d(spacing=0.02, grid=64)]


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_batch_equals_solo(prec):
    geoms = _geoms()
    steps = 40
    solo = []
    for c in geoms:
        g = SPHMeshGeneration(c, precision=prec)
        g.Initialize_case()
        g.SPH_run_mesh_generation(steps)
        solo.append(g.particles(("xyz", "type", "h")))
        g.close()
    hs = []
    for c in geoms:
        g = SPHMeshGeneration(c, precision=prec)
        g.Initialize_case()
        hs.append(g)
    b = BatchRelaxation(hs)
    b.SPH_run_mesh_generation(25)
    b.SPH_run_mesh_generation(steps - 25)
    for g, ref in zip(hs, solo):
        got = g.particles(("xyz", "type", "h"))
        assert np.array_equal(got["xyz"], ref["xyz"])
        assert np.array_equal(got["type"], ref["type"])
        assert np.array_equal(got["h"], ref["h"])
        assert g.stats()["step"] == steps
    ms = b.step_timed(3)
    assert ms > 0
    for g in hs:
        assert g.stats()["step"] == steps + 3
    b.close()
    for g in hs:
        g.close()


def test_batch_then_solo_steps():
    """A handle may be stepped alone between batch calls."""
    geoms = _geoms()[:3]
    ref = []
    for c in geoms:
        g = SPHMeshGeneration(c, precision="fp32")
        g.Initialize_case()
        g.SPH_run_mesh_generation(12)
        ref.append(g.particles(("xyz",))["xyz"])
        g.close()
    hs = []
    for c in geoms:
        g = SPHMeshGeneration(c, precision="fp32")
        g.Initialize_case()
        hs.append(g)
    b = BatchRelaxation(hs)
    b.SPH_run_mesh_generation(5)
    hs[1].SPH_run_mesh_generation(1)
    for k in (0, 2):
        hs[k].SPH_run_mesh_generation(1)
    b.SPH_run_mesh_generation(6)
    for g, r in zip(hs, ref):
        assert np.array_equal(g.particles(("xyz",))["xyz"], r)
    b.close()
    for g in hs:
        g.close()
