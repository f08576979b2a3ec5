"""Batched relaxation (mrsph_batch_*): a batch of independent 2D and 3D
geometries of uneven size, stepped together, gives every handle exactly the
state that stepping it alone gives (both precisions; FP32-split in the
persistent, the per-phase and the per-handle-stream modes), across a
neighbour-list capacity check; the persistent kernel's grid barrier gives up
after its time limit."""
import numpy as np
import pytest

from mrsph import BatchRelaxation, SPHMeshGeneration, cases
from mrsph.solver import barrier_selftest

pytestmark = pytest.mark.gpu


def _geoms():
    return [cases.star_shape(2, 5, 3000), cases.star_shape(3, 6, 6000), cases.star_shape(2, 7, 12000),
            cases.star_shape(3, 8, 2500), cases.disc_hole_2d(spacing=0.02, grid=64)]


@pytest.mark.parametrize("prec,mode", [("fp32", "persistent"), ("fp32", "phases"), ("fp32", "streams"),
                                       ("fp64", "streams")])
def test_batch_equals_solo(prec, mode):
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
    assert b.mode == ("persistent" if prec == "fp32" else "streams")
    b.set_mode(mode)
    assert b.mode == mode
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


def test_batch_kernels_need_fp32_split():
    hs = []
    for c in _geoms()[:2]:
        g = SPHMeshGeneration(c, precision="fp64")
        g.Initialize_case()
        hs.append(g)
    b = BatchRelaxation(hs)
    assert b.mode == "streams"
    for mode in ("persistent", "phases"):
        with pytest.raises(Exception):
            b.set_mode(mode)
    b.close()
    for g in hs:
        g.close()


def test_persistent_barrier_wait_is_bounded():
    """A barrier that one block of the launch never reaches: the wait gives
    up after its limit, the kernel returns with its error bit raised, and the
    device still runs a persistent batch afterwards."""
    assert barrier_selftest(0, 200.0)
    hs = []
    for c in _geoms()[:2]:
        g = SPHMeshGeneration(c, precision="fp32")
        g.Initialize_case()
        hs.append(g)
    b = BatchRelaxation(hs)
    assert b.mode == "persistent"
    b.SPH_run_mesh_generation(3)
    b.sync()
    assert all(g.stats()["step"] == 3 for g in hs)
    b.close()
    for g in hs:
        g.close()


@pytest.mark.parametrize("prec,mode", [("fp32", "persistent"), ("fp32", "phases"), ("fp64", "streams")])
def test_batch_with_characteristic_particles(prec, mode):
    """Geometries with corners and edges (SINGULARITY and SEGMENT particles,
    the hyperbolic kernel) batched with a star: every handle ends where
    stepping it alone ends, bit for bit."""
    geoms = [cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic", h_over_dx=1.0),
             cases.box_with_corners(dim=2, spacing=0.02, grid=64, kernel="hyperbolic", h_over_dx=1.0),
             cases.star_shape(3, 8, 2500)]
    steps = 160
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
    b = BatchRelaxation(hs, mode=mode)
    b.SPH_run_mesh_generation(steps)
    for g, ref in zip(hs, solo):
        got = g.particles(("xyz", "type", "h"))
        assert np.array_equal(got["xyz"], ref["xyz"])
        assert np.array_equal(got["type"], ref["type"])
        assert np.array_equal(got["h"], ref["h"])
    t = solo[0]["type"]
    assert (t == 2).any() and (t == 3).any()
    b.close()
    for g in hs:
        g.close()


def test_destroy_handle_before_batch():
    """A handle destroyed while a batch holds it leaves the batch (after its
    queued work): the batch then refuses to step, and both destructions in
    either order are safe."""
    from mrsph import _lib as L
    geoms = _geoms()[:2]
    hs = []
    for c in geoms:
        g = SPHMeshGeneration(c, precision="fp32")
        g.Initialize_case()
        hs.append(g)
    b = BatchRelaxation(hs)
    b.SPH_run_mesh_generation(2)
    hs[0].close()
    with pytest.raises(L.MrsphError):
        b.SPH_run_mesh_generation(1)
    b.close()
    hs[1].SPH_run_mesh_generation(1)
    hs[1].sync()
    assert hs[1].stats()["step"] == 3
    hs[1].close()
