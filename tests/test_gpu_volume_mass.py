"""GPU cut-cell volume, surface area and particle count (mrsph_volume_mass)
against the FP64 oracle: per-cell volumes bit-exact (every partial volume of
the bisection is a dyadic fraction, so the sum is exact in any order),
per-cell areas within 1e-12 relative, the level sums within 1e-10 (the
oracle adds up to ~10^6 cells in sequence, the GPU in a tree: n * eps of
the sequential sum), particle numbers equal.  At the benchmark size: size-independent checks
against the analytic torus."""
import numpy as np
import pytest

import oracle
from mrsph import cases
from paritylib import make_gpu, small_cases

pytestmark = pytest.mark.gpu



def dyadic_case(dim: int, kind: str):
    """Planes at dyadic positions on a dyadic grid (cell 1/64): corner values
    and bisection midpoints hit exact zeros at many refinement levels, where
    FP32 cannot decide a sign and the FP64 path must."""
    p = cases.default_params(dim)
    p.update(min_dl=1 / 32, max_dl=1 / 32, cell_ratio=2.6, box_l=[0, 0, 0], box_r=[1, 1, 1 if dim == 3 else 0],
             seed=1)
    if kind == "box":
        def sdf(X, Y, Z):
            f = np.minimum(np.minimum(X - 13 / 64, 51 / 64 + 1 / 512 - X), np.minimum(Y - 0.25 - 3 / 1024, 0.75 - Y))
            return np.minimum(f, np.minimum(Z - 0.3125, 0.6875 + 1 / 128 - Z)) if dim == 3 else f
    else:
        def sdf(X, Y, Z):
            return 0.25 - np.abs((X - 0.5) + 0.5 * (Y - 0.5) - (0.25 * (Z - 0.5) if dim == 3 else 0.0))
    lv = cases.make_level(sdf, dim, [0, 0, 0], [1 / 16, 1 / 16, 1 / 16 if dim == 3 else 1.0],
                          [16, 16, 16 if dim == 3 else 1])
    return cases.Case(f"{kind}_dyadic_{dim}d", p, [lv], 1000, steps=10)


CASES = dict(small_cases())
CASES["disc2d_fine"] = lambda: cases.disc_hole_2d(spacing=0.01, grid=128)
CASES["torus3d_single"] = lambda: cases.torus_3d(dx_min=0.01, dx_max=0.04, fine_pkg=24, nlevels=1)
# corners and edges: the segment mass and the singularity / segment particle numbers
CASES["box3d_corners"] = lambda: cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic",
                                                        h_over_dx=1.0)
CASES["box2d_corners"] = lambda: cases.box_with_corners(dim=2, spacing=0.02, grid=64, kernel="hyperbolic",
                                                        h_over_dx=1.0)
for _d in (2, 3):
    for _k in ("box", "tilted"):
        CASES[f"{_k}_dyadic_{_d}d"] = (lambda d=_d, k=_k: dyadic_case(d, k))


@pytest.mark.parametrize("name", sorted(CASES))
def test_volume_mass_matches_oracle(name):
    case = CASES[name]()
    orc = oracle.Oracle(case)
    gpu = make_gpu(case, "fp64")
    try:
        for level in range(len(case.levels)):
            ref = orc.volume_mass(level)
            got = gpu.volume_mass(level, cells=True)
            vol = got["vol"].ravel()
            area = got["area"].ravel()
            assert np.array_equal(vol, ref["vol"]), f"cell volumes, level {level}"
            scale = max(np.abs(ref["area"]).max(), 1e-300)
            assert np.max(np.abs(area - ref["area"])) <= 1e-12 * scale, f"cell areas, level {level}"
            for k in ("total_mass", "total_mass_surface", "total_volume", "total_area", "total_mass_segment",
                      "total_length"):
                assert abs(got[k] - ref[k]) <= 1e-10 * abs(ref[k]) + 1e-300, (k, level)
            for k in ("num_interface_cell", "num_particle_mesh", "num_particle_surface", "num_particle",
                      "num_particle_segment", "num_particle_singularity"):
                assert got[k] == ref[k], (k, level)
            assert got["device_ms"] > 0
    finally:
        gpu.close()


def test_volume_mass_deterministic():
    case = CASES["torus3d_adaptive"]()
    gpu = make_gpu(case, "fp32")
    try:
        a = gpu.volume_mass(-1)
        b = gpu.volume_mass(-1)
        for k in ("total_mass", "total_mass_surface", "total_volume", "total_area", "num_particle"):
            assert a[k] == b[k]
    finally:
        gpu.close()


def test_volume_mass_full_torus():
    """The benchmark torus (finest level 256 x 256 x 96 cells): volume above the
    body's by less than a one-cell band, area within 0.5% of 4 pi^2 R r, the
    particle numbers by Get_num_particles."""
    case = cases.torus_3d()
    gpu = make_gpu(case, "fp32", cap=0)
    try:
        r = gpu.volume_mass(-1)
    finally:
        gpu.close()
    exact_v, exact_a = 2 * np.pi ** 2 * 0.35 ** 2, 4 * np.pi ** 2 * 0.35
    dl = case.levels[-1].dpkg[0] / 4.0
    assert -1e-3 * exact_v < r["total_volume"] - exact_v < exact_a * dl
    assert abs(r["total_area"] - exact_a) / exact_a < 5e-3
    assert r["num_particle_surface"] == min(int(r["total_mass_surface"]), r["num_interface_cell"])
    assert r["num_particle_mesh"] == max(int(r["total_mass"] - 0.5 * r["total_mass_surface"]), 0)
    assert r["num_particle"] == r["num_particle_mesh"] + r["num_particle_surface"]


def test_initialize_with_cut_cell_count():
    """Initialize_case(cut_cell_count=True) seeds Get_num_particles particles."""
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    g = make_gpu(case, "fp64")
    try:
        n = g.Get_num_particles()
        g.Initialize_case(cut_cell_count=True)
        assert g.n == n and g.stats()["n"] == n
    finally:
        g.close()
