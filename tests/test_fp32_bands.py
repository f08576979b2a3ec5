"""The bands of the FP32-split decisions against the FP32 error they cover.

The FP32-split engine makes three decisions in FP32 and re-makes them in
FP64 only inside a band around the threshold: the half cell of the sort key
(band 2^-16 of a half cell), the neighbour criterion (band 2^-15 of the squared
cut-off radius) and the surface filter |n_i . n_j| > cos(angle_thres) (band
2^-16).  A decision outside its band is final, so the FP32 value must never be
farther from the FP64 value of the world positions than the band.  These
tests emulate the kernels' FP32 arithmetic with numpy on many random
configurations (anchor cells of the finest cell-list level, offsets inside
them, pairs at the cut-off across several anchor cells) and check that the
largest error seen stays a factor of 4 or more inside each band.
"""
import numpy as np

BAND_KEY = 2.0 ** -16
BAND_D2 = 2.0 ** -15
BAND_COS = 2.0 ** -16

f32 = np.float32


def fma32(a, b, c):
    """FP32 fused multiply-add: the product of two floats is exact in FP64."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f32)


def world(box_l, k, A, o):
    """The engine's world coordinate box_l + (k A + o) in FP64 (one fused
    multiply-add, then one add)."""
    t = np.array([np.float64(ki) * A + np.float64(oi) for ki, oi in zip(k, o)])  # the multiply-add
    return box_l + t


def test_key_band_covers_fp32_error():
    rng = np.random.default_rng(1)
    box_l = -1.45
    A = 2.9 / 1160          # finest cell of a 1160-cell axis (the torus)
    Af = f32(A)
    worst = 0.0
    for sh in (0, 1, 2, 3):  # the level-L cell is 2^sh anchor cells
        hs = 0.5 * A * 2 ** sh
        ihs_f = f32(1.0 / hs)
        k = rng.integers(0, 1160, 20000)
        o = (rng.random(20000) * A).astype(f32)
        cc = k >> sh
        m = (k - (cc << sh)).astype(f32)
        u32 = fma32(m, np.full_like(m, Af), o) * ihs_f
        rel = world(box_l, k, A, o) - box_l
        u64 = rel / hs - 2 * cc
        worst = max(worst, float(np.max(np.abs(u32.astype(np.float64) - u64))))
    assert worst < BAND_KEY / 4, worst


def test_distance_band_covers_fp32_error():
    """Pairs at their cut-off radius R = h cutoff over 1-16 anchor cells, in
    the warp-tile form: both positions relative to an anchor up to 3 cells
    away ((k - k_anchor) Af + o), then the squared difference in FP32."""
    rng = np.random.default_rng(2)
    box_l = -1.45
    A = 2.9 / 1160
    Af = f32(A)
    cutoff = 2.0
    worst = 0.0
    for cells in (0.5, 1.0, 2.0, 4.0, 8.0, 16.0):
        n = 20000
        R = cells * A
        h = f32(R / cutoff)
        ki = rng.integers(100, 1000, (n, 3))
        oi = (rng.random((n, 3)) * A).astype(f32)
        d = rng.normal(size=(n, 3))
        d /= np.linalg.norm(d, axis=1)[:, None]
        xi = np.stack([world(box_l, ki[:, a], A, oi[:, a]) for a in range(3)], 1)
        xj_target = xi + d * R
        kj = np.floor((xj_target - box_l) / A).astype(np.int64)
        oj = ((xj_target - box_l) - kj * A).astype(f32)
        wa = ki + rng.integers(-3, 4, (n, 3))  # the warp's anchor cell
        pi = fma32((ki - wa).astype(f32), np.full((n, 3), Af), oi)
        pj = fma32((kj - wa).astype(f32), np.full((n, 3), Af), oj)
        dr = (pi - pj).astype(f32)
        d2_32 = (dr[:, 0] * dr[:, 0]).astype(f32)
        d2_32 = (d2_32 + (dr[:, 1] * dr[:, 1]).astype(f32)).astype(f32)
        d2_32 = (d2_32 + (dr[:, 2] * dr[:, 2]).astype(f32)).astype(f32)
        R2_32 = (h * f32(cutoff)) * (h * f32(cutoff))
        xw_i = np.stack([world(box_l, ki[:, a], A, oi[:, a]) for a in range(3)], 1)
        xw_j = np.stack([world(box_l, kj[:, a], A, oj[:, a]) for a in range(3)], 1)
        d64 = np.sqrt(np.sum((xw_i - xw_j) ** 2, axis=1))
        r64 = np.float64(h) * cutoff + 1e-10
        # the FP32 quantity d2 / R^2 against the FP64 decision's dist / r
        e = np.abs(d2_32.astype(np.float64) / np.float64(R2_32) - (d64 / r64) ** 2)
        worst = max(worst, float(np.max(e)))
    assert worst < BAND_D2 / 4, worst


def test_plus_1e10_inside_distance_band():
    """The reference's +1e-10 on the radius moves R^2 by at most
    2 1e-10 / R_min relative; with R_min = 1e-4 (enforced for FP32-split
    handles) that is well inside the band."""
    assert 2 * 1e-10 / 1e-4 < BAND_D2 / 4


def test_cos_band_covers_fp32_error():
    rng = np.random.default_rng(3)
    n = 200000
    ni = rng.normal(size=(n, 3))
    nj = rng.normal(size=(n, 3))
    ni = (ni / np.linalg.norm(ni, axis=1)[:, None] * rng.uniform(0.5, 1.0, (n, 1))).astype(f32)
    nj = (nj / np.linalg.norm(nj, axis=1)[:, None] * rng.uniform(0.5, 1.0, (n, 1))).astype(f32)
    c32 = (ni[:, 0] * nj[:, 0]).astype(f32)
    c32 = (c32 + (ni[:, 1] * nj[:, 1]).astype(f32)).astype(f32)
    c32 = (c32 + (ni[:, 2] * nj[:, 2]).astype(f32)).astype(f32)
    c64 = np.sum(ni.astype(np.float64) * nj.astype(np.float64), axis=1)
    cos_t64 = np.cos(0.4 * np.pi)
    worst = float(np.max(np.abs(np.abs(c32.astype(np.float64)) - np.float32(cos_t64) -
                                (np.abs(c64) - cos_t64))))
    assert worst < BAND_COS / 4, worst
