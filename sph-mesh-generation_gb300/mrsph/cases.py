"""Case definitions: analytic level sets and relaxation parameters.

This is the user-defined part of a run, the counterpart of the reference's
``SPH_mesh_generation::Load_case`` (sph_mesh_generation/sph_mesh_generation.cpp:156-319)
and ``Levelset::F_phi`` (level_set_solver/level_set.cpp:92-173): it chooses the
domain, the level-set grid(s) and the target spacing range, and evaluates phi
(positive inside the body) at level-set cell centres.  Normals, cut-cell tags,
curvature and the maximum phi are computed on the GPU by the library
(``mrsph_set_levelset``).

Grid layout (one nested level): interior packages of 4^D cells cover
``[box_l, box_l + num_pkg*dpkg)`` and ``margin`` packages pad every side
(lset_level_infor.cpp:17-85).  Cell centres are
``pkg*dpkg + (cell + 0.5)*dcell + box_l`` (lset_package.cpp:70-79), evaluated
in that order so phi matches what the reference would sample.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

PI_REF = 3.1415926  # glbparam.h:186

KERNELS = {"hyperbolic": 0, "cubic": 1, "wendland": 2, "gaussian": 3, "quintic": 4}
PRECISIONS = {"fp64": 0, "fp32": 1}


@dataclass
class LevelGrid:
    box_l: List[float]
    dpkg: List[float]
    num_pkg: List[int]
    margin: int
    phi: np.ndarray                    # float64, shape (nz, ny, nx) incl. margins (nz = 1 in 2D)
    active: Optional[np.ndarray] = None  # uint8 per package incl. margins, or None


@dataclass
class Case:
    name: str
    params: dict
    levels: List[LevelGrid]
    n_particles: int
    steps: int = 200
    notes: str = ""
    extra: dict = field(default_factory=dict)


def default_params(dim: int) -> dict:
    """Reference defaults: Wendland C2 off, hyperbolic kernel (Makefile.in:36),
    CELL_RATIO 2.0 (2D) / 1.45 (3D) (glbparam.h:171-183), CUT_OFF 2,
    angle_thres 0.4*PI, nu 0.1, damping 0 (sph_mesh_generation.cpp:688-703)."""
    return {
        "dim": dim,
        "kernel": KERNELS["hyperbolic"],
        "precision": PRECISIONS["fp64"],
        "cell_ratio": 2.0 if dim == 2 else 1.45,
        "cutoff": 2.0,
        "angle_thres": PI_REF * 0.4,
        "nu_coeff": 0.1,
        "damp_coeff": 0.0,
        "min_dl": 0.01,
        "max_dl": 0.01,
        "box_l": [0.0, 0.0, 0.0],
        "box_r": [1.0, 1.0, 1.0],
        "seed": 0,
        "neighbor_cap": 0,
        "scale_law": 0,      # 0: tanh law of phi (the reference's); 1: curvature law
        "middle_dl": 0.0,    # law 1; <= 0: 5 x the level-0 level-set cell
    }


def cell_centres(box_l, dpkg, num_pkg, margin, dim):
    """Axis coordinates of the cell centres incl. margin packages."""
    axes = []
    for d in range(3):
        if d >= dim:
            axes.append(np.zeros(1))
            continue
        pk = np.repeat(np.arange(-margin, num_pkg[d] + margin), 4).astype(np.float64)
        cl = np.tile(np.arange(4), num_pkg[d] + 2 * margin).astype(np.float64)
        dcell = dpkg[d] / 4.0
        axes.append(pk * dpkg[d] + (cl + 0.5) * dcell + box_l[d])
    return axes


def make_level(sdf: Callable, dim: int, box_l, dpkg, num_pkg, margin: int = 1, broadcast: bool = False) -> LevelGrid:
    """phi of one level at the cell centres; broadcast=True hands sdf the
    axes as broadcastable (1, 1, nx), (1, ny, 1), (nz, 1, 1) arrays instead
    of full meshgrids."""
    ax = cell_centres(box_l, dpkg, num_pkg, margin, dim)
    if broadcast:
        X, Y, Z = ax[0][None, None, :], ax[1][None, :, None], ax[2][:, None, None]
    else:
        Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    phi = np.ascontiguousarray(sdf(X, Y, Z), dtype=np.float64)
    return LevelGrid(list(box_l), list(dpkg), list(num_pkg), margin, phi, None)


def nested_active(level: LevelGrid, band: float, dim: int) -> np.ndarray:
    """Package mask of a finer nested level: active where any cell has |phi| < band."""
    m = level.margin
    nz = (level.num_pkg[2] + 2 * m) if dim == 3 else 1
    ny = level.num_pkg[1] + 2 * m
    nx = level.num_pkg[0] + 2 * m
    a = np.abs(level.phi)
    if dim == 3:
        blk = a.reshape(nz, 4, ny, 4, nx, 4).min(axis=(1, 3, 5))
    else:
        blk = a.reshape(1, ny, 4, nx, 4).min(axis=(2, 4))
    return (blk < band).astype(np.uint8)


def scale_law(phi, min_dl, max_dl, max_phi, dl0):
    """Levelset::Get_scale, level_set_solver/level_set.cpp:311-351 (tanh law)."""
    phi = np.asarray(phi, dtype=np.float64)
    s = min_dl + np.tanh(2.5 * np.abs(phi) / max_phi) / np.tanh(2.5) * (max_dl - min_dl)
    return np.where((phi > 0) | (np.abs(phi) < dl0), s, min_dl)


def curvature_estimate(lv: LevelGrid, dim: int) -> np.ndarray:
    """|curvature| of phi on the cells next to the interface (0 elsewhere) by
    the level-set build's difference formulas, clamped to 2 / |cell|; the
    interface test is a sign change over the 3^D neighbourhood.  Used only to
    count particles under the curvature law.  The interface cells are found
    first and the differences evaluated there only (the grid's outermost two
    cells are never interface cells: they are margin cells far from phi = 0)."""
    ph = lv.phi if dim == 3 else lv.phi[0]
    dc = [lv.dpkg[d] / 4.0 for d in range(dim)]
    ax = list(range(dim))[::-1]  # array axis of coordinate d
    shape = ph.shape
    # sign change over the axis neighbours: min / max of the cell and its 2D
    # neighbours along the axes (array edges compare with themselves)
    lo = ph.copy()
    hi = ph.copy()
    for d in range(dim):
        a = ax[d]
        for k in (-1, 1):
            sl_dst = [slice(None)] * ph.ndim
            sl_src = [slice(None)] * ph.ndim
            if k == 1:
                sl_dst[a], sl_src[a] = slice(0, -1), slice(1, None)
            else:
                sl_dst[a], sl_src[a] = slice(1, None), slice(0, -1)
            np.minimum(lo[tuple(sl_dst)], ph[tuple(sl_src)], out=lo[tuple(sl_dst)])
            np.maximum(hi[tuple(sl_dst)], ph[tuple(sl_src)], out=hi[tuple(sl_dst)])
    cut = (lo < 0) & (hi > 0)
    del lo, hi
    idx = np.flatnonzero(cut)
    coords = np.unravel_index(idx, shape)
    inner = np.ones(idx.shape, dtype=bool)
    for a in range(ph.ndim):
        inner &= (coords[a] >= 2) & (coords[a] < shape[a] - 2)
    idx = idx[inner]
    flat = ph.ravel()
    stride = [int(np.prod(shape[a + 1:])) for a in range(ph.ndim)]

    def sh(d, k):  # phi at offset k along coordinate d of the interface cells
        return flat[idx + k * stride[ax[d]]]

    def sh2(a_, ka, b_, kb):
        return flat[idx + ka * stride[ax[a_]] + kb * stride[ax[b_]]]
    p0 = flat[idx]
    g1 = [(8.0 * (sh(d, 1) - sh(d, -1)) - (sh(d, 2) - sh(d, -2))) / dc[d] / 12.0 for d in range(dim)]
    g2 = [(sh(d, 1) - 2 * p0 + sh(d, -1)) / dc[d] / dc[d] for d in range(dim)]

    def mixed(a, b):
        return 0.25 * (sh2(a, 1, b, 1) - sh2(a, -1, b, 1) - sh2(a, 1, b, -1) + sh2(a, -1, b, -1)) / dc[a] / dc[b]
    if dim == 2:
        px, py = g1
        pxx, pyy = g2
        pxy = mixed(0, 1)
        num = px * px * pyy - 2 * px * py * pxy + py * py * pxx
        den = (px * px + py * py) ** 1.5
    else:
        px, py, pz = g1
        pxx, pyy, pzz = g2
        pxy, pxz, pyz = mixed(0, 1), mixed(0, 2), mixed(1, 2)
        num = (px * px * pyy - 2 * px * py * pxy + py * py * pxx + px * px * pzz - 2 * px * pz * pxz
               + pz * pz * pxx + py * py * pzz - 2 * py * pz * pyz + pz * pz * pyy)
        den = (px * px + py * py + pz * pz) ** 1.5
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.where(den > 0, num / den, 0.0)
    cd = np.sqrt(sum(v * v for v in dc))
    c = np.abs(np.clip(c, -2.0 / cd, 2.0 / cd))
    out = np.zeros(ph.size)
    out[idx] = c
    return out.reshape(lv.phi.shape)


def particle_count(levels: List[LevelGrid], params: dict) -> int:
    """Target count from the spacing integral over phi > 0 (the reference's
    total_mass = sum vol/scale^D, lset_package.cpp:1283-1397, without the
    cut-cell geometry refinement), evaluated on the finest level."""
    dim = params["dim"]
    mp = max_phi(levels, dim)
    fine = levels[-1]
    m = fine.margin * 4
    sl = [slice(m, -m) for _ in range(dim)]
    if dim == 2:
        inner = fine.phi[0][sl[1], sl[0]]
    else:
        inner = fine.phi[sl[2], sl[1], sl[0]]
    dV = 1.0
    for d in range(dim):
        dV *= fine.dpkg[d] / 4.0
    dl0 = min(levels[0].dpkg[d] / 4.0 for d in range(dim))
    if params.get("scale_law", 0) == 1:
        cv = curvature_estimate(fine, dim)
        cv = cv[0][sl[1], sl[0]] if dim == 2 else cv[sl[2], sl[1], sl[0]]
        cut = cv > 0
        cmax, cmin = (cv[cut].max(), cv[cut].min()) if cut.any() else (0.0, 1e20)
        mid = params.get("middle_dl", 0.0)
        if mid <= 0:
            mid = 5.0 * dl0
        q = np.clip((cmax - cv) / (cmax - cmin + 1e-20), 0.0, 1.0)
        lo = params["min_dl"] + q * q * (mid - params["min_dl"])
        t = np.tanh(2.5 * np.abs(inner) / mp) / np.tanh(2.5)
        sc = np.where((inner > 0) | (np.abs(inner) < dl0), lo + t * (params["max_dl"] - lo), params["min_dl"])
    else:
        sc = scale_law(inner, params["min_dl"], params["max_dl"], mp, dl0)
    return int(np.sum(np.where(inner > 0, dV / sc ** dim, 0.0)))


def max_phi(levels: List[LevelGrid], dim: int) -> float:
    mp = 0.0
    for lv in levels:
        m = lv.margin * 4
        if dim == 2:
            inner = lv.phi[0][m:-m, m:-m]
        else:
            inner = lv.phi[m:-m, m:-m, m:-m]
        pos = inner[inner > 0]
        if pos.size:
            mp = max(mp, float(pos.max()))
    return mp


def cell_levels_consistent(box_l, box_r, dim: int, max_scale: float, min_scale: float) -> bool:
    """True when the reference's tight level plan (sph.cpp:144-180) gives every
    cell-list level a cell size of max_scale' / 2^l, max_scale' = domain /
    floor(domain / max_scale).  The plan truncates domain / max_scale' per axis,
    which for some domains loses a cell to rounding (1.125 / (1.125 / 28) < 28);
    the library rejects such domains."""
    dom = [box_r[d] - box_l[d] for d in range(dim)]
    st = min(dom)
    temp = math.floor(st / max_scale)
    if temp < 1:
        return False
    ini = st / temp
    sc, nl = ini, 1
    while sc + 1.e-6 > min_scale:
        sc /= 2
        nl += 1
    nl -= 1
    n0 = [int(dom[d] / ini) for d in range(dim)]
    for l in range(nl):
        s = min(dom[d] / (n0[d] * 2.0 ** l) for d in range(dim))
        if abs(s - math.ldexp(ini, -l)) > 1.e-10:
            return False
    return True


# ---------------------------------------------------------------------------
# Workloads
# ---------------------------------------------------------------------------
def disc_hole_2d(spacing: float = 0.01, grid: int = 256, kernel: str = "wendland",
                 h_over_dx: float = 1.3, precision: str = "fp64", seed: int = 0,
                 steps: int = 200) -> Case:
    """Unit square minus a disc (r = 0.2 at (0.5, 0.5)), analytic SDF sampled
    at grid cells per unit length (grid^2 cells over the unit square), constant
    spacing.  The domain adds grid/16 cells of margin on every side so that the
    seeding clamp (one package inside the box, Random_particle_distribution,
    sph_mesh_generation.cpp:1331-1345) falls outside the body."""
    p = default_params(2)
    npkg_unit = grid // 4
    dpkg = 1.0 / npkg_unit
    cell_ratio = 2.0 * h_over_dx
    margin_pkg = max(npkg_unit // 16, 1)
    while not cell_levels_consistent([-margin_pkg * dpkg] * 2, [1.0 + margin_pkg * dpkg] * 2, 2,
                                     spacing * cell_ratio, spacing * cell_ratio):
        margin_pkg += 1
    lo = -margin_pkg * dpkg
    hi = 1.0 + margin_pkg * dpkg
    npkg = npkg_unit + 2 * margin_pkg
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=spacing, max_dl=spacing,
             cell_ratio=cell_ratio, box_l=[lo, lo, 0.0], box_r=[hi, hi, 0.0], seed=seed)

    def sdf(X, Y, Z):
        disc = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2) - 0.2
        return np.minimum(np.minimum(np.minimum(X, 1.0 - X), np.minimum(Y, 1.0 - Y)), disc)

    lv = make_level(sdf, 2, [lo, lo, 0.0], [dpkg, dpkg, 1.0], [npkg, npkg, 1])
    n = particle_count([lv], p)
    return Case("disc_hole_2d", p, [lv], n, steps=steps)


def box_with_corners(dim: int = 2, spacing: float = 0.02, grid: int = 64, kernel: str = "wendland",
                     h_over_dx: float = 1.3, precision: str = "fp64", seed: int = 0, lo_b: float = 0.1,
                     hi_b: float = 0.9, edges: bool = True, steps: int = 200) -> Case:
    """A box [lo_b, hi_b]^dim (phi = the distance to the nearest face inside,
    min over the faces), whose corners are the geometry's singularity points
    and, in 3D with edges=True, whose 12 edges are its segments
    (Levelset::singularity / Levelset::segment): the characteristic cells
    of the reference's level set, where particles become SINGULARITY and
    SEGMENT particles.  Constant spacing; the same unit-cube domain with
    margins as disc_hole_2d (grid cells per unit length)."""
    p = default_params(dim)
    npkg_unit = grid // 4
    dpkg = 1.0 / npkg_unit
    cell_ratio = 2.0 * h_over_dx
    margin_pkg = max(npkg_unit // 16, 1)
    while not cell_levels_consistent([-margin_pkg * dpkg] * dim, [1.0 + margin_pkg * dpkg] * dim, dim,
                                     spacing * cell_ratio, spacing * cell_ratio):
        margin_pkg += 1
    lo = -margin_pkg * dpkg
    hi = 1.0 + margin_pkg * dpkg
    npkg = npkg_unit + 2 * margin_pkg
    box_l = [lo, lo, lo if dim == 3 else 0.0]
    box_r = [hi, hi, hi if dim == 3 else 0.0]
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=spacing, max_dl=spacing,
             cell_ratio=cell_ratio, box_l=box_l, box_r=box_r, seed=seed)

    def sdf(X, Y, Z):
        out = np.minimum(np.minimum(X - lo_b, hi_b - X), np.minimum(Y - lo_b, hi_b - Y))
        if dim == 3:
            out = np.minimum(out, np.minimum(Z - lo_b, hi_b - Z))
        return out

    lv = make_level(sdf, dim, box_l, [dpkg, dpkg, dpkg if dim == 3 else 1.0],
                    [npkg, npkg, npkg if dim == 3 else 1])
    n = particle_count([lv], p)
    cs = Case(f"box_{dim}d", p, [lv], n, steps=steps)
    v = (lo_b, hi_b)
    if dim == 2:
        corners = np.array([[x, y, 0.0] for y in v for x in v])
    else:
        corners = np.array([[x, y, z] for z in v for y in v for x in v])
    cs.extra["singularities"] = corners
    if dim == 3 and edges:
        segs = []
        for a in v:
            for b_ in v:
                segs.append([lo_b, a, b_, hi_b, a, b_])   # along x
                segs.append([a, lo_b, b_, a, hi_b, b_])   # along y
                segs.append([a, b_, lo_b, a, b_, hi_b])   # along z
        cs.extra["segments"] = np.array(segs)
    return cs


def torus_3d(dx_min: float = 0.005, dx_max: float = 0.02, kernel: str = "wendland",
             h_over_dx: float = 1.3, precision: str = "fp32", seed: int = 0, steps: int = 500,
             fine_pkg: int = 64, nlevels: int = 3) -> Case:
    """Inside of a torus (R = 1, r = 0.35) in the box [-1.6, 1.6]^2 x [-0.6, 0.6]
    on nested level-set grids of fine_pkg/4, fine_pkg/2, fine_pkg packages along
    x (64/128/256 cells for fine_pkg = 64), finer levels active where |phi| is
    below 4 cells of the next-coarser level.  The box leaves one coarse package
    between the body and the seeding clamp.  Spacing dx_min..dx_max by the
    reference's tanh law."""
    p = default_params(3)
    npx0 = fine_pkg >> (nlevels - 1)
    dpkg0 = 3.2 / npx0
    npz0 = int(round(1.2 / dpkg0))
    zhalf = 0.5 * npz0 * dpkg0
    box_l = [-1.6, -1.6, -zhalf]
    box_r = [1.6, 1.6, zhalf]
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=dx_min, max_dl=dx_max,
             cell_ratio=2.0 * h_over_dx, box_l=box_l, box_r=box_r, seed=seed)
    if not cell_levels_consistent(box_l, box_r, 3, dx_max * p["cell_ratio"], dx_min * p["cell_ratio"]):
        raise ValueError("torus box gives an inconsistent cell-list level plan")

    def sdf(X, Y, Z):
        return 0.35 - np.sqrt((np.sqrt(X * X + Y * Y) - 1.0) ** 2 + Z * Z)

    levels = []
    for l in range(nlevels):
        f = 1 << l
        dp = dpkg0 / f
        lv = make_level(sdf, 3, box_l, [dp, dp, dp], [npx0 * f, npx0 * f, npz0 * f])
        if l > 0:
            lv.active = nested_active(lv, 4.0 * (dp * 2 / 4.0), 3)
        levels.append(lv)
    n = particle_count(levels, p)
    return Case("torus_3d", p, levels, n, steps=steps)


def spheres_3d(n_spheres: int = 32, seed: int = 7, dx_min: float = 0.0025, dx_max: float = 0.012,
               middle_dl: float = 0.004, radii=(0.05, 0.3), fine_pkg: int = 64, nlevels: int = 3,
               kernel: str = "wendland", h_over_dx: float = 1.3, precision: str = "fp32",
               steps: int = 500) -> Case:
    """Union of n_spheres spheres, radii log-uniform in `radii`, centres
    uniform in [0, 1]^3, phi = max_k (r_k - |x - c_k|), on nested level sets of
    fine_pkg >> (nlevels - 1) ... fine_pkg packages per axis over the box
    [-0.45, 1.45]^3 (4 cells per package; finer levels active within 4 cells
    of the next-coarser level's surface), curvature spacing law (law 1):
    dx_min at the sharpest interface features, middle_dl at the flattest,
    growing with phi to dx_max."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.uniform(np.log(radii[0]), np.log(radii[1]), n_spheres))
    c = rng.random((n_spheres, 3))

    def sdf(X, Y, Z):
        # X, Y, Z broadcastable axes; each sphere adds ((x-cx)^2 + (y-cy)^2) +
        # (z-cz)^2 in that order, square root, r - d, running maximum
        # slabs of z planes small enough to stay in cache, operations in place
        shape = np.broadcast_shapes(np.shape(X), np.shape(Y), np.shape(Z))
        out = np.full(shape, -1.0e9)
        nz = shape[0]
        plane = int(np.prod(shape[1:]))
        step = max(1, (1 << 21) // max(plane, 1))
        zs = np.broadcast_to(Z, (nz, 1, 1))
        ys = np.broadcast_to(Y, (1,) + (shape[1], 1))
        for (cx, cy, cz), rk in zip(c, r):
            dx = X - cx
            dy = ys - cy
            dxy = dx * dx + dy * dy  # (1, ny, nx)
            dz = zs - cz
            dz2 = dz * dz
            for z0 in range(0, nz, step):
                z1 = min(nz, z0 + step)
                tmp = dxy + dz2[z0:z1]
                np.sqrt(tmp, out=tmp)
                np.subtract(rk, tmp, out=tmp)
                np.maximum(out[z0:z1], tmp, out=out[z0:z1])
        return out

    p = default_params(3)
    npx0 = fine_pkg >> (nlevels - 1)
    box_l = [-0.45] * 3
    box_r = [1.45] * 3
    dpkg0 = 1.9 / npx0
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=dx_min, max_dl=dx_max,
             cell_ratio=2.0 * h_over_dx, box_l=box_l, box_r=box_r, seed=seed, scale_law=1, middle_dl=middle_dl)
    if not cell_levels_consistent(box_l, box_r, 3, dx_max * p["cell_ratio"], dx_min * p["cell_ratio"]):
        raise ValueError("spheres box gives an inconsistent cell-list level plan")
    levels = []
    for l in range(nlevels):
        f = 1 << l
        dp = dpkg0 / f
        lv = make_level(sdf, 3, box_l, [dp, dp, dp], [npx0 * f] * 3, broadcast=True)
        if l > 0:
            lv.active = nested_active(lv, 4.0 * (dp * 2 / 4.0), 3)
        levels.append(lv)
    n = particle_count(levels, p)
    cs = Case("spheres_3d", p, levels, n, steps=steps)
    cs.extra["spheres"] = (c, r)
    return cs


def star_shape(dim: int, seed: int, n_target: int, kernel: str = "wendland", h_over_dx: float = 1.3,
               precision: str = "fp32") -> Case:
    """A random star-shaped body: r = r0 (1 + sum_k a_k g_k(direction)) with
    M = 8..32 harmonics, sum |a_k| <= 0.3, phi = r(direction) - |x| (positive
    inside; not an exact distance away from the surface).  2D: g_k =
    cos(k theta + phase) on a 128^2 grid; 3D: g_k = sin(pol)^p cos(p az +
    phase) cos(q pol + phase') on a 64^3 grid (continuous at the poles).
    Constant spacing chosen so that the spacing integral is about n_target."""
    rng = np.random.default_rng(seed)
    M = int(rng.integers(8, 33))
    a = rng.random(M)
    a *= 0.3 * (0.5 + 0.5 * rng.random()) / a.sum()
    ph = rng.uniform(0.0, 2 * np.pi, M)
    r0 = 1.0
    if dim == 2:
        ks = np.arange(1, M + 1)

        def radius(X, Y, Z):
            th = np.arctan2(Y, X)
            r = np.ones_like(th)
            for k, ak, pk in zip(ks, a, ph):
                r += ak * np.cos(k * th + pk)
            return r0 * r
    else:
        pk_ = rng.integers(1, 7, M)
        qk_ = rng.integers(0, 7, M)
        ph2 = rng.uniform(0.0, 2 * np.pi, M)

        def radius(X, Y, Z):
            az = np.arctan2(Y, X)
            pol = np.arctan2(np.sqrt(X * X + Y * Y), Z)
            sp = np.sin(pol)
            r = np.ones_like(az)
            for ak, p_, q_, f1, f2 in zip(a, pk_, qk_, ph, ph2):
                r += ak * sp ** p_ * np.cos(p_ * az + f1) * np.cos(q_ * pol + f2)
            return r0 * r

    def sdf(X, Y, Z):
        return radius(X, Y, Z) - np.sqrt(X * X + Y * Y + Z * Z)

    npk = 32 if dim == 2 else 16          # 128^2 / 64^3 interior cells
    half = 1.5 * r0                        # body within 1.3 r0; one package of clearance
    dpkg = 2 * half / npk
    box_l = [-half, -half, -half if dim == 3 else 0.0]
    box_r = [half, half, half if dim == 3 else 0.0]
    # volume of the body from sampled directions, for the spacing
    u = rng.normal(size=(20000, 3))
    if dim == 2:
        u[:, 2] = 0.0
    u /= np.linalg.norm(u, axis=1)[:, None]
    rr = radius(u[:, 0], u[:, 1], u[:, 2])
    vol = np.pi * np.mean(rr ** 2) if dim == 2 else 4.0 / 3.0 * np.pi * np.mean(rr ** 3)
    dx = (vol / n_target) ** (1.0 / dim)
    p = default_params(dim)
    cell_ratio = 2.0 * h_over_dx
    while not cell_levels_consistent(box_l, box_r, dim, dx * cell_ratio, dx * cell_ratio):
        dx *= 1.001
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=dx, max_dl=dx,
             cell_ratio=cell_ratio, box_l=box_l, box_r=box_r, seed=seed)
    num = [npk, npk, npk if dim == 3 else 1]
    lv = make_level(sdf, dim, box_l, [dpkg, dpkg, dpkg if dim == 3 else 1.0], num)
    n = particle_count([lv], p)
    return Case(f"star_{dim}d_{seed}", p, [lv], n, steps=300)


def _star_job(job):
    dim, seed, n, precision = job
    return star_shape(dim, seed, n, precision=precision)


def star_batch(count: int = 512, seed: int = 11, n_min: int = 2000, n_max: int = 200000,
               precision: str = "fp32", workers: int = 1) -> List[Case]:
    """count independent star-shaped geometries, even indices 2D and odd 3D,
    particle counts log-uniform in [n_min, n_max] (about 20M in total for
    512 geometries).  workers > 1 builds them in that many spawned processes
    (spawned, so a caller that already uses the GPU is not forked)."""
    rng = np.random.default_rng(seed)
    targets = np.exp(rng.uniform(np.log(n_min), np.log(n_max), count))
    jobs = [(2 if g % 2 == 0 else 3, seed * 100003 + g, int(targets[g]), precision) for g in range(count)]
    if workers > 1 and count > 1:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(min(workers, count)) as pool:
            return pool.map(_star_job, jobs, chunksize=4)
    return [_star_job(j) for j in jobs]


def _ellipse_root(r0, z0, z1, g, iters=160):
    """Bisection for the root s of (r0 z0/(s+r0))^2 + (z1/(s+1))^2 = 1 on
    [z1 - 1, |(r0 z0, z1)| - 1] (Eberly, "Distance from a point to an
    ellipse, an ellipsoid, or a hyperellipsoid", 2013), vectorised; stops per
    point when the midpoint no longer moves."""
    n0 = r0 * z0
    s0 = z1 - 1.0
    s1 = np.where(g < 0, 0.0, np.hypot(n0, z1) - 1.0)
    s = 0.5 * (s0 + s1)
    live = np.ones_like(s, dtype=bool)
    for _ in range(iters):
        s = np.where(live, 0.5 * (s0 + s1), s)
        live &= (s != s0) & (s != s1)
        if not live.any():
            break
        gg = (n0 / (s + r0)) ** 2 + (z1 / (s + 1.0)) ** 2 - 1.0
        s0 = np.where(live & (gg > 0), s, s0)
        s1 = np.where(live & (gg < 0), s, s1)
        live &= gg != 0
    return s


def ellipse_distance(px, py, cx, cy, a, b, ang):
    """Signed distance from points to an ellipse (semi-axes a >= b, rotated by
    ang about its centre), positive outside: Eberly's robust method in the
    first quadrant of the ellipse frame."""
    ca, sa = np.cos(ang), np.sin(ang)
    dx, dy = px - cx, py - cy
    y0 = np.abs(ca * dx + sa * dy)
    y1 = np.abs(-sa * dx + ca * dy)
    e0, e1 = a, b
    dist = np.empty_like(y0)
    m_a = (y1 > 0) & (y0 > 0)
    z0 = y0[m_a] / e0
    z1 = y1[m_a] / e1
    g = z0 * z0 + z1 * z1 - 1.0
    r0 = (e0 / e1) ** 2
    sbar = _ellipse_root(r0, z0, z1, g)
    x0 = r0 * y0[m_a] / (sbar + r0)
    x1 = y1[m_a] / (sbar + 1.0)
    dist[m_a] = np.where(g != 0, np.hypot(x0 - y0[m_a], x1 - y1[m_a]), 0.0)
    m_b = (y1 > 0) & ~(y0 > 0)
    dist[m_b] = np.abs(y1[m_b] - e1)
    m_c = ~(y1 > 0)
    numer0 = e0 * y0[m_c]
    denom0 = e0 * e0 - e1 * e1
    inside = numer0 < denom0
    xde0 = np.where(inside, numer0 / max(denom0, 1e-300), 1.0)
    d_in = np.hypot(e0 * xde0 - y0[m_c], e1 * np.sqrt(np.maximum(1.0 - xde0 * xde0, 0.0)))
    dist[m_c] = np.where(inside, d_in, np.abs(y0[m_c] - e0))
    outside = (y0 / e0) ** 2 + (y1 / e1) ** 2 > 1.0
    return np.where(outside, dist, -dist)


def ellipses_2d(n_ellipses: int = 64, seed: int = 11, dx_min: float = 0.0005, dx_max: float = 0.004,
                grid: int = 1024, axes=(0.01, 0.05), kernel: str = "wendland", h_over_dx: float = 1.3,
                precision: str = "fp32", steps: int = 400) -> Case:
    """Unit square minus non-overlapping random ellipses (semi-axes uniform in
    `axes`, uniform orientation; rejection of overlapping bounding circles,
    0.01 apart, and of circles within 0.02 of the square), exact signed
    distance by Eberly's method; spacing dx_min..dx_max by the reference's
    tanh law.  grid cells per unit length; the domain adds grid/16 cells (or
    more, for a consistent cell-list plan) on every side."""
    rng = np.random.default_rng(seed)
    el = []
    tries = 0
    while len(el) < n_ellipses and tries < 200000:
        tries += 1
        a, b = np.sort(rng.uniform(axes[0], axes[1], 2))[::-1]
        cx, cy = rng.uniform(0.02 + a, 0.98 - a, 2)
        if all(np.hypot(cx - e[0], cy - e[1]) > a + e[2] + 0.01 for e in el):
            el.append((cx, cy, a, b, rng.uniform(0.0, np.pi)))
    p = default_params(2)
    npkg_unit = grid // 4
    dpkg = 1.0 / npkg_unit
    cell_ratio = 2.0 * h_over_dx
    margin_pkg = max(npkg_unit // 16, 1)
    while not cell_levels_consistent([-margin_pkg * dpkg] * 2, [1.0 + margin_pkg * dpkg] * 2, 2,
                                     dx_max * cell_ratio, dx_min * cell_ratio):
        margin_pkg += 1
    lo, hi = -margin_pkg * dpkg, 1.0 + margin_pkg * dpkg
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=dx_min, max_dl=dx_max,
             cell_ratio=cell_ratio, box_l=[lo, lo, 0.0], box_r=[hi, hi, 0.0], seed=seed)
    window = 0.25

    def sdf(X, Y, Z):
        phi = np.minimum(np.minimum(X, 1.0 - X), np.minimum(Y, 1.0 - Y))
        for (cx, cy, a, b, ang) in el:
            near = (np.abs(X - cx) < a + window) & (np.abs(Y - cy) < a + window)
            lower = np.hypot(X[near] - cx, Y[near] - cy) - a  # distance to the ellipse >= this
            cur = phi[near]
            need = lower < cur
            d = cur.copy()
            d[need] = np.minimum(cur[need], ellipse_distance(X[near][need], Y[near][need], cx, cy, a, b, ang))
            phi[near] = d
        return phi

    lv = make_level(sdf, 2, [lo, lo, 0.0], [dpkg, dpkg, 1.0], [npkg_unit + 2 * margin_pkg] * 2 + [1])
    n = particle_count([lv], p)
    c = Case("ellipses_2d", p, [lv], n, steps=steps)
    c.extra["ellipses"] = el
    return c


def case_by_name(name: str, **kw) -> Case:
    if name == "disc_hole_2d":
        return disc_hole_2d(**kw)
    if name == "torus_3d":
        return torus_3d(**kw)
    raise KeyError(name)


def restart_num_particles(total_mass: float, total_mass_surface: float, total_mass_segment: float,
                          num_singularity: int, num_interface_cell: int) -> int:
    """SPH_mesh_generation::Get_num_particles (sph_mesh_generation.cpp:900-930)
    over a level set's totals: one particle per singularity point; segment,
    surface and interior counts each less half the next-lower-dimensional
    mass, truncated and at least 0; the surface count at most the number of
    interface cells."""
    seg = max(int(total_mass_segment - 0.5 * num_singularity), 0)
    surf = max(int(total_mass_surface - 0.5 * total_mass_segment), 0)
    surf = min(surf, int(num_interface_cell))
    mesh = max(int(total_mass - 0.5 * total_mass_surface), 0)
    return mesh + surf + int(num_singularity) + seg


# The factors of the reference's restart run that re-targets the spacing
# (_READ_TARGET_FIELD_, sph_mesh_generation.cpp:658-666): minimum, middle and
# maximum spacing in cells of the level set (level_set.cpp:939-941).
RETARGET_FACTORS = (2.0, 5.0, 16.0)


def from_lset_restart(path: str, kernel: str = "wendland", h_over_dx: float = 1.3, precision: str = "fp32",
                      seed: int = 0, scale_law: int = 0, retarget: Optional[Sequence[float]] = None) -> Case:
    """A case from a level-set restart (rstfile/levelset.rst, the layout of
    Levelset::Save_lset_restart_file, level_set.cpp:1022-1094, read by
    Load_lset_restart_file, :1098-1175, and Load_level_set_rstfile,
    lset_level_infor.cpp:932-1080): the domain, the level's packages and the
    interior cells' phi, the spacing bounds and middle spacing, and the
    singularity points and segments.

    The file holds the interior cells only.  The reference fills the margin
    packages from its analytic geometry before reading the file
    (Levelset::Initialize); here a margin cell takes the phi of the nearest
    interior cell minus its distance to that cell, i.e. a distance field
    continued outward.  The particle count is the reference's restart count,
    Get_num_particles over the file's totals (restart_num_particles).

    retarget = (fac_min, fac_mid, fac_max) (RETARGET_FACTORS are the
    reference's) is the restart run that re-targets the spacing: minimum,
    middle and maximum spacing become the factors times the level's cell
    size, and the count is the spacing integral of the new law;
    Initialize_case(cut_cell_count=True) seeds Get_num_particles over the
    recomputed cut-cell totals, as that run does."""
    from .io import load_lset_restart
    r = load_lset_restart(path)
    dim = int(r["dim"])
    m = int(r["num_pkg_margin"][0])
    npkg = [int(r["num_pkg"][d]) if d < dim else 1 for d in range(3)]
    dpkg = [float(r["dpkg"][d]) for d in range(3)]
    dcell = [float(r["dcell"][d]) for d in range(3)]
    box_l = [float(r["box_l"][d]) if d < dim else 0.0 for d in range(3)]
    box_r = [float(r["box_r"][d]) if d < dim else 0.0 for d in range(3)]
    inner = np.asarray(r["phi"], dtype=np.float64)
    pad = [4 * m if d < dim else 0 for d in range(3)]
    shape = tuple(inner.shape[a] + 2 * pad[2 - a] for a in range(3))
    # nearest interior index and the offset to it, per axis (arrays are z, y, x)
    idx, off = [], []
    for a in range(3):
        d = 2 - a
        g = np.arange(shape[a]) - pad[d]
        c = np.clip(g, 0, inner.shape[a] - 1)
        idx.append(c)
        off.append((g - c) * (dcell[d] if d < dim else 0.0))
    # open-mesh gather and offsets (no full-size index arrays), summed in x, y, z order
    dz, dy, dx = off[0][:, None, None], off[1][None, :, None], off[2][None, None, :]
    phi = inner[np.ix_(*idx)] - np.sqrt(dx * dx + dy * dy + dz * dz)
    lv = LevelGrid(box_l, dpkg, npkg, m, np.ascontiguousarray(phi), None)
    p = default_params(dim)
    cell_ratio = 2.0 * h_over_dx
    min_dl, max_dl, mid_dl = float(r["minimum_dl"]), float(r["maximum_dl"]), float(r["middel_dl"])
    if retarget is not None:
        dl = min(dcell[d] for d in range(dim))
        min_dl, mid_dl, max_dl = (float(f) * dl for f in retarget)
    if not cell_levels_consistent(box_l, box_r, dim, max_dl * cell_ratio, min_dl * cell_ratio):
        raise ValueError("the restart's domain and spacing give an inconsistent cell-list level plan "
                         "(sph.cpp:144-180); choose another h_over_dx")
    p.update(kernel=KERNELS[kernel], precision=PRECISIONS[precision], min_dl=min_dl, max_dl=max_dl,
             cell_ratio=cell_ratio, box_l=box_l, box_r=box_r, seed=seed, scale_law=scale_law,
             middle_dl=mid_dl)
    if retarget is not None:
        n = particle_count([lv], p)
    else:
        n = restart_num_particles(r["total_mass"], r["total_mass_surface"], r["total_mass_segment"],
                                  len(r["singularities"]), r["glbl_num_interface_cell"])
    cs = Case("lset_restart", p, [lv], n)
    if len(r["singularities"]):
        cs.extra["singularities"] = np.asarray(r["singularities"])
    if len(r["segments"]):
        cs.extra["segments"] = np.asarray(r["segments"])
    return cs
