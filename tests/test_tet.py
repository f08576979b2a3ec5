"""3D tetrahedralisation (Graphmeshcls::Reconstruct_tets, geometry_tools/
graph_mesh.cpp:981-1100; Check_whether_this_tet_should_be_delete, :675-979;
Tet_quality_statistics, :1967-2400) on the CPU: the oracle's certified
local Delaunay tets pinned against qhull's Delaunay tetrahedralisation
(scipy) of the same snapped points.

* Every oracle tet is a qhull tet, none twice, and every qhull tet whose
  circumsphere lies inside the neighbour ball of one of its particles is
  found: kept, or dropped by the reference's deletion rule (all four
  particles not REAL and aspect ratio above 10).
* The quality statistics equal a numpy evaluation of the same tets.
"""
import numpy as np
import pytest

import oracle

Delaunay = pytest.importorskip("scipy.spatial").Delaunay
cKDTree = pytest.importorskip("scipy.spatial").cKDTree


def _rows(x, h, cutoff):
    """Neighbour rows of the engine's rule: dist <= cutoff max(h_i, h_j) + 1e-10."""
    tr = cKDTree(x)
    cand = tr.query_ball_point(x, cutoff * h.max() + 1e-9)
    off, lst = [0], []
    for i, js in enumerate(cand):
        js = np.array(sorted(js))
        d = np.linalg.norm(x[js] - x[i], axis=1)
        lst += list(js[d <= cutoff * np.maximum(h[i], h[js]) + 1e-10])
        off.append(len(lst))
    return np.array(off, dtype=np.int64), np.array(lst, dtype=np.int32)


def _lattice(k, seed):
    rng = np.random.default_rng(seed)
    dx = 1.0 / k
    g = (np.stack(np.meshgrid(*[np.arange(k)] * 3, indexing="ij"), -1).reshape(-1, 3) + 0.5) * dx
    return g + rng.uniform(-0.3, 0.3, g.shape) * dx, dx


def _ball(k, seed):
    """Jittered lattice inside a ball of radius 0.4 (REAL) and a Fibonacci
    sphere of surface particles on it (SURFACE)."""
    x, dx = _lattice(k, seed)
    rng = np.random.default_rng(seed + 1)
    c = np.array([0.5, 0.5, 0.5])
    inner = x[np.linalg.norm(x - c, axis=1) < 0.4 - 0.5 * dx]
    m = int(4 * np.pi * 0.4 ** 2 / dx ** 2)
    i = np.arange(m) + 0.5
    phi = np.arccos(1 - 2 * i / m)
    th = np.pi * (1 + 5 ** 0.5) * i
    s = c + 0.4 * np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], -1)
    # surface particles a little off the sphere, as relaxed ones are: flat
    # tets of four of them then have small circumspheres
    s = c + (s - c) * (1 + rng.uniform(-0.05, 0.05, (m, 1)) * dx / 0.4)
    xyz = np.concatenate([inner, s])
    typ = np.concatenate([np.zeros(len(inner), np.int32), np.ones(len(s), np.int32)])
    return xyz, typ, dx


def _circ(P):
    A = P[:3] - P[3]
    c = np.linalg.solve(A, 0.5 * (A * A).sum(1))
    return P[3] + c, np.linalg.norm(c)


def _aspect(P):
    A = P[:3] - P[3]
    det = np.dot(A[0], np.cross(A[1], A[2]))
    n = [np.cross(A[1], A[2]) / det, np.cross(A[2], A[0]) / det, np.cross(A[0], A[1]) / det]
    n.append(-(n[0] + n[1] + n[2]))
    e = [P[a] - P[b] for a in range(4) for b in range(a + 1, 4)]
    return np.sqrt(max(np.dot(v, v) for v in e)) * max(np.linalg.norm(v) for v in n), n, det


@pytest.mark.parametrize("kind", ["lattice", "ball"])
def test_oracle_tets_pinned_against_qhull(kind):
    if kind == "lattice":
        x, dx = _lattice(10, 1)
        typ = np.zeros(len(x), np.int32)
    else:
        x, typ, dx = _ball(12, 2)
    h = np.full(len(x), 1.3 * dx)
    cutoff = 2.0
    off, nb = _rows(x, h, cutoff)
    tets, q = oracle.tetrahedralize(x, typ, h, off, nb, cutoff, [0, 0, 0], [1, 1, 1])
    xs = oracle.snap(x, [0, 0, 0], [1, 1, 1])
    qh = set(map(tuple, np.sort(Delaunay(xs).simplices, axis=1)))
    mine = [tuple(t) for t in tets]
    assert all(list(t) == sorted(t) for t in mine)
    assert len(set(mine)) == len(mine) and set(mine) <= qh
    held, dropped = set(), 0
    for t in qh:
        P = xs[list(t)]
        c, r = _circ(P)
        if any(np.linalg.norm(c - xs[v]) + r <= cutoff * h[v] * (1 - 1e-5) for v in t):
            held.add(t)
            if all(typ[v] != 0 for v in t) and _aspect(P)[0] > 10.0:
                dropped += 1
    assert len(held - set(mine)) == dropped == q["ndeleted"]
    assert q["ntie"] == 0 and q["ntrunc"] == 0 and q["ntet"] == len(mine) > 4 * len(x) // 2
    if kind == "ball":
        assert dropped > 0
    # quality statistics against numpy
    vols, asp, rr, dmin, dmax, dih = [], [], [], [], [], []
    for t in mine:
        P = xs[list(t)]
        a, n, det = _aspect(P)
        H = [np.linalg.norm(v) for v in n]
        u = [v / np.linalg.norm(v) for v in n]
        ang = [np.arccos(np.clip(-np.dot(u[i], u[j]), -1, 1)) / 3.1415926 * 180.0 for i in range(4)
               for j in range(i + 1, 4)]
        vols.append(abs(det) / 6)
        asp.append(a)
        rr.append(3.0 / sum(H) / _circ(P)[1])
        dmin.append(min(ang))
        dmax.append(max(ang))
        dih += ang
    assert abs(q["total_volume"] - sum(vols)) <= 1e-12 * sum(vols)
    assert np.isclose(q["max_aspect"], max(asp), rtol=1e-9) and np.isclose(q["min_aspect"], min(asp), rtol=1e-9)
    assert np.isclose(q["avg_aspect"], np.mean(asp), rtol=1e-9)
    assert np.isclose(q["avg_radius_ratio"], np.mean(rr), rtol=1e-9)
    assert np.isclose(q["min_dihedral"], min(dmin), atol=1e-7) and np.isclose(q["max_dihedral"], max(dmax), atol=1e-7)
    tab = [1.5, 2.0, 2.5, 3.0, 4.0, 6.0, 10.0, 15.0, 25.0, 50.0, 100.0]
    assert q["aspect_hist"] == list(np.bincount(np.searchsorted(tab, asp, side="left"), minlength=12))
    assert sum(q["radius_hist"]) == len(mine) and sum(q["dihedral_hist"]) == 6 * len(mine)
    want = np.bincount(np.minimum(np.floor(np.array(dih) / 4.0).astype(int), 44), minlength=45)
    assert np.abs(np.array(q["dihedral_hist"]) - want).max() <= 1  # bin edges by cosine vs by angle
    assert q["nsmall_dihedral"] == [int(np.sum(np.array(dmin) < a)) for a in (10, 20, 30, 40)]


def test_oracle_tets_on_relaxed_particles_pinned_against_qhull():
    """The same pins on particles the oracle relaxed (a box whose corners
    and edges are singularity points and segments, 30 steps, the oracle's
    own neighbour rows): every tet is a qhull tet, none twice, and every
    qhull tet whose circumsphere lies in one of its particles' balls is
    found or dropped by the deletion rule."""
    from mrsph import cases
    case = cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic", h_over_dx=1.0)
    o = oracle.Oracle(case)
    n = case.n_particles
    o.alloc(n)
    o.seed(n)
    o.pre_run()
    o.steps(30)
    st = o.get_state()
    xyz = np.stack([st["x"], st["y"], st["z"]], 1)
    typ, h = st["type"].astype(np.int32), st["h"]
    assert (typ == 1).any() and (typ == 3).any()
    off, nb = o.neighbors()
    p = case.params
    tets, q = oracle.tetrahedralize(xyz, typ, h, off, nb, p["cutoff"], p["box_l"], p["box_r"])
    xs = oracle.snap(xyz, p["box_l"], p["box_r"])
    simp = np.sort(Delaunay(xs).simplices, axis=1)
    qh = set(map(tuple, simp))
    mine = set(map(tuple, tets))
    assert len(mine) == len(tets) > 5 * n and mine <= qh
    P = xs[simp]
    A = P[:, :3] - P[:, 3:4]
    c = P[:, 3] + np.linalg.solve(A, 0.5 * (A * A).sum(2)[..., None])[..., 0]
    r = np.linalg.norm(c - P[:, 3], axis=1)
    held = np.zeros(len(simp), bool)
    for k in range(4):
        held |= np.linalg.norm(c - P[:, k], axis=1) + r <= p["cutoff"] * h[simp[:, k]] * (1 - 1e-5)
    missing = [tuple(t) for t in simp[held] if tuple(t) not in mine]
    dropped = [t for t in missing if all(typ[v] != 0 for v in t) and _aspect(xs[list(t)])[0] > 10.0]
    assert len(missing) == len(dropped) == q["ndeleted"] and q["ntie"] == 0 and q["ntrunc"] == 0
    # the mesh writer's per-tet fields (io.tet_quality) against the quality pass
    from mrsph import io
    vol, asp, rr, mind = io.tet_quality(xs, tets)
    assert np.isclose(vol.sum(), q["total_volume"], rtol=1e-12)
    assert np.isclose(asp.max(), q["max_aspect"], rtol=1e-12) and np.isclose(asp.mean(), q["avg_aspect"], rtol=1e-12)
    assert np.isclose(rr.min(), q["min_radius_ratio"], rtol=1e-12)
    assert np.isclose(rr.mean(), q["avg_radius_ratio"], rtol=1e-12)
    assert np.isclose(mind.min(), q["min_dihedral"], rtol=1e-12)
    assert np.isclose(mind.mean(), q["avg_min_dihedral"], rtol=1e-12)
