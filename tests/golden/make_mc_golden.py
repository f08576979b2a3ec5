"""Generates tests/golden/mc_reference.npz from the reference's own
marching-cubes polygoniser (geometry_tools/polygonise.cpp, built by
oracle/build_ref.py into oracle/_ref/).  Run where the reference sources
exist:  python tests/golden/make_mc_golden.py

Contents:
  case_polygons [256, 4] int16: per sign case (bit v set: cube vertex v below
      zero), the reference's polygons as 12-bit masks of the cube edges they
      cut, ascending, 0 padded;
  case_ntri [256] int8: the reference's triangle count per sign case;
  lattices [n, 27], h [n], kind [n]: seeded 3x3x3 corner lattices ([x][y][z]
      on a half-cell grid of cell size h) of planes (kind 0) and spheres
      (kind 1) through the cell;
  area [n]: the reference's get_area_MQ of each lattice (its polygoniser and
      get_area_tri, geometry_calculator.cpp:283-350).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

V = [(0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1)]
E = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5), (2, 6), (3, 7)]


def polygons_of(tris):
    """Edge sets (bit masks) of the connected triangle fans in tris (lists of edge triples)."""
    comps = []
    for t in tris:
        m = sum(1 << e for e in t)
        hit = [c for c in comps if c & m]
        for c in hit:
            comps.remove(c)
            m |= c
        comps.append(m)
    return sorted(comps)


def main():
    lib_path = build_ref.build(force=True)
    if lib_path is None:
        raise SystemExit("reference sources not found")
    R = C.CDLL(lib_path)
    R.refp_polygonise.argtypes = [C.c_void_p] * 3
    R.refp_area_mq.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
    R.refp_area_mq.restype = C.c_double
    mid = {}
    for k, (a, b) in enumerate(E):
        mid[tuple((np.array(V[a]) + np.array(V[b])) / 2.0)] = k
    p = np.array(V, dtype=np.float64).ravel()
    case_polygons = np.zeros((256, 4), dtype=np.int16)
    case_ntri = np.zeros(256, dtype=np.int8)
    for ci in range(256):
        val = np.array([-1.0 if (ci >> v) & 1 else 1.0 for v in range(8)])
        tr = np.zeros(45)
        n = R.refp_polygonise(p.ctypes.data, val.ctypes.data, tr.ctypes.data)
        tris = [[mid[tuple(np.round(tr[9 * q + 3 * k: 9 * q + 3 * k + 3], 9))] for k in range(3)] for q in range(n)]
        polys = polygons_of(tris)
        case_ntri[ci] = n
        case_polygons[ci, :len(polys)] = polys
    rng = np.random.default_rng(20240611)
    lat, hs, kinds, areas = [], [], [], []
    g = np.array([(i, j, k) for i in range(3) for j in range(3) for k in range(3)], dtype=np.float64)
    while len(lat) < 600:
        h = float(rng.choice([0.01, 0.02, 0.05]))
        x = (g - 1.0) * 0.5 * h  # half-cell lattice around the cell centre
        kind = len(lat) % 2
        if kind == 0:
            nrm = rng.normal(size=3)
            nrm /= np.linalg.norm(nrm)
            phi = x @ nrm - rng.uniform(-0.4, 0.4) * h
        else:
            r = rng.uniform(1.5, 30.0) * h
            d = rng.normal(size=3)
            d /= np.linalg.norm(d)
            c = d * (r + rng.uniform(-0.4, 0.4) * h)
            phi = r - np.linalg.norm(x - c, axis=1)
        if (phi > 0).all() or (phi < 0).all():
            continue
        c27 = np.ascontiguousarray(phi)
        lat.append(c27)
        hs.append(h)
        kinds.append(kind)
        areas.append(R.refp_area_mq(c27.ctypes.data, h, h, h))
    np.savez_compressed(os.path.join(HERE, "mc_reference.npz"), case_polygons=case_polygons, case_ntri=case_ntri,
                        lattices=np.array(lat), h=np.array(hs), kind=np.array(kinds, dtype=np.int8),
                        area=np.array(areas))
    print("wrote", os.path.join(HERE, "mc_reference.npz"), len(lat), "lattices")


if __name__ == "__main__":
    main()
