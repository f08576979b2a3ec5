"""Writes tests/golden/aabb_reference.npz: segment-in-box lengths computed by
the reference's own AABB_calculator.cpp (compiled from its sources into
oracle/_ref/libref_aabb.so by oracle/build_ref.py), the term of the SEGMENT
cells in the cut-cell pass (GeometryCalculator::Get_segment_length).

Cases: cells of a level-set grid against random segments, segments along the
grid axes (the edges of a box geometry: parallel to two slabs, so the slab
tests see infinities, and NaNs where an end lies on a cell face), segments
inside one cell, missing the cell, touching a face or an edge, and of zero
length."""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def cases(seed: int = 3):
    rng = np.random.default_rng(seed)
    mn, mx, v0, v1 = [], [], [], []

    def add(a, b, p, q):
        mn.append(a); mx.append(b); v0.append(p); v1.append(q)
    dc = 1.0 / 64
    for _ in range(400):  # random segments through random cells
        c = rng.integers(0, 64, 3) * dc
        p = c + rng.uniform(-2 * dc, 3 * dc, 3)
        q = c + rng.uniform(-2 * dc, 3 * dc, 3)
        add(c, c + dc, p, q)
    for ax in range(3):  # axis-aligned edges (box [0.1, 0.9]^3)
        for a in (0.1, 0.9):
            for b in (0.1, 0.9):
                p = np.array([a, b, 0.1]); q = np.array([a, b, 0.9])
                p = np.roll(p, ax + 1); q = np.roll(q, ax + 1)
                for _ in range(30):
                    c = np.floor(p / dc) * dc + rng.integers(-1, 2, 3) * dc
                    c[ax] = rng.integers(0, 64) * dc
                    add(c, c + dc, p, q)
    for _ in range(60):  # ends on cell faces, touching faces and edges
        c = rng.integers(0, 64, 3) * dc
        p = c.copy(); q = c + dc * rng.integers(0, 2, 3)
        add(c, c + dc, p, q)
        add(c, c + dc, c + dc * np.array([1.0, 0.5, 0.5]), c + dc * np.array([1.0, 2.0, 0.5]))
    for _ in range(20):  # zero length, inside and outside
        c = rng.integers(0, 64, 3) * dc
        p = c + dc * rng.uniform(-1, 2, 3)
        add(c, c + dc, p, p.copy())
    return (np.array(mn), np.array(mx), np.array(v0), np.array(v1))


def reference_lengths(mn, mx, v0, v1):
    import build_ref
    lib = ctypes.CDLL(build_ref.build_aabb())
    f = lib.ref_segment_length
    f.restype = ctypes.c_double
    f.argtypes = [ctypes.c_void_p] * 4
    out = np.zeros(len(mn))
    for i in range(len(mn)):
        a = [np.ascontiguousarray(x[i], dtype=np.float64) for x in (mn, mx, v0, v1)]
        out[i] = f(*[x.ctypes.data for x in a])
    return out


if __name__ == "__main__":
    mn, mx, v0, v1 = cases()
    L = reference_lengths(mn, mx, v0, v1)
    np.savez_compressed(os.path.join(HERE, "aabb_reference.npz"), mn=mn, mx=mx, v0=v0, v1=v1, length=L)
    print(len(L), "cases;", int((L > 0).sum()), "non-zero")
