"""Generates tests/golden/kernels_reference.npz from the reference's own
particle.cpp (the smoothing kernels, their gradients and Set_particle_scale),
compiled by oracle/build_ref.py into oracle/_ref/libref_kernels_*.so.  Run
where the reference sources exist:  python tests/golden/make_kernel_golden.py

Contents (FP64, produced by the reference's code):
  dist [m], h [3]: seeded distances over [0, 2.2 h_max] plus the edge points
      0, h, 2h and 2h one ulp either side, for each smoothing length h;
  W_<D>d_<kernel>_<which> [3, m], dW_<D>d_<kernel>_<which> [3, m]: for the
      build of dimension D (_DIM2_ / _DIM3_) and each kernel macro, which = 0
      Kernel_function / Derivative_kernel_function (the build's DIM), 1, 2, 3
      the explicit _1D / _2D / _3D variants (particle.cpp:31-807);
  scale_in [k, 4] (h, scale, max_scale, min_scale), scale_out [k], scale_flag
      [k]: Particle_base::Set_particle_scale (particle.cpp:957-975).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

OUT = os.path.join(HERE, "kernels_reference.npz")
H = np.array([0.013, 0.0029, 0.07])


def inputs():
    rng = np.random.default_rng(2024)
    dist = np.sort(rng.random(240)) * 2.2 * H.max()
    return dist


def edge_points(h):
    two = 2.0 * h
    return np.array([0.0, h, two, np.nextafter(two, 0.0), np.nextafter(two, 4.0), np.nextafter(h, 0.0)])


def scale_inputs():
    rng = np.random.default_rng(7)
    rows = []
    for _ in range(400):
        max_scale = 0.05 * 2.0 ** rng.integers(0, 3)
        min_scale = max_scale / 2.0 ** rng.integers(1, 6)
        scale = max_scale / 2.0 ** rng.integers(0, 7)
        h = rng.uniform(0.3, 1.2) * max_scale * 2.0 ** -rng.integers(0, 6)
        rows.append((h, scale, max_scale, min_scale))
    # exactly on the bracket edges h * 2 == scale and h * 2 == scale / 2
    rows += [(0.025, 0.05, 0.1, 0.0125), (0.0125, 0.05, 0.1, 0.0125), (0.05, 0.1, 0.1, 0.0125)]
    return np.array(rows)


class Quiet:
    """Silences the reference's own prints (the Wendland 1D message) on fd 1."""

    def __enter__(self):
        sys.stdout.flush()
        self.saved = os.dup(1)
        self.null = os.open(os.devnull, os.O_WRONLY)
        os.dup2(self.null, 1)

    def __exit__(self, *a):
        C.CDLL(None).fflush(None)  # the C/C++ stdout buffer, before fd 1 is restored
        os.dup2(self.saved, 1)
        os.close(self.saved)
        os.close(self.null)


def load(dim, kernel):
    L = C.CDLL(build_ref.kernel_lib(dim, kernel))
    for f in (L.ref_kernel_W, L.ref_kernel_dW):
        f.restype = C.c_double
        f.argtypes = [C.c_int, C.c_double, C.c_double]
    L.ref_set_particle_scale.restype = C.c_int
    L.ref_set_particle_scale.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_double)]
    L.ref_dim.restype = C.c_int
    return L


def evaluate(L, which, dists):
    W = np.zeros((len(H), len(dists[0])))
    dW = np.zeros_like(W)
    with Quiet():
        for a, h in enumerate(H):
            for b, d in enumerate(dists[a]):
                W[a, b] = L.ref_kernel_W(which, float(d), float(h))
                dW[a, b] = L.ref_kernel_dW(which, float(d), float(h))
    return W, dW


def dist_rows():
    base = inputs()
    return np.stack([np.concatenate([base, edge_points(h)]) for h in H])


def main():
    build_ref.build()
    dists = dist_rows()
    out = {"dist": dists, "h": H}
    for dim in (2, 3):
        for k, name in build_ref.KERNEL_NAMES.items():
            L = load(dim, k)
            assert L.ref_dim() == dim
            for which in range(4):
                W, dW = evaluate(L, which, dists)
                out[f"W_{dim}d_{name}_{which}"] = W
                out[f"dW_{dim}d_{name}_{which}"] = dW
    L = load(3, 0)
    si = scale_inputs()
    so = np.zeros(len(si))
    sf = np.zeros(len(si), dtype=np.int32)
    for r, (h, sc, mx, mn) in enumerate(si):
        v = C.c_double(0.0)
        sf[r] = L.ref_set_particle_scale(h, sc, mx, mn, C.byref(v))
        so[r] = v.value
    out.update(scale_in=si, scale_out=so, scale_flag=sf)
    np.savez_compressed(OUT, **out)
    print(OUT)


if __name__ == "__main__":
    main()
