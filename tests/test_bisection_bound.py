"""The error bound behind the FP32 signs of the cut-cell bisection (CPU).

The device walk (csrc/mrsph_levelset.cu, k_vm_walk) refines a level-2 node
four more times with FP32 copies of its corners (gc_child32) and trusts an
FP32 sign when the value is beyond 2^-20 * M, M the largest |corner| of the
node; the reference's FP64 values come from gc_path64.  The bound is
|v32 - exact| <= 13 * 2^-24 * M and |v64 - exact| <= 12 * 2^-53 * M, exact
being the trilinear refinement of the node's FP64 corners in rational
arithmetic.  The product's own functions are compiled for the host and
checked here against Fractions on seeded corner sets."""
import os
import shutil
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sph-mesh-generation_gb300", "csrc", "mrsph_levelset.cu")

HARNESS = r'''
#include "%s"
#include <cstdio>
using namespace mrsph;
int main() {
  int ncase;
  if (scanf("%%d", &ncase) != 1) return 1;
  for (int t = 0; t < ncase; t++) {
    double node[8];
    int path[4];
    for (int q = 0; q < 8; q++) scanf("%%lf", &node[q]);
    for (int l = 0; l < 4; l++) scanf("%%d", &path[l]);
    float c32[8], nx[8];
    for (int q = 0; q < 8; q++) c32[q] = (float)node[q];
    for (int l = 0; l < 4; l++) {
      gc_child32<3>(c32, path[l], nx);
      for (int q = 0; q < 8; q++) c32[q] = nx[q];
    }
    double s64[8];
    gc_path64<3>(node, path, 4, s64);
    for (int q = 0; q < 8; q++) printf("%%.9g %%.17g\n", (double)c32[q], s64[q]);
  }
  return 0;
}
'''


def exact_child(cor, c):
    """Corners ([x][y][z], 8 values) of child c of a node, exact."""
    i, j, k = (c >> 2) & 1, (c >> 1) & 1, c & 1

    def val(X, Y, Z):  # lattice point (X, Y, Z) in {0, 1, 2}^3 of the node
        wx = [(1 - Fraction(X, 2)), Fraction(X, 2)]
        wy = [(1 - Fraction(Y, 2)), Fraction(Y, 2)]
        wz = [(1 - Fraction(Z, 2)), Fraction(Z, 2)]
        return sum(wx[a] * wy[b] * wz[d] * cor[(a * 2 + b) * 2 + d] for a in (0, 1) for b in (0, 1) for d in (0, 1))

    return [val(i + r, j + s, k + t) for r in (0, 1) for s in (0, 1) for t in (0, 1)]


@pytest.mark.skipif(shutil.which("nvcc") is None, reason="nvcc not available")
def test_fp32_sign_bound(tmp_path):
    src = tmp_path / "h.cu"
    src.write_text(HARNESS % SRC)
    exe = tmp_path / "h"
    r = subprocess.run(["nvcc", "-std=c++17", "-O2", "-fmad=false", "-Xcompiler", "-ffp-contract=off",
                        "-gencode", "arch=compute_103a,code=sm_103a", "-I", os.path.dirname(SRC), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    rng = np.random.default_rng(12)
    cases = []
    for t in range(300):
        scale = 10.0 ** rng.integers(-6, 3)
        if t % 3 == 0:  # near-planar, as at a surface
            n = rng.normal(size=3)
            g = np.array([(x, y, z) for x in (0, 1) for y in (0, 1) for z in (0, 1)], dtype=float) - 0.5
            node = (g @ n + rng.normal(scale=1e-3, size=8)) * scale
        else:
            node = rng.uniform(-1, 1, 8) * scale
        cases.append((node, rng.integers(0, 8, 4)))
    inp = f"{len(cases)}\n" + "\n".join(" ".join(repr(float(v)) for v in nd) + " " + " ".join(str(int(c)) for c in p)
                                          for nd, p in cases)
    out = subprocess.run([str(exe)], input=inp, capture_output=True, text=True, check=True).stdout.split()
    vals = np.array(out, dtype=float).reshape(len(cases), 8, 2)
    for (node, path), got in zip(cases, vals):
        ex = [Fraction(float(v)) for v in node]
        for c in path:
            ex = exact_child(ex, int(c))
        M = max(abs(float(v)) for v in node)
        for q in range(8):
            e = ex[q]
            assert abs(Fraction(got[q, 0]) - e) <= Fraction(13, 2 ** 24) * Fraction(M)
            assert abs(Fraction(got[q, 1]) - e) <= Fraction(12, 2 ** 53) * Fraction(M)
            if abs(got[q, 0]) > M * 2.0 ** -20:
                assert np.sign(got[q, 0]) == np.sign(got[q, 1])
        # the leaf rule's corner sum, in FP32 in the kernel's order, within 2^-16 M
        cv = np.float32(0.0)
        for q in range(8):
            cv = np.float32(cv + np.float32(got[q, 0]))
        assert abs(Fraction(float(cv)) - sum(ex)) <= Fraction(160, 2 ** 24) * Fraction(M)
        if abs(float(cv)) > M * 2.0 ** -16:
            assert np.sign(float(cv)) == np.sign(sum(Fraction(float(v)) for v in got[:, 1]))
