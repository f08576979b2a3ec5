"""The no-allocation level-set sampler against the allocating one.

mrsph_sample_levelset_noalloc serves callers that cannot call cudaMalloc
(it synchronises the device, and some hosts forbid it outright); it stages
through a fixed scratch array in the library image instead.  Two calls in a
row must reproduce mrsph_sample_levelset, so the shared scratch carries no
state from one call into the next.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from mrsph import SPHMeshGeneration, cases
from mrsph import _lib as L

pytestmark = pytest.mark.gpu

MAX_POINTS = 65536


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_noalloc_sampling_matches_allocating_entry_point(prec):
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    gpu = SPHMeshGeneration(case, precision=prec)
    lo = np.array(case.params["box_l"])
    hi = np.array(case.params["box_r"])
    for call, npts in enumerate((5000, 1200)):  # two calls in a row, the second smaller
        rng = np.random.default_rng(100 + call)
        pts = lo + rng.random((npts, 3)) * (hi - lo)
        ref = gpu.sample_levelset(pts)
        got = gpu.sample_levelset_noalloc(pts)
        tol = 1e-13 if prec == "fp64" else 1e-6
        assert np.max(np.abs(got[0] - ref[0])) <= tol
        assert np.max(np.abs(got[1] - ref[1])) <= tol
        assert np.max(np.abs(got[2] - ref[2])) <= tol * 1e3
        assert np.array_equal(got[3], ref[3])
    gpu.close()


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """After the first call on the device (its set-up: the scratch address
    looked up), further calls at the largest size take no device memory: free
    memory before and after three calls is the same (cudaMemGetInfo, seen
    through torch on the same primary context)."""
    torch = pytest.importorskip("torch")
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    gpu = SPHMeshGeneration(case, precision="fp32")
    lo = np.array(case.params["box_l"])
    hi = np.array(case.params["box_r"])
    pts = lo + np.random.default_rng(3).random((MAX_POINTS, 3)) * (hi - lo)
    first = gpu.sample_levelset_noalloc(pts)
    torch.cuda.synchronize(0)
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        again = gpu.sample_levelset_noalloc(pts)
    torch.cuda.synchronize(0)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0
    for a, b in zip(first, again):
        assert np.array_equal(a, b)
    gpu.close()


def test_noalloc_rejects_oversized_requests():
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    gpu = SPHMeshGeneration(case, precision="fp64")
    n = MAX_POINTS + 1
    pts = np.full((n, 3), 0.5)
    out = np.zeros(n)
    rc = gpu.lib.mrsph_sample_levelset_noalloc(gpu.h, n, pts.ctypes.data_as(ctypes.c_void_p),
                                               out.ctypes.data_as(ctypes.c_void_p), None, None, None)
    assert rc == -5
    buf = ctypes.create_string_buffer(256)
    gpu.lib.mrsph_last_error(gpu.h, buf, 256)
    assert b"65536" in buf.value
    # the maximum size itself is accepted
    phi, _, _, _ = gpu.sample_levelset_noalloc(np.full((MAX_POINTS, 3), 0.3))
    assert phi.shape == (MAX_POINTS,)
    gpu.close()
