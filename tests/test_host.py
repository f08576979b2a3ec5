"""The C++ host layer (host/*.cpp: SPH_mesh_generation, Solver and the
mrsph_relax driver over the C ABI) on the CPU: it builds, its workloads
count the same particles as the Python workloads, and without a GPU it
fails with the engine's message and status 2.  The GPU runs are in
test_gpu_host.py."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sph-mesh-generation_gb300"))
from mrsph import build, cases  # noqa: E402


@pytest.fixture(scope="module")
def binary():
    return build.build_host()


def run(binary, *args):
    return subprocess.run([binary, *args], capture_output=True, text=True, timeout=300)


def test_help(binary):
    r = run(binary, "--help")
    assert r.returncode == 0 and "--case" in r.stdout
    for flag in ("--load-lset-restart", "--retarget", "--mesh", "--lset-restart", "--cvp"):
        assert flag in r.stdout, flag
    assert run(binary, "--bogus").returncode == 1


def test_counts_match_python_workloads(binary):
    d = json.loads(run(binary, "--case", "disc_hole_2d", "--count-only").stdout)
    assert d["n_particles"] == cases.disc_hole_2d(spacing=0.02, grid=64).n_particles
    t = json.loads(run(binary, "--case", "torus_3d", "--count-only").stdout)
    assert t["n_particles"] == cases.torus_3d().n_particles
    for dim, kw in ((2, dict(spacing=0.02, grid=64)), (3, dict(spacing=0.04, grid=32))):
        b = json.loads(run(binary, "--case", f"box_{dim}d", "--count-only").stdout)
        assert b["n_particles"] == cases.box_with_corners(dim=dim, kernel="hyperbolic", h_over_dx=1.0,
                                                          **kw).n_particles


def test_engine_error_without_gpu(binary):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    r = run(binary, "--case", "disc_hole_2d", "--steps", "1")
    assert r.returncode == 2 and "mrsph_create" in r.stderr


def test_cpp_particle_vtu_matches_python_writer(binary, tmp_path):
    """The C++ Particle_binary_writer writes the same bytes as the Python
    writer (mrsph/io.py) for the same particle arrays."""
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_particle_vtu
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_longlong] + [ctypes.c_void_p] * 5
    rng = np.random.default_rng(4)
    n = 1000
    xyz = rng.random((n, 3))
    typ = rng.integers(0, 2, n).astype(np.int32)
    h = rng.random(n)
    nn = rng.integers(1, 90, n).astype(np.int32)
    nrm = rng.normal(size=(n, 3))
    p = tmp_path / "c.vtu"
    size = f(str(p).encode(), n, xyz.ctypes.data, typ.ctypes.data, h.ctypes.data, nn.ctypes.data, nrm.ctypes.data)
    pd = [("id", np.arange(n, dtype="<i4")), ("local_id", np.arange(n, dtype="<i4")), ("type", typ),
          ("h", h.astype("<f4")), ("NN", nn), ("color", np.zeros(n, dtype="<i4")), ("norm", nrm.astype("<f4"))]
    ref = io.vtu_bytes(xyz, np.arange(n, dtype="<i4"), 1, pd)
    got = p.read_bytes()
    assert size == len(ref) and got == ref
    back = io.read_vtu(str(p))
    assert np.array_equal(back["NN"], nn) and np.array_equal(back["Position"], xyz.astype(np.float32))


@pytest.mark.parametrize("dim", [2, 3])
def test_cpp_lset_vti_matches_python_writer(binary, tmp_path, dim):
    """The C++ Level_set_binary_writer's image bytes equal the Python
    writer's (vti_bytes) for the same arrays, origin and spacing included."""
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_lset_vti
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p] * 10
    rng = np.random.default_rng(dim)
    nc = np.array([12, 8, 6 if dim == 3 else 0], dtype=np.int32)
    origin = np.array([-1.6, 0.0001, -0.45 if dim == 3 else 0.0])
    spacing = np.array([0.0125, 1.0 / 3.0, 0.05 if dim == 3 else 1.0])
    npt = int(np.prod(nc + 1))
    ncl = int(np.prod(np.maximum(nc, 1)))
    phi, curv, scale = (rng.normal(size=npt).astype("<f4") for _ in range(3))
    tag = rng.integers(0, 2, ncl).astype("<i4")
    vol, area = (rng.random(ncl).astype("<f4") for _ in range(2))
    chr_ = rng.integers(0, 3, ncl).astype("<i4")
    p = tmp_path / "c.vti"
    size = f(str(p).encode(), nc.ctypes.data, origin.ctypes.data, spacing.ctypes.data, phi.ctypes.data,
             curv.ctypes.data, scale.ctypes.data, tag.ctypes.data, vol.ctypes.data, area.ctypes.data,
             chr_.ctypes.data)
    ref = io.vti_bytes([int(x) for x in nc], list(origin), list(spacing),
                       [("phi", phi), ("curv", curv), ("scale", scale)],
                       [("interface", tag), ("char", chr_), ("vol", vol), ("area", area)])
    assert size == len(ref) and p.read_bytes() == ref


def test_repr_double_matches_python(binary):
    import ctypes
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    assert lib is not None
    import numpy as np
    from mrsph import io
    # through the image header: Origin / Spacing are written with repr
    vals = [0.0, 1.0, -1.6, 0.0001, 1e-05, 123456789.0, 1e16, 2.5e-7, 0.1 + 0.2, 3.2 / 256]
    f = lib.mrsph_host_lset_vti
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p] + [ctypes.c_void_p] * 10
    import tempfile
    nc = np.array([1, 1, 1], dtype=np.int32)
    z8, z1 = np.zeros(8, dtype="<f4"), np.zeros(1, dtype="<f4")
    t1 = np.zeros(1, dtype="<i4")
    with tempfile.TemporaryDirectory() as d:
        for v in vals:
            o = np.array([v, -v, v / 3])
            s = np.array([v + 1.0, 2.0, 0.5])
            path = os.path.join(d, "r.vti")
            f(path.encode(), nc.ctypes.data, o.ctypes.data, s.ctypes.data, z8.ctypes.data, z8.ctypes.data,
              z8.ctypes.data, t1.ctypes.data, z1.ctypes.data, z1.ctypes.data, None)
            head = open(path, "rb").read().split(b"<PointData")[0].decode()
            ref = io.vti_bytes([1, 1, 1], list(o), list(s), [("phi", z8)], []).split(b"<PointData")[0].decode()
            assert head == ref, (v, head, ref)


def test_cpp_mesh_vtu_matches_python_writer(binary, tmp_path):
    """The C++ triangle-mesh VTU (Mesh_binary_writer) equals the Python
    writer's bytes for the same particles and triangles."""
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_mesh_vtu
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_longlong] + [ctypes.c_void_p] * 5 + [ctypes.c_longlong, ctypes.c_void_p]
    rng = np.random.default_rng(9)
    n, m = 400, 700
    xyz = np.concatenate([rng.random((n, 2)), np.zeros((n, 1))], axis=1)
    typ = rng.integers(0, 2, n).astype(np.int32)
    h = rng.random(n)
    nn = rng.integers(1, 30, n).astype(np.int32)
    nrm = np.concatenate([rng.normal(size=(n, 2)), np.zeros((n, 1))], axis=1)
    tris = np.stack([rng.choice(n, 3, replace=False) for _ in range(m)]).astype(np.int32)
    p = tmp_path / "m.vtu"
    size = f(str(p).encode(), n, xyz.ctypes.data, typ.ctypes.data, h.ctypes.data, nn.ctypes.data, nrm.ctypes.data,
             m, tris.ctypes.data)
    pd = [("id", np.arange(n, dtype="<i4")), ("local_id", np.arange(n, dtype="<i4")), ("type", typ),
          ("h", h.astype("<f4")), ("NN", nn), ("color", np.zeros(n, dtype="<i4")), ("norm", nrm.astype("<f4"))]
    vol, aspect = io.triangle_quality(xyz, tris)
    ref = io.vtu_bytes(xyz, tris, 5, pd, [("vol", vol.astype("<f4")), ("aspect", aspect.astype("<f4"))])
    assert size == len(ref) and p.read_bytes() == ref


def test_cpp_tet_vtu_matches_python_writer(binary, tmp_path):
    """The C++ tet-mesh VTU (the 3D branch of Mesh_binary_writer) equals the
    Python writer's bytes for the same particles and tets (cell fields from
    each side's own tet quality evaluation)."""
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_tet_vtu
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_longlong] + [ctypes.c_void_p] * 5 + [ctypes.c_longlong, ctypes.c_void_p]
    rng = np.random.default_rng(10)
    n, m = 300, 600
    xyz = rng.random((n, 3))
    typ = rng.integers(0, 3, n).astype(np.int32)
    h = rng.random(n)
    nn = rng.integers(1, 60, n).astype(np.int32)
    nrm = rng.normal(size=(n, 3))
    tets = np.stack([rng.choice(n, 4, replace=False) for _ in range(m)]).astype(np.int32)
    p = tmp_path / "t.vtu"
    size = f(str(p).encode(), n, xyz.ctypes.data, typ.ctypes.data, h.ctypes.data, nn.ctypes.data, nrm.ctypes.data,
             m, tets.ctypes.data)
    pd = [("id", np.arange(n, dtype="<i4")), ("local_id", np.arange(n, dtype="<i4")), ("type", typ),
          ("h", h.astype("<f4")), ("NN", nn), ("color", np.zeros(n, dtype="<i4")), ("norm", nrm.astype("<f4"))]
    vol, aspect, ratio, mind = io.tet_quality(xyz, tets)
    cd = [("vol", vol.astype("<f4")), ("aspect", aspect.astype("<f4")), ("radius_ratio", ratio.astype("<f4")),
          ("mindihedangle", mind.astype("<f4"))]
    ref = io.vtu_bytes(xyz, tets, 10, pd, cd)
    got = p.read_bytes()
    assert size == len(ref)
    if got != ref:  # report which cell field differs
        r, q = io.read_vtu(str(p)), io.read_vtu_bytes(ref) if hasattr(io, "read_vtu_bytes") else None
        bad = [k for k, v in cd if not np.array_equal(r[k], v)]
        raise AssertionError(f"tet VTU bytes differ; fields {bad}")


@pytest.mark.parametrize("mesh", [0, 1, 2])
def test_cpp_pvtu_matches_python(binary, mesh):
    import ctypes
    import numpy as np
    from mrsph import io
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_pvtu
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_int, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_longlong]
    buf = ctypes.create_string_buffer(8192)
    n = f(mesh, b"piece_0.vtu", buf, 8192)
    pd = [("id", np.zeros(1, "<i4")), ("local_id", np.zeros(1, "<i4")), ("type", np.zeros(1, "<i4")),
          ("h", np.zeros(1, "<f4")), ("NN", np.zeros(1, "<i4")), ("color", np.zeros(1, "<i4")),
          ("norm", np.zeros((1, 3), "<f4"))]
    cd = [("vol", np.zeros(1, "<f4")), ("aspect", np.zeros(1, "<f4"))] if mesh else []
    if mesh == 2:
        cd += [("radius_ratio", np.zeros(1, "<f4")), ("mindihedangle", np.zeros(1, "<f4"))]
    ref = io._pvtu_text(["piece_0.vtu"], io._fields_meta(pd), io._fields_meta(cd))
    assert n == len(ref) and buf.value.decode() == ref


@pytest.mark.parametrize("name", ["disc2d", "box3d"])
def test_cpp_case_from_lset_restart_matches_python(binary, tmp_path, name):
    """The C++ restart run (Load_lset_restart + case_from_lset_restart, the
    reference's Load_rst_case) builds the case the Python loader builds from
    the same rstfile/levelset.rst: phi incl. margins bit-equal, the same
    spacing bounds, domain, characteristic points and segments, and the
    reference's restart count (Get_num_particles over the file's totals);
    the driver seeds that count.  A truncated file is an error (status 2)."""
    import ctypes
    import oracle
    from mrsph import io
    from test_io import _restart_sim
    case = {"disc2d": lambda: cases.disc_hole_2d(spacing=0.02, grid=64),
            "box3d": lambda: cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic",
                                                    h_over_dx=1.0)}[name]()
    orc = oracle.Oracle(case)
    path = io.save_lset_restart(_restart_sim(case, orc), str(tmp_path / "levelset.rst"))
    kern = {v: k for k, v in cases.KERNELS.items()}[case.params["kernel"]]
    hdx = case.params["cell_ratio"] / 2
    py = cases.from_lset_restart(path, kernel=kern, h_over_dx=hdx)
    lib = ctypes.CDLL(os.path.join(ROOT, "sph-mesh-generation_gb300", "libmrsph_host.so"))
    f = lib.mrsph_host_lset_case
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_longlong,
                  ctypes.c_int]
    import numpy as np
    phi = np.empty(py.levels[0].phi.size)
    prm = np.empty(10)
    cnt = np.empty(4, dtype=np.int64)
    err = ctypes.create_string_buffer(256)
    assert f(path.encode(), py.params["kernel"], hdx, 0, 0, phi.ctypes.data, len(phi), prm.ctypes.data,
             cnt.ctypes.data, err, 256, 0) == 0, err.value
    assert cnt[1] == py.levels[0].phi.size
    assert np.array_equal(phi, py.levels[0].phi.ravel())
    p = py.params
    assert list(prm[:4]) == [p["min_dl"], p["max_dl"], p["middle_dl"], p["cell_ratio"]]
    assert list(prm[4:7]) == list(p["box_l"]) and list(prm[7:10]) == list(p["box_r"])
    assert cnt[0] == py.n_particles == orc.volume_mass(0)["num_particle"]
    assert cnt[2] == len(py.extra.get("singularities", [])) and cnt[3] == len(py.extra.get("segments", []))
    d = json.loads(run(binary, "--load-lset-restart", path, "--kernel", kern, "--h-over-dx", str(hdx),
                       "--count-only").stdout)
    assert d["n_particles"] == py.n_particles and d["workload"] == "lset_restart"
    short = tmp_path / "short.rst"
    short.write_bytes(open(path, "rb").read()[:-8])
    assert f(str(short).encode(), 2, 1.3, 0, 0, phi.ctypes.data, len(phi), prm.ctypes.data, cnt.ctypes.data,
             err, 256, 0) == -1 and b"too short" in err.value
    # the re-targeting restart run: spacing 2, 5, 16 cells; count = spacing integral
    rt = cases.from_lset_restart(path, kernel=kern, h_over_dx=hdx, retarget=cases.RETARGET_FACTORS)
    assert f(path.encode(), py.params["kernel"], hdx, 0, 0, phi.ctypes.data, len(phi), prm.ctypes.data,
             cnt.ctypes.data, err, 256, 1) == 0, err.value
    dl = min(rt.levels[0].dpkg[d] / 4.0 for d in range(rt.params["dim"]))
    assert list(prm[:3]) == [rt.params["min_dl"], rt.params["max_dl"], rt.params["middle_dl"]]
    assert rt.params["min_dl"] == 2.0 * dl and rt.params["max_dl"] == 16.0 * dl
    assert cnt[0] == rt.n_particles == cases.particle_count(rt.levels, rt.params)
    d2 = json.loads(run(binary, "--load-lset-restart", path, "--retarget", "--kernel", kern, "--h-over-dx",
                        str(hdx), "--count-only").stdout)
    assert d2["n_particles"] == rt.n_particles
    r = run(binary, "--load-lset-restart", str(short), "--count-only")
    assert r.returncode == 2 and "too short" in r.stderr


def test_cpp_lset_restart_rejects_bad_headers(binary, tmp_path):
    """Load_lset_restart refuses a file whose dimension is not 2 or 3 or that
    holds more than one level (status 2 from the driver, with the reason)."""
    import struct
    import oracle
    from mrsph import io
    from test_io import _restart_sim
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    path = io.save_lset_restart(_restart_sim(case, oracle.Oracle(case)), str(tmp_path / "levelset.rst"))
    raw = bytearray(open(path, "rb").read())
    bad_dim = tmp_path / "dim.rst"
    bad_dim.write_bytes(struct.pack("<i", 4) + bytes(raw[4:]))
    r = run(binary, "--load-lset-restart", str(bad_dim), "--count-only")
    assert r.returncode == 2 and "dimension" in r.stderr
    lv = 4 + 18 * 8 + 8 * 4  # dim, domain/box/particle box, resolution, Lmin, Lmax, ini_num_cell
    assert struct.unpack_from("<i", raw, lv)[0] == 1
    two = tmp_path / "two.rst"
    two.write_bytes(bytes(raw[:lv]) + struct.pack("<i", 2) + bytes(raw[lv + 4:]))
    r = run(binary, "--load-lset-restart", str(two), "--count-only")
    assert r.returncode == 2 and "one level" in r.stderr
