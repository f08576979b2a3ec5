"""Writers and restart files (mrsph/io.py) on the CPU: the byte layout of
.pst restarts and list.csv, VTU pieces read back array by array, PVTU / PVD
collections, and the particle and mesh writers over a stand-in for a solver
handle (the GPU round trip is in test_gpu_io.py)."""
import os
import struct

import numpy as np
import pytest

from mrsph import cases, io


class FakeSim:
    """The slice of SPHMeshGeneration the writers read."""

    def __init__(self, n=50, seed=0):
        rng = np.random.default_rng(seed)
        self.n = n
        self.xyz = rng.random((n, 3))
        self.xyz[:, 2] = 0.0
        self.type = (rng.random(n) < 0.3).astype(np.int32)
        self.h = 0.01 + 0.01 * rng.random(n)
        self.norm = rng.standard_normal((n, 3))
        self.cnt = rng.integers(1, 30, n)
        self.case = type("C", (), {"params": {"cutoff": 2.0, "cell_ratio": 2.0}})()
        self.loaded = None

    def particles(self, fields):
        src = {"xyz": self.xyz, "type": self.type, "h": self.h, "norm": self.norm, "phi": self.h * 3,
               "curv": self.h * 0, "a2": self.norm * 2, "v": self.norm * 3}
        return {f: src[f].copy() for f in fields}

    def neighbors(self):
        off = np.concatenate([[0], np.cumsum(self.cnt)])
        return off, np.zeros(off[-1], dtype=np.int32)

    def stats(self):
        return {"step": 7, "dt": 0.5}

    def set_state(self, st, pre_run=False):
        self.loaded = (np.asarray(st["xyz"]).copy(), pre_run)


def test_pst_layout_and_round_trip(tmp_path):
    xyz = np.random.default_rng(1).random((17, 3))
    p = tmp_path / "a.pst"
    io.write_pst(str(p), xyz)
    raw = p.read_bytes()
    assert len(raw) == 4 + 17 * 24
    assert struct.unpack("<i", raw[:4])[0] == 17
    assert np.array_equal(np.frombuffer(raw[4:], dtype="<f8").reshape(17, 3), xyz)
    assert np.array_equal(io.read_pst(str(p)), xyz)
    p.write_bytes(raw[:-8])
    with pytest.raises(ValueError):
        io.read_pst(str(p))


def test_save_and_load_post_file(tmp_path):
    sim = FakeSim()
    path = io.save_particle_post_file(sim, str(tmp_path), run_time=0, first=True)
    io.save_particle_post_file(sim, str(tmp_path), run_time=100)
    assert os.path.basename(path) == "step_0_rank_0.pst"
    assert (tmp_path / "rstfile_particles" / "list.csv").read_text() == "1\n0 50\n100 50\n"
    assert io.read_particle_list(str(tmp_path)) == (1, [(0, 50), (100, 50)])
    other = FakeSim(seed=3)
    assert io.load_data_for_post(other, path) == 50
    assert np.array_equal(other.loaded[0], sim.xyz) and other.loaded[1] is True


def test_vtu_arrays_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    pts = rng.random((9, 3))
    tris = np.array([[0, 1, 2], [2, 3, 4], [5, 6, 7]], dtype=np.int32)
    pd = [("id", np.arange(9, dtype="<i4")), ("h", rng.random(9).astype("<f4")),
          ("norm", rng.random((9, 3)).astype("<f4"))]
    cd = [("vol", rng.random(3).astype("<f4"))]
    p = tmp_path / "m.vtu"
    p.write_bytes(io.vtu_bytes(pts, tris, 5, pd, cd))
    r = io.read_vtu(str(p))
    assert np.array_equal(r["Position"], pts.astype("<f4"))
    assert np.array_equal(r["connectivity"], tris.reshape(-1))
    assert np.array_equal(r["offsets"], [3, 6, 9])
    assert np.array_equal(r["types"], [5, 5, 5])
    for name, a in pd + cd:
        assert np.array_equal(r[name], a), name
    head = p.read_bytes().split(b"<AppendedData")[0].decode()
    assert 'NumberOfPoints="9" NumberOfCells="3"' in head
    assert head.count("<DataArray") == 8


def test_particle_writer_series(tmp_path):
    sim = FakeSim()
    w = io.ParticleWriter(str(tmp_path / "outdata"), fields=io.PARTICLE_FIELDS_ALL)
    f0 = w.Output_particle(0, sim, run_time=0)
    w.Output_particle(1, sim, run_time=10)
    r = io.read_vtu(f0)
    assert np.array_equal(r["id"], np.arange(50))
    assert np.array_equal(r["type"], sim.type)
    assert np.array_equal(r["NN"], sim.cnt)
    assert np.allclose(r["h"], sim.h.astype(np.float32))
    assert np.allclose(r["scale"], (sim.h * 2.0 / 2.0).astype(np.float32))
    assert np.allclose(r["accel"], (sim.norm * 2).astype(np.float32))
    assert r["norm"].shape == (50, 3) and np.array_equal(r["types"], np.ones(50))
    pvd = (tmp_path / "outdata" / "particle.pvd").read_text()
    assert pvd.count("<DataSet") == 2 and 'file="./particle_step_1.pvtu"' in pvd
    pvtu = (tmp_path / "outdata" / "particle_step_0.pvtu").read_text()
    assert '<Piece Source="particle_rank_0_step_0.vtu"/>' in pvtu
    assert pvtu.count("<PDataArray") == len(io.PARTICLE_FIELDS_ALL) + 1
    with pytest.raises(ValueError):
        io.ParticleWriter(str(tmp_path), fields=("nope",))


def test_mesh_writer_and_quality(tmp_path):
    sim = FakeSim(n=4)
    sim.xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0]], dtype=np.float64)
    tris = np.array([[0, 1, 2], [1, 3, 2]])
    area, aspect = io.triangle_quality(sim.xyz, tris)
    assert np.allclose(area, [0.5, 0.5]) and np.allclose(aspect, [np.sqrt(2), np.sqrt(2)])
    f = io.MeshWriter(str(tmp_path)).Output_mesh(0, sim, tris=tris, run_time=3)
    r = io.read_vtu(f)
    assert np.array_equal(r["connectivity"], tris.reshape(-1)) and np.array_equal(r["types"], [5, 5])
    assert np.allclose(r["vol"], 0.5) and np.allclose(r["aspect"], np.sqrt(2))
    assert 'timestep="3"' in (tmp_path / "mesh_tris.pvd").read_text()


def test_tet_mesh_writer_and_quality(tmp_path):
    """The 3D branch of Mesh_binary_writer (mesh_binary_writer.cpp:392-640):
    tet cells (VTK type 10) with 'vol', 'aspect', 'radius_ratio' and
    'mindihedangle'; a regular tetrahedron has radius ratio 1, aspect
    ratio sqrt(3/2) and dihedral angles arccos(1/3)."""
    sim = FakeSim(n=5)
    sim.case.params["dim"] = 3
    s = 1.0 / np.sqrt(2.0)
    sim.xyz = np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1], [0, 0, -3]], dtype=np.float64) * s
    tets = np.array([[0, 1, 2, 3], [1, 2, 3, 4]])
    vol, aspect, ratio, mind = io.tet_quality(sim.xyz, tets)
    edge = 2.0
    assert np.isclose(vol[0], edge ** 3 / (6 * np.sqrt(2))) and np.isclose(ratio[0], 1.0)
    assert np.isclose(aspect[0], np.sqrt(1.5)) and np.isclose(mind[0], np.arccos(1 / 3) / 3.1415926 * 180.0)
    assert ratio[1] < 1.0 and aspect[1] > aspect[0]
    f = io.MeshWriter(str(tmp_path)).Output_mesh(0, sim, tets=tets, run_time=4)
    assert os.path.basename(f) == "mesh_tets_rank_0_step_0.vtu"
    r = io.read_vtu(f)
    assert np.array_equal(r["connectivity"], tets.reshape(-1)) and np.array_equal(r["types"], [10, 10])
    assert np.array_equal(r["offsets"], [4, 8])
    for k, v in (("vol", vol), ("aspect", aspect), ("radius_ratio", ratio), ("mindihedangle", mind)):
        assert np.array_equal(r[k], v.astype(np.float32)), k
    assert 'timestep="4"' in (tmp_path / "mesh_tets.pvd").read_text()
    assert (tmp_path / "mesh_tets_step_0.pvtu").exists()


def test_corner_average_and_levelset_writer(tmp_path):
    from mrsph import cases
    case = cases.disc_hole_2d(spacing=0.02, grid=64)
    lv = case.levels[0]
    m = 4 * lv.margin
    # a linear phi averages to its value at the corners
    ny, nx = lv.phi.shape[1:]
    xc = np.arange(nx)[None, :] + 0.0 * np.arange(ny)[:, None]
    lin = (2.0 * xc + 3.0 * np.arange(ny)[:, None])[None]
    cor = io.corner_average(lin, m, 2)
    assert cor.shape == (1, ny - 2 * m + 1, nx - 2 * m + 1)
    assert np.allclose(cor[0, 0, 0], 2.0 * (m - 0.5) + 3.0 * (m - 0.5))

    class LsSim(FakeSim):
        def __init__(self):
            super().__init__()
            self.case = case

        def levelset_fields(self, level):
            shp = case.levels[level].phi.shape
            tag = (np.abs(case.levels[level].phi) < 0.02).astype(np.uint8)
            return {"curv": np.ones(shp), "tag": tag, "max_phi": float(case.levels[level].phi.max()),
                    "nx": np.zeros(shp), "ny": np.zeros(shp), "nz": np.zeros(shp)}

        def volume_mass(self, level, cells=False):
            phi = case.levels[level].phi
            return {"vol": np.where(phi > 0, 1e-4, 0.0), "area": np.where(np.abs(phi) < 0.02, 0.01, 0.0)}

    sim = LsSim()
    f = io.LevelSetWriter(str(tmp_path)).Output_lset(0, sim, run_time=0)
    r = io.read_vtu(f)
    nc = 4 * lv.num_pkg[0]
    assert r["phi"].size == (nc + 1) * (4 * lv.num_pkg[1] + 1)
    assert np.allclose(r["phi"].reshape(cor.shape[1:]), io.corner_average(lv.phi, m, 2)[0].astype(np.float32))
    assert np.allclose(r["curv"], 1.0)
    assert r["interface"].size == nc * 4 * lv.num_pkg[1]
    assert r["interface"].sum() == sim.levelset_fields(0)["tag"][0, m:-m, m:-m].sum()
    assert np.array_equal(r["vol"], np.where(lv.phi[0, m:-m, m:-m] > 0, 1e-4, 0.0).ravel().astype(np.float32))
    assert np.array_equal(r["area"], np.where(np.abs(lv.phi[0, m:-m, m:-m]) < 0.02, 0.01, 0.0).ravel().astype(np.float32))
    sc = r["scale"]
    assert sc.min() >= case.params["min_dl"] - 1e-7 and sc.max() <= case.params["max_dl"] + 1e-7
    head = open(f, "rb").read().split(b"<AppendedData")[0].decode()
    assert f'WholeExtent="0 {nc} 0 {4 * lv.num_pkg[1]} 0 0"' in head
    assert (tmp_path / "mesh_lset_step_0.pvti").exists() and (tmp_path / "mesh_lset.pvd").exists()


@pytest.mark.parametrize("dim", [2, 3])
def test_lset_restart_round_trip(tmp_path, dim):
    """save_lset_restart / load_lset_restart: the reference's levelset.rst
    layout (one level) round-trips the level's fields over the interior
    cells, the cut-cell totals and the package bookkeeping; the level-set
    fields come from the FP64 oracle (standing in for the engine)."""
    import oracle
    if dim == 2:
        case = cases.disc_hole_2d(spacing=0.02, grid=64)
    else:
        case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2)
    orc = oracle.Oracle(case)

    class RstSim(FakeSim):
        def __init__(self):
            super().__init__()
            self.case = case

        def levelset_fields(self, level):
            f = orc.fields[level]
            shp = case.levels[level].phi.shape
            return {"nx": f["nx"].reshape(shp), "ny": f["ny"].reshape(shp), "nz": f["nz"].reshape(shp),
                    "curv": f["curv"].reshape(shp), "tag": f["tag"].reshape(shp).astype(np.uint8),
                    "max_phi": orc.ctx.max_phi}

        def volume_mass(self, level, cells=False):
            return orc.volume_mass(level)

    sim = RstSim()
    path = io.save_lset_restart(sim, str(tmp_path / "rstfile" / "levelset.rst"))
    r = io.load_lset_restart(path)
    lv = case.levels[-1]
    m = 4 * lv.margin
    inner = (slice(None),) if dim == 2 else (slice(m, -m),)
    inner = inner + (slice(m, -m), slice(m, -m))
    f = sim.levelset_fields(len(case.levels) - 1)
    assert r["dim"] == dim and r["num_level"] == 1
    assert np.array_equal(r["phi"], lv.phi[inner])
    for k, g in (("n_x", "nx"), ("n_y", "ny"), ("n_z", "nz"), ("curv", "curv")):
        assert np.array_equal(r[k], f[g][inner]), k
    assert np.array_equal(r["tag_interface"], f["tag"][inner].astype(np.int32))
    assert np.all(r["idx_characteristic"] == -1) and np.all(r["tag_characteristic"] == 0)
    assert r["singularities"].shape == (0, 3) and r["segments"].shape == (0, 6)
    vm = orc.volume_mass(-1)
    assert r["total_mass"] == vm["total_mass"] and r["glbl_num_interface_cell"] == vm["num_interface_cell"]
    assert r["maximum_phi"] == orc.ctx.max_phi
    npkg = [lv.num_pkg[d] if d < dim else 1 for d in range(3)]
    assert tuple(r["num_pkg"]) == tuple(npkg)
    assert r["glbl_total_num_pkg"] == int(np.prod([n + (2 if d < dim else 0) for d, n in enumerate(npkg)]))
    counted = (lv.phi[inner] > 0) | (np.abs(lv.phi[inner]) < r["dl"])
    assert np.all((r["scale_cells"] > 0) == counted)


def _oracle_chr(orc, level):
    f = orc.fields[level]
    shp = orc.case.levels[level].phi.shape
    enc = np.where(f["chr"] == 2, f["chr_idx"] + 1, np.where(f["chr"] == 1, -(f["chr_idx"] + 1), 0))
    return enc.reshape(shp).astype(np.int32)


@pytest.mark.parametrize("dim", [2, 3])
def test_lset_restart_characteristics(tmp_path, dim):
    """A geometry with corners (and edges in 3D): the restart carries the
    singularity points, the segments and each cell's tag_characteristic /
    idx_characteristic (level_set.cpp:1053-1070)."""
    import oracle
    case = cases.box_with_corners(dim=dim, spacing=0.04 if dim == 3 else 0.02, grid=32 if dim == 3 else 64,
                                  kernel="hyperbolic", h_over_dx=1.0)
    orc = oracle.Oracle(case)

    r = io.load_lset_restart(io.save_lset_restart(_restart_sim(case, orc), str(tmp_path / "levelset.rst")))
    assert np.array_equal(r["singularities"], case.extra["singularities"])
    segs = case.extra.get("segments", np.zeros((0, 6)))
    assert np.array_equal(r["segments"], np.asarray(segs).reshape(-1, 6))
    lv = case.levels[-1]
    m = 4 * lv.margin
    inner = ((slice(None),) if dim == 2 else (slice(m, -m),)) + (slice(m, -m), slice(m, -m))
    f = orc.fields[-1]
    shp = lv.phi.shape
    assert np.array_equal(r["tag_characteristic"], f["chr"].reshape(shp)[inner])
    assert np.array_equal(r["idx_characteristic"], f["chr_idx"].reshape(shp)[inner])
    assert np.count_nonzero(r["tag_characteristic"] == 1) == len(case.extra["singularities"])
    vm = orc.volume_mass(len(case.levels) - 1)
    assert r["total_mass_segment"] == vm["total_mass_segment"] and r["total_length"] == vm["total_length"]
    if dim == 3:
        assert np.count_nonzero(r["tag_characteristic"] == 2) > 0
        assert r["total_mass_segment"] > 0


def _restart_sim(case, orc):
    class RstSim(FakeSim):
        def __init__(self):
            super().__init__()
            self.case = case

        def levelset_fields(self, level):
            g = orc.fields[level]
            shp = case.levels[level].phi.shape
            return {"nx": g["nx"].reshape(shp), "ny": g["ny"].reshape(shp), "nz": g["nz"].reshape(shp),
                    "curv": g["curv"].reshape(shp), "tag": g["tag"].reshape(shp).astype(np.uint8),
                    "max_phi": orc.ctx.max_phi}

        def characteristic_tags(self, level):
            return _oracle_chr(orc, level)

        def volume_mass(self, level, cells=False):
            return orc.volume_mass(level)
    return RstSim()


@pytest.mark.parametrize("name", ["disc2d", "torus3d", "box2d", "box3d"])
def test_cpp_lset_restart_bytes_match_python(tmp_path, name):
    """The C++ host layer's level-set restart serialiser writes the bytes the
    Python writer wrote, for the values and fields read back from it (with
    and without characteristic points and segments)."""
    import ctypes
    from mrsph import build
    import oracle
    build.build_host()
    lib = ctypes.CDLL(os.path.join(os.path.dirname(io.__file__), "..", "libmrsph_host.so"))
    f = lib.mrsph_host_lset_restart
    f.restype = ctypes.c_longlong
    f.argtypes = [ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong] + [ctypes.c_void_p] * 7 + \
        [ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    case = {"disc2d": lambda: cases.disc_hole_2d(spacing=0.02, grid=64),
            "torus3d": lambda: cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2),
            "box2d": lambda: cases.box_with_corners(dim=2, spacing=0.02, grid=64, kernel="hyperbolic",
                                                    h_over_dx=1.0),
            "box3d": lambda: cases.box_with_corners(dim=3, spacing=0.04, grid=32, kernel="hyperbolic",
                                                    h_over_dx=1.0)}[name]()
    orc = oracle.Oracle(case)

    py = io.save_lset_restart(_restart_sim(case, orc), str(tmp_path / "py.rst"))
    r = io.load_lset_restart(py)
    box_r = [r["box_l"][d] + r["domain"][d] for d in range(3)]
    hd = np.array(list(r["box_l"]) + box_r + list(r["dpkg"]) + list(r["dcell"]) +
                  [r[k] for k in ("fac_maximum_dl", "fac_middel_dl", "fac_minimum_dl", "maximum_curv_artificial",
                                  "total_mass", "total_mass_surface", "total_volume", "total_area", "maximum_phi",
                                  "maximum_dl", "middel_dl", "minimum_dl", "maximum_curv", "minimum_curv",
                                  "total_mass_segment", "total_length")])
    hi = np.array([r["dim"], *r["num_pkg"], *r["num_pkg_margin"], r["glbl_num_interface_cell"]], dtype=np.int32)
    arrs = [np.ascontiguousarray(r[k].ravel()) for k in ("phi", "n_x", "n_y", "n_z", "curv")]
    tag = np.ascontiguousarray(r["tag_interface"].ravel())
    scale = np.ascontiguousarray(r["scale_cells"].ravel())
    out = tmp_path / "cpp.rst"
    sing = np.ascontiguousarray(r["singularities"])
    seg = np.ascontiguousarray(r["segments"])
    ctag = np.ascontiguousarray(r["tag_characteristic"].ravel())
    cidx = np.ascontiguousarray(r["idx_characteristic"].ravel())
    size = f(str(out).encode(), hd.ctypes.data, hi.ctypes.data, len(tag), *[a.ctypes.data for a in arrs],
             tag.ctypes.data, scale.ctypes.data, len(sing), sing.ctypes.data if len(sing) else None,
             len(seg), seg.ctypes.data if len(seg) else None, ctag.ctypes.data, cidx.ctypes.data)
    ref = open(py, "rb").read()
    assert size == len(ref) and out.read_bytes() == ref


@pytest.mark.parametrize("name", ["disc2d", "box2d", "torus3d"])
def test_case_from_lset_restart(tmp_path, name):
    """A case read back from a level-set restart (Load_lset_restart_file,
    level_set.cpp:1098-1175): the interior cells' phi, the domain, the
    spacing bounds and the characteristic points and segments are the
    written ones; a margin cell holds the nearest interior cell's phi minus
    its distance to it; and the oracle relaxes the same particles from it as
    from the case that wrote the file (the margins are never sampled)."""
    import oracle
    case = {"disc2d": lambda: cases.disc_hole_2d(spacing=0.02, grid=64),
            "box2d": lambda: cases.box_with_corners(dim=2, spacing=0.02, grid=64),
            "torus3d": lambda: cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=1)}[name]()
    orc = oracle.Oracle(case)
    path = io.save_lset_restart(_restart_sim(case, orc), str(tmp_path / "levelset.rst"))
    kern = {v: k for k, v in cases.KERNELS.items()}[case.params["kernel"]]
    c2 = cases.from_lset_restart(path, kernel=kern, h_over_dx=case.params["cell_ratio"] / 2,
                                 precision="fp64", scale_law=case.params.get("scale_law", 0))
    dim = case.params["dim"]
    lv, lv2 = case.levels[0], c2.levels[0]
    m = 4 * lv.margin
    inner = (slice(m, -m) if dim == 3 else slice(None), slice(m, -m), slice(m, -m))
    assert lv2.phi.shape == lv.phi.shape and lv2.margin == lv.margin
    assert np.array_equal(lv2.phi[inner], lv.phi[inner])
    assert lv2.num_pkg[:dim] == lv.num_pkg[:dim] and lv2.dpkg[:dim] == lv.dpkg[:dim]
    for k in ("min_dl", "max_dl", "cell_ratio", "box_l", "box_r", "kernel", "dim"):
        assert np.array_equal(np.asarray(c2.params[k])[:dim] if k.startswith("box") else c2.params[k],
                              np.asarray(case.params[k])[:dim] if k.startswith("box") else case.params[k]), k
    for k in ("singularities", "segments"):
        assert (k in c2.extra) == (k in case.extra)
        if k in case.extra:
            assert np.array_equal(np.asarray(c2.extra[k]), np.asarray(case.extra[k]))
    # corner of the margin: (m, m[, m]) cells outward along each axis
    dc = [lv.dpkg[d] / 4.0 for d in range(dim)]
    corner = (0 if dim == 2 else 0, 0, 0)
    near = (0 if dim == 2 else m, m, m)
    want = lv.phi[near] - np.sqrt(sum((m * dc[d]) ** 2 for d in range(dim)))
    assert lv2.phi[corner] == want
    assert c2.n_particles == orc.volume_mass(0)["num_particle"]
    o2 = oracle.Oracle(c2)
    n = case.n_particles
    for o in (orc, o2):
        o.alloc(n)
        o.seed(n)
        o.pre_run()
        o.steps(3)
    s1, s2 = orc.get_state(), o2.get_state()
    for k in s1:
        assert np.array_equal(s1[k], s2[k]), k


def test_case_from_lset_restart_retarget_curvature_law(tmp_path):
    """The re-targeting restart run under the curvature law: minimum, middle
    and maximum spacing are 2, 5 and 16 level-set cells, and the count is the
    spacing integral of that law (between the counts at the two bounds)."""
    import oracle
    case = cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=1)
    orc = oracle.Oracle(case)
    path = io.save_lset_restart(_restart_sim(case, orc), str(tmp_path / "levelset.rst"))
    kern = {v: k for k, v in cases.KERNELS.items()}[case.params["kernel"]]
    hdx = case.params["cell_ratio"] / 2
    rt = cases.from_lset_restart(path, kernel=kern, h_over_dx=hdx, scale_law=1, retarget=cases.RETARGET_FACTORS)
    dl = min(case.levels[0].dpkg[d] / 4.0 for d in range(3))
    p = rt.params
    assert (p["min_dl"], p["middle_dl"], p["max_dl"]) == (2.0 * dl, 5.0 * dl, 16.0 * dl) and p["scale_law"] == 1
    assert rt.n_particles == cases.particle_count(rt.levels, p) > 0
    lo = cases.particle_count(rt.levels, dict(p, scale_law=0, max_dl=p["min_dl"]))
    hi = cases.particle_count(rt.levels, dict(p, scale_law=0, min_dl=p["max_dl"]))
    assert hi < rt.n_particles < lo
