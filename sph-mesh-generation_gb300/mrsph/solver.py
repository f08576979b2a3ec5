"""Host-side mirror of the reference's relaxation driver.

``SPHMeshGeneration`` keeps the entry-point names of the reference's
``SPH_mesh_generation`` class (src/sph_mesh_generation/sph_mesh_generation.h:10-154,
driven by Solver, src/solver.cpp:35-321) and forwards every call through the C
ABI of include/mrsph_relax.h to the CUDA engine.  Arrays in and out are numpy,
in particle-id order.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib as L
from .cases import Case


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class SPHMeshGeneration:
    """One geometry on one GPU (the reference's SPH_mesh_generation + Levelset)."""

    def __init__(self, case: Case, precision: Optional[str] = None, device: int = 0,
                 neighbor_cap: int = 0):
        self.lib = L.load()
        self.case = case
        p = dict(case.params)
        if precision is not None:
            p["precision"] = {"fp64": L.FP64_PLAIN, "fp32": L.FP32_SPLIT}[precision]
        self.params = p
        prm = L.Params()
        prm.dim = p["dim"]
        prm.kernel = p["kernel"]
        prm.precision = p["precision"]
        prm.cell_ratio = p["cell_ratio"]
        prm.cutoff = p["cutoff"]
        prm.angle_thres = p["angle_thres"]
        prm.nu_coeff = p["nu_coeff"]
        prm.damp_coeff = p["damp_coeff"]
        prm.min_dl = p["min_dl"]
        prm.max_dl = p["max_dl"]
        for d in range(3):
            prm.box_l[d] = p["box_l"][d]
            prm.box_r[d] = p["box_r"][d]
        prm.seed = p["seed"]
        prm.neighbor_cap = neighbor_cap or p.get("neighbor_cap", 0)
        prm.device = device
        prm.scale_law = int(p.get("scale_law", 0))
        prm.middle_dl = float(p.get("middle_dl", 0.0))
        h = C.c_void_p()
        L.check(self.lib.mrsph_create(C.byref(prm), C.byref(h)), None, "mrsph_create")
        self.h = h
        self.n = 0
        self._set_levelset()

    # ------------------------------------------------------------------ setup
    def _set_levelset(self):
        levels = self.case.levels
        extra = getattr(self.case, "extra", None) or {}
        sing = np.ascontiguousarray(np.asarray(extra.get("singularities", np.zeros((0, 3))),
                                               dtype=np.float64).reshape(-1, 3))
        seg = np.ascontiguousarray(np.asarray(extra.get("segments", np.zeros((0, 6))),
                                              dtype=np.float64).reshape(-1, 6))
        if len(sing) or len(seg):
            # Levelset::singularity / ::segment, tagged by Get_singularity_tag
            # and Get_segment_tag when the level set is built
            L.check(self.lib.mrsph_set_characteristics(
                self.h, len(sing), sing.ctypes.data_as(C.c_void_p) if len(sing) else None,
                len(seg), seg.ctypes.data_as(C.c_void_p) if len(seg) else None),
                self.h, "mrsph_set_characteristics")
        arr = (L.LevelsetLevel * len(levels))()
        self._ls_keep = []
        for i, lv in enumerate(levels):
            a = arr[i]
            for d in range(3):
                a.box_l[d] = lv.box_l[d]
                a.dpkg[d] = lv.dpkg[d]
                a.num_pkg[d] = lv.num_pkg[d]
            a.margin = lv.margin
            phi = np.ascontiguousarray(lv.phi, dtype=np.float64)
            self._ls_keep.append(phi)
            a.phi = phi.ctypes.data_as(C.c_void_p)
            if lv.active is not None:
                act = np.ascontiguousarray(lv.active, dtype=np.uint8)
                self._ls_keep.append(act)
                a.active = act.ctypes.data_as(C.c_void_p)
            else:
                a.active = None
        L.check(self.lib.mrsph_set_levelset(self.h, len(levels), arr), self.h, "mrsph_set_levelset")

    def close(self):
        if getattr(self, "h", None):
            self.lib.mrsph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --------------------------------------------------- reference entry points
    def Initialize_case(self, n: Optional[int] = None, cut_cell_count: bool = False):
        """Random_particle_distribution + Pre_run (sph_mesh_generation.cpp:594-1050).
        n defaults to the workload's count, or with cut_cell_count to the
        reference's own (Get_num_particles over the cut-cell volume pass of the
        finest level, sph_mesh_generation.cpp:900-940)."""
        if n is None and cut_cell_count:
            n = self.Get_num_particles()
        n = int(n if n is not None else self.case.n_particles)
        L.check(self.lib.mrsph_seed(self.h, n), self.h, "mrsph_seed")
        self.n = n

    def SPH_run_mesh_generation(self, nsteps: int = 1):
        """SPH_mesh_generation::SPH_run_mesh_generation x nsteps (asynchronous)."""
        L.check(self.lib.mrsph_step(self.h, int(nsteps)), self.h, "mrsph_step")

    def step_timed(self, nsteps: int) -> float:
        """nsteps relaxation steps; returns device milliseconds (CUDA events on the engine stream)."""
        ms = C.c_double(0)
        L.check(self.lib.mrsph_step_timed(self.h, int(nsteps), C.byref(ms)), self.h, "mrsph_step_timed")
        return ms.value

    def profile_steps(self, nsteps: int) -> dict:
        """Mean device milliseconds per step of each phase (eager launches)."""
        out = np.zeros(len(L.TIMERS))
        L.check(self.lib.mrsph_profile_steps(self.h, int(nsteps), _ptr(out), len(L.TIMERS)), self.h,
                "mrsph_profile_steps")
        return dict(zip(L.TIMERS, out.tolist()))

    def Get_timestep(self) -> float:
        return self.stats()["dt"]

    # ------------------------------------------------------------- parity API
    def set_state(self, st: dict, pre_run: bool = False):
        xyz = np.ascontiguousarray(st["xyz"], dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        keep = [xyz]
        s = L.StateIn()
        s.xyz = _ptr(xyz)

        def opt(key, dtype, shape):
            if key not in st or st[key] is None:
                return None
            a = np.ascontiguousarray(st[key], dtype=dtype).reshape(shape)
            keep.append(a)
            return _ptr(a)

        s.v = opt("v", np.float64, (-1, 3))
        s.type = opt("type", np.int32, (-1,))
        s.h = opt("h", np.float64, (-1,))
        s.level = opt("level", np.int32, (-1,))
        s.nu = opt("nu", np.float64, (-1,))
        s.dt = float(st.get("dt", 0.0))
        s.step = int(st.get("step", 0))
        L.check(self.lib.mrsph_set_state(self.h, n, C.byref(s), 1 if pre_run else 0), self.h, "mrsph_set_state")
        self.n = n

    def run_phase(self, phase: int):
        L.check(self.lib.mrsph_run_phase(self.h, phase), self.h, "mrsph_run_phase")

    def sync(self):
        L.check(self.lib.mrsph_sync(self.h), self.h, "mrsph_sync")

    def stats(self) -> dict:
        s = L.Stats()
        L.check(self.lib.mrsph_get_stats(self.h, C.byref(s)), self.h, "mrsph_get_stats")
        return {f: getattr(s, f) for f, _ in L.Stats._fields_}

    def particles(self, fields=("xyz", "v", "type", "h", "level", "phi", "curv", "norm", "sum", "rho", "nu",
                                "a1", "a2")) -> dict:
        n = self.n
        out = {}
        v = L.ParticleView()
        for f in fields:
            if f in ("xyz", "v", "norm", "a1", "a2"):
                out[f] = np.zeros((n, 3), dtype=np.float64)
            elif f in ("type", "level"):
                out[f] = np.zeros(n, dtype=np.int32)
            else:
                out[f] = np.zeros(n, dtype=np.float64)
            setattr(v, f, _ptr(out[f]))
        L.check(self.lib.mrsph_get_particles(self.h, C.byref(v)), self.h, "mrsph_get_particles")
        return out

    def cells(self):
        lc = np.zeros((self.n, 4), dtype=np.int32)
        ids = np.zeros(self.n, dtype=np.int32)
        L.check(self.lib.mrsph_get_cells(self.h, _ptr(lc), _ptr(ids)), self.h, "mrsph_get_cells")
        return lc, ids

    def neighbors(self):
        tot = C.c_longlong(0)
        L.check(self.lib.mrsph_get_neighbors(self.h, None, None, 0, C.byref(tot)), self.h, "mrsph_get_neighbors")
        off = np.zeros(self.n + 1, dtype=np.int64)
        nb = np.zeros(max(tot.value, 1), dtype=np.int32)
        L.check(self.lib.mrsph_get_neighbors(self.h, _ptr(off), _ptr(nb), tot.value, C.byref(tot)), self.h,
                "mrsph_get_neighbors")
        return off, nb[: tot.value]

    def levelset_fields(self, level: int):
        lv = self.case.levels[level]
        shp = lv.phi.shape
        out = {k: np.zeros(shp, dtype=np.float64) for k in ("nx", "ny", "nz", "curv")}
        out["tag"] = np.zeros(shp, dtype=np.uint8)
        mp = C.c_double(0)
        L.check(self.lib.mrsph_get_levelset(self.h, level, _ptr(out["nx"]), _ptr(out["ny"]), _ptr(out["nz"]),
                                            _ptr(out["curv"]), _ptr(out["tag"]), C.byref(mp)), self.h,
                "mrsph_get_levelset")
        out["max_phi"] = mp.value
        return out

    def characteristic_tags(self, level: int) -> np.ndarray:
        """Per cell of one level: 0 (NORMAL), k + 1 (on segment k) or -(k + 1)
        (at singularity point k)."""
        out = np.zeros(self.case.levels[level].phi.shape, dtype=np.int32)
        L.check(self.lib.mrsph_get_characteristics(self.h, level, _ptr(out)), self.h, "mrsph_get_characteristics")
        return out

    def sample_levelset(self, xyz: np.ndarray):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        phi = np.zeros(n)
        nrm = np.zeros((n, 3))
        curv = np.zeros(n)
        tag = np.zeros(n, dtype=np.int32)
        L.check(self.lib.mrsph_sample_levelset(self.h, n, _ptr(xyz), _ptr(phi), _ptr(nrm), _ptr(curv), _ptr(tag)),
                self.h, "mrsph_sample_levelset")
        return phi, nrm, curv, tag

    def volume_mass(self, level: int = -1, cells: bool = False) -> dict:
        """Cut-cell volume, surface area and particle numbers of one level-set
        level (Levelset::Calculate_total_volume_mass + Get_num_particles).
        With cells=True the dict also holds per-cell 'vol' and 'area' arrays
        shaped like the level's phi."""
        s = L.VolumeMassStats()
        lv = self.case.levels[level]
        vol = area = None
        if cells:
            vol = np.zeros(lv.phi.shape)
            area = np.zeros(lv.phi.shape)
        L.check(self.lib.mrsph_volume_mass(self.h, level, C.byref(s), _ptr(vol) if cells else None,
                                           _ptr(area) if cells else None), self.h, "mrsph_volume_mass")
        out = {f: getattr(s, f) for f, _ in L.VolumeMassStats._fields_}
        if cells:
            out["vol"], out["area"] = vol, area
        return out

    def Get_num_particles(self, level: int = -1) -> int:
        """SPH_mesh_generation::Get_num_particles (sph_mesh_generation.cpp:900-940)
        over the cut-cell volume pass of one level."""
        return int(self.volume_mass(level)["num_particle"])

    def sample_levelset_noalloc(self, xyz: np.ndarray):
        """Same as sample_levelset without any device allocation (<= 65536 points)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        phi = np.zeros(n)
        nrm = np.zeros((n, 3))
        curv = np.zeros(n)
        tag = np.zeros(n, dtype=np.int32)
        L.check(self.lib.mrsph_sample_levelset_noalloc(self.h, n, _ptr(xyz), _ptr(phi), _ptr(nrm), _ptr(curv),
                                                       _ptr(tag)), self.h, "mrsph_sample_levelset_noalloc")
        return phi, nrm, curv, tag

    # ------------------------------------------------------------------ CVP
    @staticmethod
    def _cvp_params(num_vp, max_iter, tol, relax, pressure_step):
        p = L.CvpParams()
        p.num_vp = int(num_vp)
        p.max_iter = int(max_iter)
        p.pressure_step = 1 if pressure_step else 0
        p.error_tolerance = float(tol)
        p.relax_ratio = float(relax)
        return p

    def Partitioning(self, vp_xyz: np.ndarray, max_iter: int = 4000, error_tolerance: float = 0.05,
                     relax_ratio: float = 0.8, pressure_step: bool = True):
        """Voronoi::Partitioning of the current particles (CVP/voronoi.cpp:1376-1446)."""
        vp = np.ascontiguousarray(vp_xyz, dtype=np.float64).reshape(-1, 3).copy()
        K = len(vp)
        labels = np.zeros(self.n, dtype=np.int32)
        mass = np.zeros(K)
        res = L.CvpResult()
        prm = self._cvp_params(K, max_iter, error_tolerance, relax_ratio, pressure_step)
        L.check(self.lib.mrsph_cvp(self.h, C.byref(prm), _ptr(vp), _ptr(labels), _ptr(mass), C.byref(res)),
                self.h, "mrsph_cvp")
        return vp, labels, mass, {f: getattr(res, f) for f, _ in L.CvpResult._fields_}

    def partition_points(self, xyz: np.ndarray, vp_xyz: np.ndarray, mass: Optional[np.ndarray] = None,
                         max_iter: int = 4000, error_tolerance: float = 0.05, relax_ratio: float = 0.8,
                         pressure_step: bool = True):
        """CVP of given weighted points (e.g. level-set packages, Voronoi_lset)."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        vp = np.ascontiguousarray(vp_xyz, dtype=np.float64).reshape(-1, 3).copy()
        m = None if mass is None else np.ascontiguousarray(mass, dtype=np.float64)
        K = len(vp)
        labels = np.zeros(len(xyz), dtype=np.int32)
        vmass = np.zeros(K)
        res = L.CvpResult()
        prm = self._cvp_params(K, max_iter, error_tolerance, relax_ratio, pressure_step)
        L.check(self.lib.mrsph_cvp_points(self.h, len(xyz), _ptr(xyz), _ptr(m), C.byref(prm), _ptr(vp),
                                          _ptr(labels), _ptr(vmass), C.byref(res)), self.h, "mrsph_cvp_points")
        return vp, labels, vmass, {f: getattr(res, f) for f, _ in L.CvpResult._fields_}

    def lset_packages(self, level: int = 0):
        """The interior packages of one level-set level with mass: centres and
        total / surface mass, Levelset_package::Calculate_volume_mass
        (lset_package.cpp:1283-1397): sum of vol / scale^D and of area /
        scale^(D-1) over the package's cells, scale the cell's target spacing.
        Returns (xyz, mass, mass_surface) in package order (x fastest)."""
        from .io import cell_scale
        lv = self.case.levels[level]
        dim = self.case.params["dim"]
        vm = self.volume_mass(level, cells=True)
        sc = cell_scale(self, level)
        m = lv.margin
        with np.errstate(divide="ignore", invalid="ignore"):
            cm = np.where(vm["vol"] > 0, vm["vol"] / sc ** dim, 0.0)
            cs = np.where(vm["area"] > 0, vm["area"] / sc ** (dim - 1), 0.0)
        npk = [lv.num_pkg[d] + 2 * m if d < dim else 1 for d in range(3)]
        cz = 4 if dim == 3 else 1
        def per_pkg(a):
            a = a.reshape(npk[2], cz, npk[1], 4, npk[0], 4)
            return a.sum(axis=(1, 3, 5))
        pm, ps = per_pkg(cm), per_pkg(cs)
        sl = (slice(m, -m) if dim == 3 else slice(None), slice(m, -m), slice(m, -m))
        pm, ps = pm[sl], ps[sl]
        idx = np.stack(np.meshgrid(*[np.arange(pm.shape[a]) for a in range(3)], indexing="ij"), -1).reshape(-1, 3)
        centre = np.zeros((len(idx), 3))
        for d in range(dim):
            centre[:, d] = lv.box_l[d] + (idx[:, 2 - d] + 0.5) * lv.dpkg[d]
        keep = pm.ravel() > 0
        return centre[keep], pm.ravel()[keep], ps.ravel()[keep]

    def partition_lset(self, xyz: np.ndarray, mass: np.ndarray, mass_surface: np.ndarray, vp_xyz: np.ndarray,
                       max_iter: int = 800, error_tolerance: float = 0.05, relax_ratio: float = 0.8,
                       pressure_step: bool = True):
        """Voronoi_lset::Partitioning_for_initial_VP_distribution
        (CVP/voronoi_lset.cpp:824-889): the level-set partition of weighted
        package centres with ghost VPs.  Returns (vp, labels (-1: nearest a
        ghost), vp mass, result dict incl. 'ghosts')."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        pm = np.ascontiguousarray(mass, dtype=np.float64)
        ps = np.ascontiguousarray(mass_surface, dtype=np.float64)
        vp = np.ascontiguousarray(vp_xyz, dtype=np.float64).reshape(-1, 3).copy()
        K = len(vp)
        labels = np.zeros(len(xyz), dtype=np.int32)
        vmass = np.zeros(K)
        ghost = np.zeros((K, 3))
        ng = C.c_int(0)
        res = L.CvpResult()
        prm = self._cvp_params(K, max_iter, error_tolerance, relax_ratio, pressure_step)
        L.check(self.lib.mrsph_cvp_lset(self.h, len(xyz), _ptr(xyz), _ptr(pm), _ptr(ps), C.byref(prm), _ptr(vp),
                                        _ptr(labels), _ptr(vmass), _ptr(ghost), C.byref(ng), C.byref(res)),
                self.h, "mrsph_cvp_lset")
        out = {f: getattr(res, f) for f, _ in L.CvpResult._fields_}
        out["ghosts"] = ghost[: ng.value].copy()
        return vp, labels, vmass, out

    # -------------------------------------------------------- triangulation
    def Reconstruct_tris(self):
        """2D triangle mesh of the current particles and its quality statistics
        (Graphmeshcls::Reconstruct_tris, geometry_tools/graph_mesh.cpp:37-409, on the
        local-Voronoi graph of Voronoi_construction::Local_VD_generation,
        geometry_tools/voronoi_construction.cpp:6-127; Tri_quality_statistics,
        graph_mesh.cpp:411-670).  Returns (tris (ntri x 3 ids), quality dict)."""
        q = L.TriQuality()
        nt = C.c_longlong(0)
        L.check(self.lib.mrsph_triangulate(self.h, None, 0, C.byref(nt), None), self.h, "mrsph_triangulate")
        tris = np.zeros((max(nt.value, 1), 3), dtype=np.int32)
        L.check(self.lib.mrsph_triangulate(self.h, _ptr(tris), nt.value, C.byref(nt), C.byref(q)), self.h,
                "mrsph_triangulate")
        out = {f: getattr(q, f) for f, _ in L.TriQuality._fields_ if f != "hist"}
        out["hist"] = np.array(q.hist[:], dtype=np.int64)
        return tris[: nt.value], out

    def Reconstruct_tets(self):
        """3D tet mesh of the current particles and its quality statistics
        (Graphmeshcls::Reconstruct_tets, geometry_tools/graph_mesh.cpp:981-1100,
        with the deletion rule of Check_whether_this_tet_should_be_delete,
        :675-979; Tet_quality_statistics, :1967-2400): the Delaunay tets whose
        circumsphere lies in the neighbour ball of one of their particles.
        Returns (tets (ntet x 4 ascending ids), quality dict)."""
        q = L.TetQuality()
        nt = C.c_longlong(0)
        tets = np.zeros((8 * max(self.n, 1), 4), dtype=np.int32)
        L.check(self.lib.mrsph_tetrahedralize(self.h, _ptr(tets), len(tets), C.byref(nt), C.byref(q)), self.h,
                "mrsph_tetrahedralize")
        if nt.value > len(tets):
            tets = np.zeros((nt.value, 4), dtype=np.int32)
            L.check(self.lib.mrsph_tetrahedralize(self.h, _ptr(tets), len(tets), C.byref(nt), C.byref(q)), self.h,
                    "mrsph_tetrahedralize")
        out = {f: getattr(q, f) for f, _ in L.TetQuality._fields_}
        for f in ("nsmall_dihedral", "aspect_hist", "radius_hist", "dihedral_hist"):
            out[f] = np.array(getattr(q, f)[:], dtype=np.int64)
        return tets[: nt.value], out

    def upload_positions(self, xyz: np.ndarray):
        L.check(self.lib.mrsph_upload_positions(self.h, _ptr(xyz)), self.h, "mrsph_upload_positions")

    def download_positions(self, out: np.ndarray):
        L.check(self.lib.mrsph_download_positions(self.h, _ptr(out)), self.h, "mrsph_download_positions")
        return out


BATCH_MODES = {"streams": 0, "persistent": 1, "phases": 2}


class BatchRelaxation:
    """Many independent geometries relaxed together (mrsph_batch_*).  Modes:
    "persistent" (default for FP32-split handles: one cooperative launch of
    the persistent batch kernel runs up to 32 steps of every geometry),
    "phases" (the same work lists, one launch per phase) and "streams" (each
    handle's own step graph on its own stream; FP64-plain batches).  Each
    handle's results equal those of stepping it alone."""

    def __init__(self, solvers, mode: str = None):
        self.solvers = list(solvers)
        self.lib = L.load()
        arr = (C.c_void_p * len(self.solvers))(*[s.h for s in self.solvers])
        b = C.c_void_p()
        rc = self.lib.mrsph_batch_create(arr, len(self.solvers), C.byref(b))
        if rc != 0:
            raise L.MrsphError(f"mrsph_batch_create failed ({rc})")
        self.b = b
        if mode is not None:
            self.set_mode(mode)

    def set_mode(self, mode: str):
        self._check(self.lib.mrsph_batch_set_mode(self.b, BATCH_MODES[mode]), "mrsph_batch_set_mode")

    @property
    def mode(self) -> str:
        m, g = C.c_int(0), C.c_int(0)
        self._check(self.lib.mrsph_batch_get_mode(self.b, C.byref(m), C.byref(g)), "mrsph_batch_get_mode")
        return {v: k for k, v in BATCH_MODES.items()}[m.value]

    @property
    def graph_captured(self) -> bool:
        m, g = C.c_int(0), C.c_int(0)
        self._check(self.lib.mrsph_batch_get_mode(self.b, C.byref(m), C.byref(g)), "mrsph_batch_get_mode")
        return bool(g.value)

    def _check(self, rc, what):
        if rc != 0:
            buf = C.create_string_buffer(1024)
            self.lib.mrsph_batch_last_error(self.b, buf, 1024)
            raise L.MrsphError(f"{what} failed ({rc}): {buf.value.decode(errors='replace')}")

    def SPH_run_mesh_generation(self, nsteps: int = 1):
        self._check(self.lib.mrsph_batch_step(self.b, int(nsteps)), "mrsph_batch_step")

    def step_timed(self, nsteps: int) -> float:
        ms = C.c_double(0)
        self._check(self.lib.mrsph_batch_step_timed(self.b, int(nsteps), C.byref(ms)), "mrsph_batch_step_timed")
        return ms.value

    def sync(self):
        self._check(self.lib.mrsph_batch_sync(self.b), "mrsph_batch_sync")

    def close(self):
        if getattr(self, "b", None):
            self.lib.mrsph_batch_destroy(self.b)
            self.b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def barrier_selftest(device: int = 0, limit_ms: float = 200.0) -> bool:
    """The persistent batch kernel's bounded barrier wait: a two-block
    cooperative launch in which one block never arrives; True when the other
    gave up after limit_ms and raised the error bit."""
    lib = L.load()
    raised = C.c_int(0)
    rc = lib.mrsph_batch_barrier_selftest(int(device), float(limit_ms), C.byref(raised))
    if rc != 0:
        raise L.MrsphError(f"mrsph_batch_barrier_selftest failed ({rc})")
    return bool(raised.value)
