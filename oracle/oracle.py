"""ctypes front end of the CPU FP64 oracle (oracle/mrsph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py (CPU
baseline and reference arms) use this module as the checker.  The product
library never imports it.

Parity status: partly pinned to the reference's own code.  The reference as a
program does not build here (it needs TBB, Boost.MPI and voro++) and ships no
tests or golden vectors; its smoothing kernels, their gradients and the level
law (base_cls_particle/particle.cpp) and its marching-cubes polygoniser
(geometry_tools/polygonise.cpp) are compiled from its sources into checker
libraries (build_ref.py) and the oracle's functions are checked against them
bit for bit (tests/test_ref_pinned.py, tests/golden/).  The rest is pinned by
known-answer tests derived from the equations (tests/test_oracle_kat.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "mrsph_oracle.cpp")
LIB = os.path.join(HERE, "_build", "libmrsph_oracle.so")
LIB_TUNED = os.path.join(HERE, "_build", "libmrsph_oracle_native.so")


def tuning_flags() -> list:
    """Host-CPU tuning of the timed CPU baseline build: -mcpu=native on Arm,
    -march=native elsewhere.  Results do not change: -ffp-contract=off (no
    fused multiply-add) and no fast-math hold for both builds."""
    import platform
    return ["-mcpu=native"] if platform.machine().lower() in ("aarch64", "arm64") else ["-march=native"]


def tuned() -> bool:
    """The natively tuned library is loaded when MRSPH_ORACLE_TUNED=1 (the
    benchmark's CPU legs set it before the first use of this module)."""
    return os.environ.get("MRSPH_ORACLE_TUNED") == "1"


def build(force: bool = False, native: bool = None) -> str:
    """Compile the oracle with g++ (OpenMP, no fused multiply-add); native
    adds the host-CPU tuning flags (default: tuned())."""
    native = tuned() if native is None else native
    out = LIB_TUNED if native else LIB
    os.makedirs(os.path.dirname(out), exist_ok=True)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(SRC):
        return out
    cmd = ["g++", "-O3", *(tuning_flags() if native else []), "-std=c++17", "-fopenmp", "-ffp-contract=off",
           "-fPIC", "-shared", SRC, "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


class OrcLevel(C.Structure):
    _fields_ = [("box_l", C.c_double * 3), ("dpkg", C.c_double * 3), ("num_pkg", C.c_int * 3),
                ("margin", C.c_int), ("phi", C.c_void_p), ("nx", C.c_void_p), ("ny", C.c_void_p),
                ("nz", C.c_void_p), ("curv", C.c_void_p), ("tag", C.c_void_p), ("active", C.c_void_p),
                ("chr", C.c_void_p), ("chr_idx", C.c_void_p)]


class OrcCtx(C.Structure):
    _fields_ = [("dim", C.c_int), ("kernel", C.c_int), ("cell_ratio", C.c_double), ("cutoff", C.c_double),
                ("angle_thres", C.c_double), ("nu_coeff", C.c_double), ("damp_coeff", C.c_double),
                ("min_dl", C.c_double), ("max_dl", C.c_double), ("max_phi", C.c_double),
                ("box_l", C.c_double * 3), ("box_r", C.c_double * 3), ("seed", C.c_ulonglong),
                ("nls", C.c_int), ("ls", C.POINTER(OrcLevel)), ("ncl", C.c_int),
                ("max_scale", C.c_double), ("min_scale", C.c_double), ("ini_num_cell", C.c_int * 3),
                ("cl_dcell", (C.c_double * 3) * 16), ("cl_ncell", (C.c_int * 3) * 16),
                ("cl_scale", C.c_double * 16), ("scale_law", C.c_int), ("middle_dl", C.c_double),
                ("max_curv", C.c_double), ("min_curv", C.c_double),
                ("nsing", C.c_int), ("sing", C.c_void_p), ("nseg", C.c_int), ("seg", C.c_void_p)]


_DBL_FIELDS = ["x", "y", "z", "vx", "vy", "vz"]
_INT_FIELDS = ["type", "id", "level"]
_DBL2_FIELDS = ["h", "scale", "phi", "curv", "nx", "ny", "nz", "sum", "rho", "vol", "nu"]
_ACC_FIELDS = ["ax", "ay", "az"]


class OrcState(C.Structure):
    _fields_ = ([("n", C.c_longlong)] + [(f, C.c_void_p) for f in _DBL_FIELDS]
                + [(f, C.c_void_p) for f in _INT_FIELDS] + [(f, C.c_void_p) for f in _DBL2_FIELDS]
                + [(f, C.c_void_p) for f in _ACC_FIELDS]
                + [("dt", C.c_double), ("max_v", C.c_double), ("step", C.c_longlong),
                   ("remapped", C.c_longlong)])


class OrcCvpParams(C.Structure):
    _fields_ = [("dim", C.c_int), ("num_vp", C.c_int), ("max_iter", C.c_int), ("pressure_step", C.c_int),
                ("error_tolerance", C.c_double), ("relax_ratio", C.c_double), ("box_l", C.c_double * 3),
                ("box_r", C.c_double * 3)]


class OrcCvpResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("error_max", C.c_double),
                ("total_energy", C.c_double)]


class OrcTriQuality(C.Structure):
    _fields_ = ([(f, C.c_longlong) for f in ("ntri", "nedge", "nedge_first", "ndeleted", "nerror")]
                + [(f, C.c_double) for f in ("max_angle", "min_angle", "max_aspect", "max_edge", "min_edge",
                                             "max_area", "min_area", "G_min", "G_avg", "min_angle_avg",
                                             "theta_30", "total_area")]
                + [("hist", C.c_longlong * 45)])


class OrcTetQuality(C.Structure):
    _fields_ = ([(f, C.c_longlong) for f in ("ntet", "nopen", "ndeleted", "ntie")]
                + [(f, C.c_double) for f in ("grid", "total_volume", "min_volume", "max_volume", "min_edge",
                                             "max_edge", "min_aspect", "max_aspect", "avg_aspect",
                                             "min_radius_ratio", "max_radius_ratio", "avg_radius_ratio",
                                             "min_dihedral", "max_dihedral", "avg_min_dihedral")]
                + [("nsmall_dihedral", C.c_longlong * 4), ("aspect_hist", C.c_longlong * 12),
                   ("radius_hist", C.c_longlong * 56), ("dihedral_hist", C.c_longlong * 45),
                   ("ntrunc", C.c_longlong)])


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.orc_define_levels.argtypes = [C.POINTER(OrcCtx)]
        L.orc_ls_build.argtypes = [C.POINTER(OrcCtx), C.c_int, C.POINTER(C.c_double)]
        L.orc_ls_characteristics.argtypes = [C.POINTER(OrcCtx), C.c_int]
        L.orc_kernel_W.argtypes = [C.c_int, C.c_int, C.c_longlong, C.c_void_p, C.c_double, C.c_void_p]
        L.orc_kernel_dW.argtypes = L.orc_kernel_W.argtypes
        L.orc_get_scale.argtypes = [C.POINTER(OrcCtx), C.c_double, C.c_double]
        L.orc_ls_curv_range.argtypes = [C.POINTER(OrcCtx), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_get_scale.restype = C.c_double
        L.orc_set_particle_scale.argtypes = [C.POINTER(OrcCtx), C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.orc_set_particle_scale.restype = C.c_int
        L.orc_philox.argtypes = [C.c_uint32] * 4 + [C.c_ulonglong, C.c_void_p]
        L.orc_sample.argtypes = [C.POINTER(OrcCtx), C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p]
        L.orc_seed.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState)]
        L.orc_pre_run.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState)]
        L.orc_phase_map.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_int]
        L.orc_cells.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_void_p]
        L.orc_neighbors.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_void_p, C.c_void_p,
                                    C.c_longlong]
        L.orc_neighbors.restype = C.c_longlong
        L.orc_density.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_void_p, C.c_void_p]
        L.orc_force.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_void_p, C.c_void_p, C.c_int]
        L.orc_reset_stage1.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState)]
        L.orc_steps.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcState), C.c_int]
        L.orc_steps.restype = C.c_longlong
        L.orc_num_threads.restype = C.c_int
        L.orc_triangulate.argtypes = [C.POINTER(OrcCtx), C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(OrcTriQuality)]
        L.orc_triangulate.restype = C.c_longlong
        L.orc_cvp.argtypes = [C.POINTER(OrcCvpParams), C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_void_p, C.c_void_p, C.POINTER(OrcCvpResult)]
        L.orc_cvp_lset.argtypes = [C.POINTER(OrcCtx), C.POINTER(OrcCvpParams), C.c_longlong, C.c_void_p,
                                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                   C.POINTER(C.c_int), C.POINTER(OrcCvpResult)]
        L.orc_segment_length.argtypes = [C.c_void_p] * 4
        L.orc_segment_length.restype = C.c_double
        L.orc_mc_table.argtypes = [C.c_void_p]
        L.orc_mc_area.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_double]
        L.orc_mc_area.restype = C.c_double
        L.orc_cut_cell.argtypes = [C.c_int, C.c_void_p, C.c_double, C.c_double, C.c_double,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_volume_mass.argtypes = [C.POINTER(OrcCtx), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_tetrahedralize.argtypes = [C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong,
                                         C.POINTER(OrcTetQuality)]
        L.orc_tetrahedralize.restype = C.c_longlong
        _lib = L
    return _lib


def mc_table() -> np.ndarray:
    """The oracle's marching-cubes table, 256 x 16 edge indices (-1 padded)."""
    t = np.zeros((256, 16), dtype=np.int8)
    lib().orc_mc_table(_p(t))
    return t


def mc_area(corners: np.ndarray, dx: float, dy: float, dz: float) -> float:
    """Marching-cubes area of a 3x3x3 corner lattice (get_area_MQ)."""
    c = np.ascontiguousarray(corners, dtype=np.float64).reshape(27)
    return float(lib().orc_mc_area(_p(c), dx, dy, dz))


def cut_cell(dim: int, nbhd: np.ndarray, dx: float, dy: float, dz: float):
    """(volume, area) of one CUT cell from its 3^D phi neighbourhood, given
    as 3x3x3 [x][y][z] (z index 0 in 2D)."""
    p = np.ascontiguousarray(nbhd, dtype=np.float64).reshape(27)
    v, a = C.c_double(0.0), C.c_double(0.0)
    lib().orc_cut_cell(dim, _p(p), dx, dy, dz, C.byref(v), C.byref(a))
    return v.value, a.value


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def middle_dl_of(p: dict, levels) -> float:
    """middle_dl of the curvature law: the given value, or 5 x the level-0
    level-set cell (fac_middel_dl = 5, sph_mesh_generation.cpp:271, level_set.cpp:940)."""
    m = float(p.get("middle_dl", 0.0))
    if m > 0:
        return m
    dim = p["dim"]
    return 5.0 * min(levels[0].dpkg[d] / 4.0 for d in range(dim))


class Oracle:
    """FP64 oracle for one geometry (mirrors the C-ABI handle of the product)."""

    def __init__(self, case):
        self.case = case
        p = case.params
        self.ctx = OrcCtx()
        c = self.ctx
        c.dim = p["dim"]
        c.kernel = p["kernel"]
        c.cell_ratio = p["cell_ratio"]
        c.cutoff = p["cutoff"]
        c.angle_thres = p["angle_thres"]
        c.nu_coeff = p["nu_coeff"]
        c.damp_coeff = p["damp_coeff"]
        c.min_dl = p["min_dl"]
        c.max_dl = p["max_dl"]
        for d in range(3):
            c.box_l[d] = p["box_l"][d]
            c.box_r[d] = p["box_r"][d]
        c.seed = p["seed"]
        # characteristic points and segments (3-vectors; z = 0 in 2D)
        sing = np.ascontiguousarray(case.extra.get("singularities", np.zeros((0, 3))), dtype=np.float64).reshape(-1, 3)
        seg = np.ascontiguousarray(case.extra.get("segments", np.zeros((0, 6))), dtype=np.float64).reshape(-1, 6)
        self.characteristics = {"singularities": sing, "segments": seg}
        c.nsing, c.sing = len(sing), (_p(sing) if len(sing) else None)
        c.nseg, c.seg = len(seg), (_p(seg) if len(seg) else None)
        has_chr = len(sing) > 0 or len(seg) > 0
        # level-set levels
        self._keep = []
        levels = case.levels
        arr = (OrcLevel * len(levels))()
        self.fields = []
        for i, lv in enumerate(levels):
            L = arr[i]
            for d in range(3):
                L.box_l[d] = lv.box_l[d]
                L.dpkg[d] = lv.dpkg[d]
                L.num_pkg[d] = lv.num_pkg[d]
            L.margin = lv.margin
            phi = np.ascontiguousarray(lv.phi, dtype=np.float64).ravel()
            f = {"phi": phi}
            for k in ("nx", "ny", "nz", "curv"):
                f[k] = np.zeros_like(phi)
            f["tag"] = np.zeros(phi.shape, dtype=np.int32)
            for k in ("phi", "nx", "ny", "nz", "curv", "tag"):
                setattr(L, k, _p(f[k]))
            if has_chr:
                f["chr"] = np.zeros(phi.shape, dtype=np.int32)
                f["chr_idx"] = np.full(phi.shape, -1, dtype=np.int32)
                L.chr, L.chr_idx = _p(f["chr"]), _p(f["chr_idx"])
            else:
                L.chr, L.chr_idx = None, None
            if lv.active is not None:
                act = np.ascontiguousarray(lv.active, dtype=np.uint8).ravel()
                f["active"] = act
                L.active = _p(act)
            else:
                L.active = None
            self.fields.append(f)
        self.levels_arr = arr
        c.nls = len(levels)
        c.ls = C.cast(arr, C.POINTER(OrcLevel))
        rc = lib().orc_define_levels(C.byref(c))
        if rc != 0:
            raise RuntimeError(f"orc_define_levels failed ({rc})")
        mp = 0.0
        cmax, cmin = 0.0, 1.e20
        for i in range(len(levels)):
            m = C.c_double(0.0)
            lib().orc_ls_build(C.byref(c), i, C.byref(m))
            if has_chr:
                lib().orc_ls_characteristics(C.byref(c), i)
            mp = max(mp, m.value)
            a_, b_ = C.c_double(0.0), C.c_double(0.0)
            lib().orc_ls_curv_range(C.byref(c), i, C.byref(a_), C.byref(b_))
            cmax, cmin = max(cmax, a_.value), min(cmin, b_.value)
        c.max_phi = mp
        c.max_curv, c.min_curv = cmax, cmin
        c.scale_law = int(p.get("scale_law", 0))
        c.middle_dl = middle_dl_of(p, levels)
        self.state = None
        self.arrays = {}

    # ------------------------------------------------------- volume / mass
    def volume_mass(self, level: int = -1):
        """Cut-cell volume, area and particle count of one level
        (Calculate_total_volume_mass + Get_num_particles).  Returns a dict of
        the totals and counts plus per-cell 'vol' and 'area' arrays over the
        full grid incl. margins."""
        if level < 0:
            level += self.ctx.nls
        ntot = self.fields[level]["phi"].size
        vol = np.zeros(ntot)
        area = np.zeros(ntot)
        tot = np.zeros(6)
        cnt = np.zeros(6, dtype=np.int64)
        lib().orc_volume_mass(C.byref(self.ctx), level, _p(vol), _p(area), _p(tot), _p(cnt))
        return {"total_mass": tot[0], "total_mass_surface": tot[1], "total_volume": tot[2],
                "total_area": tot[3], "total_mass_segment": tot[4], "total_length": tot[5],
                "num_interface_cell": int(cnt[0]), "num_particle_mesh": int(cnt[1]),
                "num_particle_surface": int(cnt[2]), "num_particle": int(cnt[3]),
                "num_particle_segment": int(cnt[4]), "num_particle_singularity": int(cnt[5]),
                "vol": vol, "area": area}

    @staticmethod
    def segment_length(mn, mx, v0, v1) -> float:
        """GeometryCalculator::Get_segment_length restated: the length of
        segment v0-v1 inside the box [mn, mx]."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (mn, mx, v0, v1)]
        return lib().orc_segment_length(*[_p(x) for x in a])

    # ----------------------------------------------------------------- state
    def alloc(self, n: int):
        a = {}
        for f in _DBL_FIELDS + _DBL2_FIELDS + _ACC_FIELDS:
            a[f] = np.zeros(n, dtype=np.float64)
        for f in _INT_FIELDS:
            a[f] = np.zeros(n, dtype=np.int32)
        a["id"][:] = np.arange(n, dtype=np.int32)
        a["scale"][:] = self.ctx.max_scale
        s = OrcState()
        s.n = n
        for f, v in a.items():
            setattr(s, f, _p(v))
        s.dt = 0.0
        s.step = 0
        self.state = s
        self.arrays = a
        return a

    def set_state(self, st: dict):
        """Load a state dictionary (FP64 arrays in particle-id order)."""
        n = len(st["x"])
        a = self.alloc(n)
        for k, v in st.items():
            if k in a:
                a[k][:] = v
        if "dt" in st:
            self.state.dt = float(st["dt"])
        if "step" in st:
            self.state.step = int(st["step"])

    def get_state(self) -> dict:
        out = {k: v.copy() for k, v in self.arrays.items()}
        out["dt"] = self.state.dt
        out["max_v"] = self.state.max_v
        out["step"] = self.state.step
        return out

    # ----------------------------------------------------------------- phases
    def seed(self, n: int):
        self.alloc(n)
        rc = lib().orc_seed(C.byref(self.ctx), C.byref(self.state))
        if rc != 0:
            raise RuntimeError("oracle seeding did not converge")

    def pre_run(self):
        lib().orc_pre_run(C.byref(self.ctx), C.byref(self.state))

    def phase_map(self, advect: bool = True):
        self.state.step += 1
        lib().orc_phase_map(C.byref(self.ctx), C.byref(self.state), 1 if advect else 0)

    def cells(self) -> np.ndarray:
        out = np.zeros((self.state.n, 4), dtype=np.int32)
        lib().orc_cells(C.byref(self.ctx), C.byref(self.state), _p(out))
        return out

    def neighbors(self):
        n = self.state.n
        off = np.zeros(n + 1, dtype=np.int64)
        tot = lib().orc_neighbors(C.byref(self.ctx), C.byref(self.state), _p(off), None, 0)
        nb = np.zeros(max(tot, 1), dtype=np.int32)
        lib().orc_neighbors(C.byref(self.ctx), C.byref(self.state), _p(off), _p(nb), tot)
        return off, nb[:tot]

    def density(self, off, nb):
        lib().orc_reset_stage1(C.byref(self.ctx), C.byref(self.state))
        lib().orc_density(C.byref(self.ctx), C.byref(self.state), _p(off), _p(nb))

    def force(self, off, nb, stage: int):
        lib().orc_force(C.byref(self.ctx), C.byref(self.state), _p(off), _p(nb), stage)

    def steps(self, k: int) -> int:
        return lib().orc_steps(C.byref(self.ctx), C.byref(self.state), k)

    def sample(self, xyz: np.ndarray):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = len(xyz)
        phi = np.zeros(n)
        nrm = np.zeros((n, 3))
        curv = np.zeros(n)
        tag = np.zeros(n, dtype=np.int32)
        lib().orc_sample(C.byref(self.ctx), n, _p(xyz), _p(phi), _p(nrm), _p(curv), _p(tag))
        return phi, nrm, curv, tag

    def cvp_lset(self, xyz, mass, mass_surface, vp_xyz, max_iter=800, error_tolerance=0.05, relax_ratio=0.8,
                 pressure_step=True):
        """Voronoi_lset::Partitioning_for_initial_VP_distribution restated
        (CVP/voronoi_lset.cpp:824-889) on weighted points with ghost VPs on
        this oracle's level set."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        vp = np.ascontiguousarray(vp_xyz, dtype=np.float64).reshape(-1, 3).copy()
        n, K = len(xyz), len(vp)
        pm = np.ascontiguousarray(mass, dtype=np.float64)
        ps = np.ascontiguousarray(mass_surface, dtype=np.float64)
        p = OrcCvpParams()
        p.dim, p.num_vp, p.max_iter, p.pressure_step = self.ctx.dim, K, max_iter, 1 if pressure_step else 0
        p.error_tolerance, p.relax_ratio = error_tolerance, relax_ratio
        for d in range(3):
            p.box_l[d] = self.case.params["box_l"][d]
            p.box_r[d] = self.case.params["box_r"][d]
        labels = np.zeros(n, dtype=np.int32)
        vmass = np.zeros(K)
        ghost = np.zeros((K, 3))
        ng = C.c_int(0)
        res = OrcCvpResult()
        lib().orc_cvp_lset(C.byref(self.ctx), C.byref(p), n, _p(xyz), _p(pm), _p(ps), _p(vp), _p(labels),
                           _p(vmass), _p(ghost), C.byref(ng), C.byref(res))
        out = {f: getattr(res, f) for f, _ in OrcCvpResult._fields_}
        out["ghosts"] = ghost[: ng.value].copy()
        return vp, labels, vmass, out

    def triangulate(self, xyz, type_, phi, off, nbr):
        """2D neighbour-graph triangulation + quality (graph_mesh.cpp:37-670), id space."""
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        t = np.ascontiguousarray(type_, dtype=np.int32)
        ph = np.ascontiguousarray(phi, dtype=np.float64)
        off = np.ascontiguousarray(off, dtype=np.int64)
        nbr = np.ascontiguousarray(nbr, dtype=np.int32)
        q = OrcTriQuality()
        n = len(xyz)
        ntri = lib().orc_triangulate(C.byref(self.ctx), n, _p(xyz), _p(t), _p(ph), _p(off), _p(nbr), None, 0, None)
        tris = np.zeros((max(ntri, 1), 3), dtype=np.int32)
        lib().orc_triangulate(C.byref(self.ctx), n, _p(xyz), _p(t), _p(ph), _p(off), _p(nbr), _p(tris), ntri,
                              C.byref(q))
        qd = {f: getattr(q, f) for f, _ in OrcTriQuality._fields_ if f != "hist"}
        qd["hist"] = list(q.hist)
        return tris[:ntri], qd

    def tetrahedralize(self, xyz, type_, h, off, nbr):
        """3D tetrahedralisation + tet quality (row F3), id space; see tetrahedralize()."""
        p = self.case.params
        return tetrahedralize(xyz, type_, h, off, nbr, p["cutoff"], p["box_l"], p["box_r"])

    def get_scale(self, phi: float, curv: float = 0.0) -> float:
        return lib().orc_get_scale(C.byref(self.ctx), phi, curv)

    def levels(self):
        c = self.ctx
        return {"ncl": c.ncl, "max_scale": c.max_scale, "min_scale": c.min_scale,
                "ncell": [list(c.cl_ncell[l]) for l in range(c.ncl)],
                "dcell": [list(c.cl_dcell[l]) for l in range(c.ncl)],
                "scale": [c.cl_scale[l] for l in range(c.ncl)]}


def kernel_W(kind: int, dim: int, dist: np.ndarray, h: float) -> np.ndarray:
    dist = np.ascontiguousarray(dist, dtype=np.float64)
    out = np.zeros_like(dist)
    lib().orc_kernel_W(kind, dim, len(dist), _p(dist), h, _p(out))
    return out


def kernel_dW(kind: int, dim: int, dist: np.ndarray, h: float) -> np.ndarray:
    dist = np.ascontiguousarray(dist, dtype=np.float64)
    out = np.zeros_like(dist)
    lib().orc_kernel_dW(kind, dim, len(dist), _p(dist), h, _p(out))
    return out


def set_particle_scale(h: float, scale: float, cutoff: float, max_scale: float, min_scale: float):
    """Particle_base::Set_particle_scale of the oracle: (new scale, flag)."""
    c = OrcCtx()
    c.cutoff = cutoff
    c.max_scale = max_scale
    c.min_scale = min_scale
    out = C.c_double(0.0)
    flag = lib().orc_set_particle_scale(C.byref(c), h, scale, C.byref(out))
    return out.value, int(flag)


def philox(c0, c1, c2, c3, seed):
    out = (C.c_uint32 * 4)()
    lib().orc_philox(c0, c1, c2, c3, seed, out)
    return list(out)


def cvp(dim, box_l, box_r, xyz, vp_xyz, mass=None, max_iter=4000, error_tolerance=0.05, relax_ratio=0.8,
        pressure_step=True):
    """Voronoi::Partitioning restated (CVP/voronoi.cpp:1376-1446) on weighted points."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    vp = np.ascontiguousarray(vp_xyz, dtype=np.float64).reshape(-1, 3).copy()
    n, K = len(xyz), len(vp)
    pm = np.ones(n) if mass is None else np.ascontiguousarray(mass, dtype=np.float64)
    p = OrcCvpParams()
    p.dim, p.num_vp, p.max_iter, p.pressure_step = dim, K, max_iter, 1 if pressure_step else 0
    p.error_tolerance, p.relax_ratio = error_tolerance, relax_ratio
    for d in range(3):
        p.box_l[d] = box_l[d]
        p.box_r[d] = box_r[d]
    labels = np.zeros(n, dtype=np.int32)
    vmass = np.zeros(K)
    res = OrcCvpResult()
    lib().orc_cvp(C.byref(p), n, _p(xyz), _p(pm), _p(vp), _p(labels), _p(vmass), C.byref(res))
    return vp, labels, vmass, {f: getattr(res, f) for f, _ in OrcCvpResult._fields_}


def num_threads() -> int:
    return lib().orc_num_threads()


def tetrahedralize(xyz, type_, h, off, nbr, cutoff, box_l, box_r):
    """Certified local Delaunay tets of the particles (the library's
    construction for Graphmeshcls::Reconstruct_tets, graph_mesh.cpp:981-1100,
    restated on the CPU) and their quality statistics
    (Tet_quality_statistics, :1967-2400): (tets (m x 4, ascending ids),
    quality dict)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
    t = np.ascontiguousarray(type_, dtype=np.int32)
    hh = np.ascontiguousarray(h, dtype=np.float64)
    off = np.ascontiguousarray(off, dtype=np.int64)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    bl = np.ascontiguousarray([float(box_l[d]) if d < len(box_l) else 0.0 for d in range(3)])
    br = np.ascontiguousarray([float(box_r[d]) if d < len(box_r) else 0.0 for d in range(3)])
    n = len(xyz)
    q = OrcTetQuality()
    args = (n, _p(xyz), _p(t), _p(hh), _p(off), _p(nbr), float(cutoff), _p(bl), _p(br))
    m = lib().orc_tetrahedralize(*args, None, 0, None)
    tets = np.zeros((max(m, 1), 4), dtype=np.int32)
    lib().orc_tetrahedralize(*args, _p(tets), m, C.byref(q))
    qd = {f: getattr(q, f) for f, _ in OrcTetQuality._fields_}
    for f in ("nsmall_dihedral", "aspect_hist", "radius_hist", "dihedral_hist"):
        qd[f] = list(getattr(q, f))
    return tets[:m], qd


def snap(xyz, box_l, box_r):
    """The tetrahedralisation's snapped positions: rint(x / g) g with g =
    2^(e - 52), 2^(e - 1) above every |coordinate| of the domain (and 1)."""
    m = max([1.0] + [abs(float(v)) for v in list(box_l) + list(box_r)])
    e = int(np.frexp(m)[1]) + 1
    g = np.ldexp(1.0, e - 52)
    return np.rint(np.asarray(xyz, dtype=np.float64) / g) * g
