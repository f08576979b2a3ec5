"""ctypes binding of the C ABI in include/mrsph_relax.h (libmrsph_relax.so).

There is no CPU fallback: if the CUDA library is missing or cannot be loaded,
loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

# MRSPH_LIB selects another build of the library (the autotuner times its
# candidates through it)
LIB_PATH = os.environ.get("MRSPH_LIB", _build.LIB)

KERNEL_HYPERBOLIC, KERNEL_CUBIC, KERNEL_WENDLAND, KERNEL_GAUSSIAN, KERNEL_QUINTIC = range(5)
FP64_PLAIN, FP32_SPLIT = 0, 1
REAL, SURFACE, SINGULARITY, SEGMENT = 0, 1, 2, 3
PHASE_MAP, PHASE_BIN, PHASE_DENSITY, PHASE_FORCE1, PHASE_FORCE2 = 1, 2, 3, 4, 5
TIMERS = ("map", "scan", "sort", "reorder", "density", "force1", "force2")
FLAG_REMAP_EXHAUSTED, FLAG_SEED_EXHAUSTED, FLAG_LEVEL_CLAMPED, FLAG_NEIGHBOR_SPILL = 1, 2, 4, 8
FLAG_CAPACITY_CLAMPED = 16


class Params(C.Structure):
    _fields_ = [("dim", C.c_int), ("kernel", C.c_int), ("precision", C.c_int), ("cell_ratio", C.c_double),
                ("cutoff", C.c_double), ("angle_thres", C.c_double), ("nu_coeff", C.c_double),
                ("damp_coeff", C.c_double), ("min_dl", C.c_double), ("max_dl", C.c_double),
                ("box_l", C.c_double * 3), ("box_r", C.c_double * 3), ("seed", C.c_ulonglong),
                ("neighbor_cap", C.c_int), ("device", C.c_int), ("scale_law", C.c_int), ("middle_dl", C.c_double)]


class LevelsetLevel(C.Structure):
    _fields_ = [("box_l", C.c_double * 3), ("dpkg", C.c_double * 3), ("num_pkg", C.c_int * 3),
                ("margin", C.c_int), ("phi", C.c_void_p), ("active", C.c_void_p)]


class Stats(C.Structure):
    _fields_ = [("dt", C.c_double), ("dt_stage1", C.c_double), ("max_v", C.c_double), ("step", C.c_longlong),
                ("n", C.c_longlong), ("n_surface", C.c_longlong), ("pairs", C.c_longlong),
                ("remapped", C.c_longlong), ("pairs_total", C.c_longlong), ("flags", C.c_int), ("num_cell_levels", C.c_int),
                ("num_cells", C.c_longlong), ("max_phi", C.c_double)]


class ParticleView(C.Structure):
    _fields_ = [(f, C.c_void_p) for f in ("xyz", "v", "type", "h", "level", "phi", "curv", "norm", "sum", "rho",
                                          "nu", "a1", "a2")]


class CvpParams(C.Structure):
    _fields_ = [("num_vp", C.c_int), ("max_iter", C.c_int), ("pressure_step", C.c_int),
                ("error_tolerance", C.c_double), ("relax_ratio", C.c_double)]


class CvpResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("error_max", C.c_double),
                ("total_energy", C.c_double)]


class TriQuality(C.Structure):
    _fields_ = ([(k, C.c_longlong) for k in ("ntri", "nedge", "nedge_first", "ndeleted", "nerror")] +
                [(k, C.c_double) for k in ("max_angle", "min_angle", "max_aspect", "max_edge", "min_edge",
                                           "max_area", "min_area", "G_min", "G_avg", "min_angle_avg", "theta_30",
                                           "total_area")] +
                [("hist", C.c_longlong * 45)])


class TetQuality(C.Structure):
    _fields_ = ([(k, C.c_longlong) for k in ("ntet", "nopen", "ndeleted", "ntie")] +
                [(k, C.c_double) for k in ("grid", "total_volume", "min_volume", "max_volume", "min_edge", "max_edge",
                                           "min_aspect", "max_aspect", "avg_aspect", "min_radius_ratio",
                                           "max_radius_ratio", "avg_radius_ratio", "min_dihedral", "max_dihedral",
                                           "avg_min_dihedral")] +
                [("nsmall_dihedral", C.c_longlong * 4), ("aspect_hist", C.c_longlong * 12),
                 ("radius_hist", C.c_longlong * 56), ("dihedral_hist", C.c_longlong * 45), ("ntrunc", C.c_longlong)])


class VolumeMassStats(C.Structure):
    _fields_ = ([(k, C.c_double) for k in ("total_mass", "total_mass_surface", "total_volume", "total_area")] +
                [(k, C.c_longlong) for k in ("num_interface_cell", "num_particle_mesh", "num_particle_surface",
                                             "num_particle")] +
                [("device_ms", C.c_double), ("total_mass_segment", C.c_double), ("total_length", C.c_double),
                 ("num_particle_segment", C.c_longlong), ("num_particle_singularity", C.c_longlong)])


class StateIn(C.Structure):
    _fields_ = [("xyz", C.c_void_p), ("v", C.c_void_p), ("type", C.c_void_p), ("h", C.c_void_p),
                ("level", C.c_void_p), ("nu", C.c_void_p), ("dt", C.c_double), ("step", C.c_longlong)]


EXPORTS = {
    "mrsph_version": ([], C.c_int),
    "mrsph_create": ([C.POINTER(Params), C.POINTER(C.c_void_p)], C.c_int),
    "mrsph_destroy": ([C.c_void_p], C.c_int),
    "mrsph_last_error": ([C.c_void_p, C.c_char_p, C.c_size_t], C.c_int),
    "mrsph_set_levelset": ([C.c_void_p, C.c_int, C.POINTER(LevelsetLevel)], C.c_int),
    "mrsph_set_characteristics": ([C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "mrsph_get_characteristics": ([C.c_void_p, C.c_int, C.c_void_p], C.c_int),
    "mrsph_get_levelset": ([C.c_void_p, C.c_int] + [C.c_void_p] * 5 + [C.POINTER(C.c_double)], C.c_int),
    "mrsph_volume_mass": ([C.c_void_p, C.c_int, C.POINTER(VolumeMassStats), C.c_void_p, C.c_void_p], C.c_int),
    "mrsph_sample_levelset": ([C.c_void_p, C.c_longlong] + [C.c_void_p] * 5, C.c_int),
    "mrsph_sample_levelset_noalloc": ([C.c_void_p, C.c_longlong] + [C.c_void_p] * 5, C.c_int),
    "mrsph_seed": ([C.c_void_p, C.c_longlong], C.c_int),
    "mrsph_set_state": ([C.c_void_p, C.c_longlong, C.POINTER(StateIn), C.c_int], C.c_int),
    "mrsph_step": ([C.c_void_p, C.c_int], C.c_int),
    "mrsph_run_phase": ([C.c_void_p, C.c_int], C.c_int),
    "mrsph_sync": ([C.c_void_p], C.c_int),
    "mrsph_step_timed": ([C.c_void_p, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "mrsph_profile_steps": ([C.c_void_p, C.c_int, C.c_void_p, C.c_int], C.c_int),
    "mrsph_get_stats": ([C.c_void_p, C.POINTER(Stats)], C.c_int),
    "mrsph_get_particles": ([C.c_void_p, C.POINTER(ParticleView)], C.c_int),
    "mrsph_get_cells": ([C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
    "mrsph_get_neighbors": ([C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)], C.c_int),
    "mrsph_cvp": ([C.c_void_p, C.POINTER(CvpParams), C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(CvpResult)],
                  C.c_int),
    "mrsph_cvp_points": ([C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p, C.POINTER(CvpParams), C.c_void_p,
                          C.c_void_p, C.c_void_p, C.POINTER(CvpResult)], C.c_int),
    "mrsph_cvp_lset": ([C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(CvpParams),
                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.POINTER(CvpResult)],
                       C.c_int),
    "mrsph_triangulate": ([C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong), C.POINTER(TriQuality)],
                          C.c_int),
    "mrsph_tetrahedralize": ([C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong),
                              C.POINTER(TetQuality)], C.c_int),
    "mrsph_batch_create": ([C.c_void_p, C.c_int, C.POINTER(C.c_void_p)], C.c_int),
    "mrsph_batch_destroy": ([C.c_void_p], C.c_int),
    "mrsph_batch_last_error": ([C.c_void_p, C.c_char_p, C.c_size_t], C.c_int),
    "mrsph_batch_step": ([C.c_void_p, C.c_int], C.c_int),
    "mrsph_batch_step_timed": ([C.c_void_p, C.c_int, C.POINTER(C.c_double)], C.c_int),
    "mrsph_batch_sync": ([C.c_void_p], C.c_int),
    "mrsph_batch_set_mode": ([C.c_void_p, C.c_int], C.c_int),
    "mrsph_batch_get_mode": ([C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)], C.c_int),
    "mrsph_batch_barrier_selftest": ([C.c_int, C.c_double, C.POINTER(C.c_int)], C.c_int),
    "mrsph_upload_positions": ([C.c_void_p, C.c_void_p], C.c_int),
    "mrsph_download_positions": ([C.c_void_p, C.c_void_p], C.c_int),
}

_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libmrsph_relax.so (building it when absent).  Raises on failure."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise RuntimeError(f"CUDA library {LIB_PATH} is missing; run __graft_entry__.build()")
        _build.build()
    lib = C.CDLL(LIB_PATH)
    for name, (args, res) in EXPORTS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


class MrsphError(RuntimeError):
    pass


def check(rc: int, handle=None, what: str = "") -> None:
    if rc != 0:
        buf = C.create_string_buffer(1024)
        load().mrsph_last_error(handle, buf, 1024)
        raise MrsphError(f"{what} failed ({rc}): {buf.value.decode(errors='replace')}")
