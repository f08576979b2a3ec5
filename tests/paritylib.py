"""Shared helpers of the parity tests: run the FP64 oracle and the CUDA engine
from identical states and compare phase by phase."""
from __future__ import annotations

import numpy as np

import oracle
from mrsph import SPHMeshGeneration, cases
from mrsph import _lib as L


def small_cases():
    """Parity-sized variants of the benchmark geometries (seconds on the oracle)."""
    return {
        "disc2d_wendland": lambda: cases.disc_hole_2d(spacing=0.02, grid=64, kernel="wendland"),
        "disc2d_hyperbolic": lambda: cases.disc_hole_2d(spacing=0.02, grid=64, kernel="hyperbolic",
                                                        h_over_dx=1.0),
        "torus3d_adaptive": lambda: cases.torus_3d(dx_min=0.03, dx_max=0.09, fine_pkg=32, nlevels=2),
        "spheres3d_curvature": lambda: cases.spheres_3d(fine_pkg=16, nlevels=2, dx_min=0.015, middle_dl=0.035,
                                                        dx_max=0.09),
    }


def oracle_state_to_gpu(st: dict) -> dict:
    xyz = np.stack([st["x"], st["y"], st["z"]], axis=1)
    v = np.stack([st["vx"], st["vy"], st["vz"]], axis=1)
    return {"xyz": xyz, "v": v, "type": st["type"], "h": st["h"], "level": st["level"], "nu": st["nu"],
            "dt": st["dt"], "step": st["step"]}


def warm_oracle(case, max_steps: int = 40, need_surface: bool = True):
    """Seed with the oracle and relax until surface particles exist."""
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    for _ in range(max_steps):
        orc.steps(1)
        if not need_surface or (orc.arrays["type"] == 1).any():
            break
    return orc


def gpu_post_map_to_oracle(orc: oracle.Oracle, gp: dict, st_in: dict):
    """Load the GPU's post-map state into the oracle (positions, types,
    spacing, levels, level-set samples; viscosity from the injected state)."""
    n = len(gp["xyz"])
    st = {"x": gp["xyz"][:, 0], "y": gp["xyz"][:, 1], "z": gp["xyz"][:, 2],
          "type": gp["type"], "h": gp["h"], "level": gp["level"], "phi": gp["phi"], "curv": gp["curv"],
          "nx": gp["norm"][:, 0], "ny": gp["norm"][:, 1], "nz": gp["norm"][:, 2], "rho": gp["rho"],
          "nu": st_in["nu"], "id": np.arange(n, dtype=np.int32), "step": st_in["step"] + 1}
    st["vol"] = 1.0 / gp["rho"]
    st["scale"] = orc.ctx.max_scale * np.ldexp(1.0, -np.asarray(gp["level"], dtype=np.int64))
    orc.set_state(st)


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = max(float(np.max(np.abs(b))) if b.size else 0.0, floor)
    if scale == 0.0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0
    return float(np.max(np.abs(a - b)) / scale) if a.size else 0.0


def neighbor_sets(off, nb):
    return [set(nb[off[i]:off[i + 1]].tolist()) for i in range(len(off) - 1)]


def make_gpu(case, precision, cap=0):
    if cap == 0:
        cap = 64 if case.params["dim"] == 2 else 2048  # taps need unspilled lists
    return SPHMeshGeneration(case, precision=precision, neighbor_cap=cap)


PHASES = L
