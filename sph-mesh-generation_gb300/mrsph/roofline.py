"""Algorithmic (compulsory) HBM bytes of one relaxation step, per particle.

The figures follow the per-phase term list of the byte model the project is
measured against: each particle's own state is read and written once per
phase; neighbour gathers are cache traffic and are not counted (reusing them
on chip is the kernels' job).  3D FP32-split, per particle:

  advect + cell key      read x 16, v 16; write x 16, key 4, idx 4      =  56
  stable cell sort       read 8 + write 8                                =  16
  reorder state          read 32, write 32                               =  64
  level set + map        read x 16; write x 16, h 4, type 4, n 12        =  52
  density sum            read x 16, h 4, type 4; write sum 4             =  28
  stage 1 + reduction    read x 16, h 4, sum 4, type 4, n 12; write v 16 =  56
  stage 2 + reduction    read x 16, h 4, v 16, type 4, n 12; write v 16, nu 4 = 72
                                                                   total 344

plus 8 bytes per cell-list cell for the cell start table and 20 bytes per
unique level-set cell the map phase touches (phi, n, curvature: five FP32
fields; 40 in FP64).  FP64-plain uses 24-byte vectors and 8-byte scalars; 2D
uses D-component vectors.
"""
from __future__ import annotations


def per_particle_bytes(dim: int, precision: str) -> dict:
    """Bytes per particle of each timed phase (keys match mrsph._lib.TIMERS)."""
    if precision == "fp32":
        x = 16 if dim == 3 else 8      # position (anchor offset + key packed separately)
        s = 4                          # scalar
    else:
        x = 24 if dim == 3 else 16
        s = 8
    v = x
    nrm = 12 if (dim == 3 and precision == "fp32") else (3 * s if dim == 3 else 2 * s)
    t = 4                              # type / level word
    advect = x + v + x + 4 + 4
    lsmap = x + x + s + t + nrm
    return {
        "map": advect + lsmap,
        "scan": 0,                     # cell term, added per cell by step_bytes()
        "sort": 16,
        "reorder": 2 * (x + v),
        "density": x + s + t + s,
        "force1": x + s + s + t + nrm + v,
        "force2": x + s + v + t + nrm + v + s,
    }


def step_bytes(dim: int, precision: str, n_particles: int, n_cells: int) -> dict:
    """Algorithmic bytes of one step per phase for the whole workload."""
    pp = per_particle_bytes(dim, precision)
    out = {k: v * n_particles for k, v in pp.items()}
    out["scan"] = 8 * n_cells
    return out


def total_bytes_per_particle(dim: int, precision: str) -> int:
    return sum(per_particle_bytes(dim, precision).values())


def algorithmic_bytes(dim: int, precision: str, n_particles: int, n_lscells_touched: int,
                      n_cells: int = 0) -> int:
    """Compulsory bytes of one whole step: the per-particle terms of every
    phase, 20 bytes (40 in FP64) per unique level-set cell touched by the map
    phase, and 8 bytes per cell-list cell for the start table."""
    ls = 20 if precision == "fp32" else 40
    return total_bytes_per_particle(dim, precision) * n_particles + ls * n_lscells_touched + 8 * n_cells
