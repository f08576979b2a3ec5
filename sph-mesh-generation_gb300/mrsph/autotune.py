"""Autotuner of the neighbour passes' tile shapes and per-block work splits.

The FP32 density and force kernels take their shared-memory tile criterion
(MRSPH_TILE_SPAN_X / _YZ: the largest spread of a warp's half cells for which
it scans through shared-memory tiles), the unroll of the tile loop
(MRSPH_TILE_UNROLL) and their resident blocks per SM, i.e. registers per
thread and work per SM (MRSPH_DENSITY_MIN_BLOCKS, MRSPH_FORCE_MIN_BLOCKS,
MRSPH_FORCE2_MIN_BLOCKS, MRSPH_MAP_MIN_BLOCKS), as compile-time macros; the
persistent batch kernel its resident blocks per SM (MRSPH_BATCH_MIN_BLOCKS)
and the items a block claims at a time from a phase's work queue
(MRSPH_BATCH_CHUNK), tuned on a batch workload (--workload star_batch_512).  This
tuner builds candidate settings side by side (one build directory each),
times each on a workload in a fresh process (device-timed steps after a
warm-up, mrsph_step_timed), searches coordinate by coordinate from the
current defaults, and writes the best setting to mrsph/tuned.json, which
mrsph/build.py then compiles in.

    python -m mrsph.autotune --workload torus_3d --steps 200
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
from typing import Callable, Dict, List, Sequence

from . import build as _build

# the engine's defaults (csrc/engine.cuh) and the values tried per macro
DEFAULTS: Dict[str, int] = {"DENSITY_MIN_BLOCKS": 6, "FORCE_MIN_BLOCKS": 5, "FORCE2_MIN_BLOCKS": 6,
                            "MAP_MIN_BLOCKS": 4, "TILE_UNROLL": 1, "TILE_SPAN_X": 3, "TILE_SPAN_YZ": 1}
BATCH_DEFAULTS: Dict[str, int] = {"BATCH_MIN_BLOCKS": 4, "BATCH_CHUNK": 2}
BATCH_SPACE: Dict[str, List[int]] = {"BATCH_MIN_BLOCKS": [2, 3, 4, 5, 6], "BATCH_CHUNK": [1, 2, 4, 8]}
SPACE: Dict[str, List[int]] = {"DENSITY_MIN_BLOCKS": [4, 5, 6], "FORCE_MIN_BLOCKS": [4, 5, 6],
                               "FORCE2_MIN_BLOCKS": [5, 6, 8], "MAP_MIN_BLOCKS": [3, 4],
                               "TILE_UNROLL": [1, 4], "TILE_SPAN_X": [3, 5, 7], "TILE_SPAN_YZ": [0, 1, 2]}

WORKLOADS = {
    "torus_3d": "cases.torus_3d(precision='fp32')",
    "torus_3d_small": "cases.torus_3d(dx_min=0.01, dx_max=0.04, precision='fp32')",
    "spheres_3d": "cases.spheres_3d(precision='fp32')",
    "ellipses_2d": "cases.ellipses_2d(precision='fp32')",
    "disc_hole_2d": "cases.disc_hole_2d(precision='fp32')",
}

# batch workloads: the persistent batch kernel over star-shaped geometries
BATCH_WORKLOADS = {"star_batch_512": 512, "star_batch_64": 64}

_BATCH_TIMER = r"""
import json
from mrsph import BatchRelaxation, SPHMeshGeneration, cases
if __name__ == "__main__":
    geoms = cases.star_batch({count}, workers=8)
    hs = [SPHMeshGeneration(c, precision='fp32') for c in geoms]
    for h in hs:
        h.Initialize_case()
    b = BatchRelaxation(hs, mode='persistent')
    b.SPH_run_mesh_generation({warmup})
    ms = b.step_timed({steps})
    print(json.dumps({{"ms_per_step": ms / {steps}, "n": sum(h.n for h in hs)}}))
"""

_TIMER = r"""
import json, sys
from mrsph import SPHMeshGeneration, cases
case = {case}
g = SPHMeshGeneration(case, precision='fp32')
g.Initialize_case()
g.SPH_run_mesh_generation({warmup})
ms = g.step_timed({steps})
print(json.dumps({{"ms_per_step": ms / {steps}, "n": g.n}}))
"""


def defines_of(setting: Dict[str, int]) -> List[str]:
    return ["-DMRSPH_%s=%d" % (k, v) for k, v in sorted(setting.items())]


def time_setting(setting: Dict[str, int], workload: str, steps: int, warmup: int, workdir: str) -> float:
    """Build one candidate into its own directory and time it in a fresh process."""
    tag = "_".join("%s%d" % (k[:3], v) for k, v in sorted(setting.items()))
    bdir = os.path.join(workdir, tag)
    lib = os.path.join(bdir, "libmrsph_relax.so")
    _build.build(defines=defines_of(setting), build_dir=bdir, lib_path=lib)
    if workload in BATCH_WORKLOADS:
        code = _BATCH_TIMER.format(count=BATCH_WORKLOADS[workload], warmup=warmup, steps=steps)
    else:
        code = _TIMER.format(case=WORKLOADS[workload], warmup=warmup, steps=steps)
    env = dict(os.environ, MRSPH_LIB=lib, PYTHONPATH=_build.ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    script = os.path.join(bdir, "time_candidate.py")  # a file, so spawned workers can import __main__
    with open(script, "w") as f:
        f.write(code)
    r = subprocess.run([sys.executable, script], capture_output=True, text=True, env=env, timeout=1800)
    if r.returncode != 0:
        raise RuntimeError(f"candidate {tag} failed:\n{r.stderr[-2000:]}")
    return float(json.loads(r.stdout.strip().splitlines()[-1])["ms_per_step"])


def coordinate_search(timer: Callable[[Dict[str, int]], float], start: Dict[str, int],
                      space: Dict[str, Sequence[int]], rounds: int = 1, log=print):
    """Coordinate descent: for each macro in turn, try its values with the
    others fixed and keep the fastest; repeat for `rounds` passes.  Returns
    (best setting, its time, every (setting, time) tried)."""
    best = dict(start)
    cache: Dict[tuple, float] = {}

    def t(s):
        key = tuple(sorted(s.items()))
        if key not in cache:
            cache[key] = timer(s)
            log(f"{dict(key)}: {cache[key]:.4f} ms/step")
        return cache[key]

    best_t = t(best)
    for _ in range(rounds):
        for name, values in space.items():
            for v in values:
                if v == best.get(name):
                    continue
                cand = dict(best, **{name: v})
                ct = t(cand)
                if ct < best_t:
                    best, best_t = cand, ct
    return best, best_t, [(dict(k), v) for k, v in cache.items()]


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--workload", default="torus_3d_small", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS))
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--rounds", type=int, default=1)
    ap.add_argument("--only", default="", help="comma-separated macros to tune (default: all)")
    ap.add_argument("--out", default=_build.TUNED)
    args = ap.parse_args(argv)
    batch = args.workload in BATCH_WORKLOADS
    full_space, start = (BATCH_SPACE, BATCH_DEFAULTS) if batch else (SPACE, DEFAULTS)
    space = {k: v for k, v in full_space.items() if not args.only or k in args.only.split(",")}
    if os.path.exists(args.out):  # keep the other search's macros of an earlier run
        with open(args.out) as f:
            prev = json.load(f).get("defines", {})
        start = dict(start, **{k: v for k, v in prev.items() if k in start})
    with tempfile.TemporaryDirectory(prefix="mrsph_tune_") as wd:
        best, best_t, tried = coordinate_search(
            lambda s: time_setting(s, args.workload, args.steps, args.warmup, wd), start, space, args.rounds)
    if os.path.exists(args.out):
        with open(args.out) as f:
            prev = json.load(f).get("defines", {})
        best = dict({k: v for k, v in prev.items() if k not in best}, **best)
    res = {"defines": best, "ms_per_step": best_t, "workload": args.workload, "steps": args.steps,
           "tried": [{"defines": s, "ms_per_step": v} for s, v in tried]}
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({"best": best, "ms_per_step": best_t, "out": args.out}))


if __name__ == "__main__":
    main()
