#!/usr/bin/env python3
"""Benchmark: adaptive SPH particle relaxation on one GB300.

Workload (default): the inside of a torus (R = 1, r = 0.35) on three nested
level-set grids, spacing 0.005..0.02 by the tanh law, ~1.0M particles,
Wendland C2, h = 1.3 dx, FP32-split positions; synthetic and seeded (Philox,
seed 0).  A step is one relaxation step (SPH_run_mesh_generation).

Prints one JSON line.  `value` = relaxed particle-steps/s of the FP32-split
path with the state resident in HBM (device-timed with CUDA events on the
engine's stream); `e2e` = the same metric through the C ABI with host buffers
(positions uploaded from pinned memory and downloaded every step); the FP64
plain path, pair-interactions/s, a per-phase roofline and the CPU oracle
(all host cores) are reported beside it.

--impl reference times the CPU implementation of the path (the FP64 oracle,
a restatement of the reference code; the reference itself does not build
here) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sph-mesh-generation_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "relaxed particle-steps/s & pair-interactions/s, batched FP32 vs FP64 plain"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mrsph", choices=["mrsph", "reference"])
    ap.add_argument("--workload", default="torus_3d")
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--e2e-steps", type=int, default=-1, help="-1: the same steps as the device-timed region")
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--cvp-vps", type=int, default=256)
    ap.add_argument("--cvp-iters", type=int, default=50)
    ap.add_argument("--batch-geoms", type=int, default=512, help="star-shaped geometries of the batched run (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--no-volume-mass", action="store_true", help="skip the cut-cell volume / particle-count leg")
    ap.add_argument("--accuracy-steps", type=int, default=100, help="relaxation steps of the accuracy leg (0: skip)")
    ap.add_argument("--ref-budget", type=float, default=60.0,
                    help="seconds of timed oracle steps in the reference arm (at least one step)")
    return ap.parse_args()


def workload(name: str, precision: str):
    from mrsph import cases
    if name == "torus_3d":
        return cases.torus_3d(precision=precision)
    if name == "disc_hole_2d":
        return cases.disc_hole_2d(precision=precision)
    if name == "torus_3d_small":
        return cases.torus_3d(dx_min=0.01, dx_max=0.04, precision=precision)
    if name == "ellipses_2d":
        return cases.ellipses_2d(precision=precision)
    if name == "spheres_3d":
        return cases.spheres_3d(precision=precision)
    if name == "spheres_3d_full":  # four nested level-set levels down to 512^3, about 6.2 M particles
        return cases.spheres_3d(fine_pkg=128, nlevels=4, dx_min=0.0015, middle_dl=0.0025, dx_max=0.012,
                                precision=precision)
    raise SystemExit(f"unknown workload {name}")


def config_of(case, name):
    p = case.params
    return {"workload": f"{name}: {case.name}, N={case.n_particles}", "n_particles": case.n_particles,
            "dim": p["dim"], "kernel": "wendland_c2" if p["kernel"] == 2 else p["kernel"],
            "h_over_dx": p["cell_ratio"] / p["cutoff"], "dx_range": [p["min_dl"], p["max_dl"]],
            "levelset_levels": len(case.levels),
            "levelset_cells": [int(lv.phi.size) for lv in case.levels],
            "l2": "working set (state + neighbour lists) larger than the 129 MB L2",
            "parallelism": "replicas"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int):
        self.lines = []
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={dev}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.t.join(timeout=2)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
                pw.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[4 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(sm), "reasons": sorted(reasons)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_summary(kernel: str, precision: str, dim: int) -> dict:
    """A kernel's entry of the committed ncu summary (DRAM bytes per particle,
    issue and FP32-pipe fractions), or {}."""
    try:
        with open(os.path.join(ROOT, "profiles", "ncu_traffic.json")) as f:
            d = json.load(f)
        return d[f"{precision}_{dim}d"][kernel]
    except Exception:
        return {}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        return ws, rank, local, dist
    return 1, 0, 0, None


def max_over_ranks(x: float, dist) -> float:
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_oracle_run(case, steps: int):
    """Time the FP64 oracle (OpenMP, all host threads, host-CPU tuned build)
    on the workload."""
    os.environ["MRSPH_ORACLE_TUNED"] = "1"
    import oracle
    orc = oracle.Oracle(case)
    t0 = time.perf_counter()
    orc.seed(case.n_particles)
    orc.pre_run()
    orc.steps(1)  # the sample starts at step 2, as the GPU window does
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    pairs = orc.steps(steps)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "steps": steps, "pairs": pairs, "setup_s": setup, "threads": oracle.num_threads()}


def cpu_volume_mass(case):
    """Time the oracle's cut-cell volume pass (OpenMP, all host threads) on
    the finest level of the workload."""
    os.environ["MRSPH_ORACLE_TUNED"] = "1"
    import oracle
    t0 = time.perf_counter()
    orc = oracle.Oracle(case)  # level-set build of every level (normals, tags, curvature, max phi)
    ls_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = orc.volume_mass(-1)
    return {"seconds": time.perf_counter() - t0, "threads": oracle.num_threads(), "result": r, "levelset_s": ls_s}


def run_reference(args, ws, rank, dist):
    """The reference arm: the CPU implementation of the path (the FP64 oracle
    restating the reference; the reference itself does not build here), on
    the same workload and over the same step window as the GPU arm: seeding
    and pre-run, the GPU arm's warm-up steps untimed, then the window's steps
    timed one by one until about --ref-budget seconds are spent (at least
    one).  The line reports the steps it timed and their window."""
    if rank != 0:
        return
    case = workload(args.workload, "fp32")
    cfg = config_of(case, args.workload)
    warm = max(args.warmup, 3)
    os.environ["MRSPH_ORACLE_TUNED"] = "1"
    import oracle
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    orc.steps(warm)
    t0 = time.perf_counter()
    done, pairs = 0, 0
    while done < args.steps:
        pairs += orc.steps(1)
        done += 1
        if time.perf_counter() - t0 > args.ref_budget:
            break
    dt = time.perf_counter() - t0
    v = case.n_particles * done / dt
    threads = oracle.num_threads()
    window = f"steps {warm + 1}..{warm + done} after seeding"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": done, "warmup": args.warmup, "window": window, "ms_per_step": 1000.0 * dt / done,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "pair_interactions_per_s": 3.0 * pairs / dt,
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": f"{done} relaxation step(s) ({window}; the GPU arm times steps "
                                       f"{warm + 1}..{warm + args.steps}) of the full workload "
                                       f"(N={case.n_particles}), FP64 oracle restating the reference, "
                                       f"OpenMP on {threads} threads, -O3 {' '.join(oracle.tuning_flags())}"},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_batched(args, dev, dist, geoms=None):
    """Many independent star-shaped 2D/3D geometries relaxed together, in the
    three batch modes: the persistent batch kernel (one cooperative launch
    runs up to 32 whole steps of every geometry; the default), the per-phase
    batch kernels (one launch per phase over every geometry's blocks) and each
    handle's own step graph on its own stream; against stepping the
    geometries one at a time in FP32 and in FP64.  All are timed on steps 2-4
    after seeding; the persistent batch also on the batch_steps steps that
    follow."""
    from mrsph import BatchRelaxation, SPHMeshGeneration, cases
    gen_s = 0.0
    if geoms is None:
        t0 = time.perf_counter()
        geoms = cases.star_batch(args.batch_geoms)
        gen_s = time.perf_counter() - t0
    ntot = sum(c.n_particles for c in geoms)
    rate = lambda steps, ms: ntot * steps / (ms / 1000.0)
    modes = {}
    flags = 0
    graph = None
    ms_long = None
    for mode in ("persistent", "phases", "streams"):
        hs = [SPHMeshGeneration(c, precision="fp32", device=dev) for c in geoms]
        for h in hs:
            h.Initialize_case()
        b = BatchRelaxation(hs, mode=mode)
        b.SPH_run_mesh_generation(1)
        b.sync()
        barrier(dist)
        modes[mode] = max_over_ranks(b.step_timed(3), dist)
        if mode == "persistent":
            ms_long = max_over_ranks(b.step_timed(args.batch_steps), dist)
            graph = b.graph_captured
        for h in hs:
            flags |= h.stats()["flags"]
        b.close()
        for h in hs:
            h.close()
    seq = {}
    for prec in ("fp32", "fp64"):
        tot = 0.0
        for c in geoms:
            g = SPHMeshGeneration(c, precision=prec, device=dev)
            g.Initialize_case()
            g.SPH_run_mesh_generation(1)
            g.sync()
            tot += g.step_timed(3)
            g.close()
        seq[prec] = max_over_ranks(tot, dist)
    ms_win = modes["persistent"]
    return {"geometries": len(geoms), "particles": ntot,
            "n_range": [min(c.n_particles for c in geoms), max(c.n_particles for c in geoms)],
            "value": rate(args.batch_steps, ms_long), "unit": "particle-steps/s",
            "ms_per_step": ms_long / args.batch_steps, "mode": "persistent",
            "launch": "one cooperative launch of the persistent batch kernel per 32 steps"
                      + (", replayed from a CUDA graph" if graph else ""),
            "steps": args.batch_steps, "window": "steps 5..%d after seeding" % (4 + args.batch_steps),
            "steps_2_4": {"persistent_fp32": rate(3, ms_win), "phases_fp32": rate(3, modes["phases"]),
                          "streams_fp32": rate(3, modes["streams"]),
                          "one_at_a_time_fp32": rate(3, seq["fp32"]), "one_at_a_time_fp64": rate(3, seq["fp64"]),
                          "ms_per_step": {"persistent": ms_win / 3, "phases": modes["phases"] / 3,
                                          "streams": modes["streams"] / 3, "one_at_a_time_fp32": seq["fp32"] / 3,
                                          "one_at_a_time_fp64": seq["fp64"] / 3}},
            "batched_fp32_over_fp64_plain": seq["fp64"] / ms_win,
            "batched_over_one_at_a_time_fp32": seq["fp32"] / ms_win,
            "persistent_over_streams": modes["streams"] / ms_win,
            "generation_s": gen_s, "device_flags": flags,
            "workload": "star-shaped bodies, 8-32 radial harmonics, sum of amplitudes <= 0.3, even ids 2D "
                        "(128^2 level set) and odd 3D (64^3), counts log-uniform 2k-200k, constant spacing, "
                        "Wendland C2, h = 1.3 dx, FP32-split"}


def spacing_stats(xyz, h, h_over_dx, dim, type_=None, phi=None):
    """Nearest-neighbour distance over the target spacing (h / (h/dx)), its
    percentiles and 40-bin histogram, the minimum pair distance, and the
    SURFACE particles' count and mean |phi| over their target spacing."""
    import numpy as np
    from scipy.spatial import cKDTree
    pts = xyz[:, :dim]
    d, _ = cKDTree(pts).query(pts, k=2)
    r = d[:, 1] / (h / h_over_dx)
    hist, _ = np.histogram(r, bins=40, range=(0.0, 2.0))
    out = {"median": float(np.median(r)), "p05": float(np.percentile(r, 5)), "p95": float(np.percentile(r, 95)),
           "min_ratio": float(r.min()), "min_distance": float(d[:, 1].min()), "hist": hist.tolist()}
    if type_ is not None:
        surf = type_ == 1
        dev_s = np.abs(phi[surf]) / (h[surf] / h_over_dx) if surf.any() else np.zeros(1)
        out.update(surface_count=int(surf.sum()), surface_dev_mean=float(dev_s.mean()),
                   surface_dev_max=float(dev_s.max()))
    return out


def run_accuracy(args, dev):
    """FP32-split against the FP64 oracle (the CPU restatement of the
    reference) on a 37,658-particle torus (dx 0.02-0.08): the oracle relaxes
    accuracy_steps steps from its seed; the GPU's FP32 path relaxes the same
    steps from the same seed state; and, from the oracle's state after those
    steps (with SURFACE particles), the GPU makes one step whose binning,
    neighbour sets, kernel sums (REAL and SURFACE) and force stages are
    compared with the oracle's on the GPU's post-map state."""
    import numpy as np
    import oracle
    from mrsph import SPHMeshGeneration, cases
    case = cases.torus_3d(dx_min=0.02, dx_max=0.08)
    dim = case.params["dim"]
    hdx = case.params["cell_ratio"] / case.params["cutoff"]
    orc = oracle.Oracle(case)
    orc.seed(case.n_particles)
    orc.pre_run()
    seed_st = orc.get_state()

    def to_gpu(st):
        return {"xyz": np.stack([st["x"], st["y"], st["z"]], axis=1),
                "v": np.stack([st["vx"], st["vy"], st["vz"]], axis=1), "type": st["type"], "h": st["h"],
                "level": st["level"], "nu": st["nu"], "dt": st["dt"], "step": st["step"]}

    t0 = time.perf_counter()
    orc.steps(args.accuracy_steps)
    st_acc = orc.get_state()
    oracle_s = time.perf_counter() - t0
    # one step from the oracle's state after accuracy_steps steps
    g = SPHMeshGeneration(case, precision="fp32", device=dev, neighbor_cap=1024)
    g.set_state(to_gpu(st_acc))
    g.run_phase(5)
    gp = g.particles()
    lc, _ = g.cells()
    off, nb = g.neighbors()
    g.close()
    o2 = oracle.Oracle(case)
    n = len(gp["xyz"])
    o2.set_state({"x": gp["xyz"][:, 0], "y": gp["xyz"][:, 1], "z": gp["xyz"][:, 2], "type": gp["type"],
                  "h": gp["h"], "level": gp["level"], "phi": gp["phi"], "curv": gp["curv"],
                  "nx": gp["norm"][:, 0], "ny": gp["norm"][:, 1], "nz": gp["norm"][:, 2], "rho": gp["rho"],
                  "nu": st_acc["nu"], "id": np.arange(n, dtype=np.int32), "step": st_acc["step"] + 1,
                  "vol": 1.0 / gp["rho"],
                  "scale": o2.ctx.max_scale * np.ldexp(1.0, -np.asarray(gp["level"], dtype=np.int64))})
    ooff, onb = o2.neighbors()

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
    o2.density(ooff, onb)
    s0 = o2.get_state()
    o2.force(ooff, onb, 1)
    s1 = o2.get_state()
    o2.force(ooff, onb, 2)
    s2 = o2.get_state()
    surf = gp["type"] == 1
    force = {"cells_equal": bool(np.array_equal(lc, o2.cells())),
             "neighbour_sets_equal": bool(np.array_equal(off, ooff) and np.array_equal(nb, onb)),
             "sum_real_max_rel": rel(gp["sum"][~surf], s0["sum"][~surf]),
             "sum_surface_max_rel": rel(gp["sum"][surf], s0["sum"][surf]) if surf.any() else None,
             "stage1_max_rel": rel(gp["a1"], np.stack([s1["ax"], s1["ay"], s1["az"]], 1)),
             "stage2_max_rel": rel(gp["a2"], np.stack([s2["ax"], s2["ay"], s2["az"]], 1)),
             "surface_particles": int(surf.sum()),
             "normalisation": "max |gpu - oracle| / max |oracle| over the particles"}
    # relaxation statistics after accuracy_steps steps from the same seed state
    g = SPHMeshGeneration(case, precision="fp32", device=dev, neighbor_cap=1024)
    g.set_state(to_gpu(seed_st))
    g.SPH_run_mesh_generation(args.accuracy_steps)
    p = g.particles(("xyz", "h", "type", "phi"))
    g.close()
    os_ = orc.get_state()
    stats = {"fp32": spacing_stats(p["xyz"], p["h"], hdx, dim, p["type"], p["phi"]),
             "oracle": spacing_stats(np.stack([os_["x"], os_["y"], os_["z"]], 1), os_["h"], hdx, dim,
                                     os_["type"], os_["phi"])}
    dif = {k: abs(stats["fp32"][k] - stats["oracle"][k]) / max(abs(stats["oracle"][k]), 1e-300)
           for k in ("median", "p05", "p95", "min_distance", "surface_count", "surface_dev_mean")}
    dif["hist_l1_over_n"] = float(np.abs(np.array(stats["fp32"]["hist"]) -
                                         np.array(stats["oracle"]["hist"])).sum() / n)
    return {"workload": f"torus_3d dx 0.02-0.08 (N={case.n_particles})", "reference": "FP64 oracle",
            "single_step": force, "single_step_state": f"the oracle's state after {args.accuracy_steps} steps",
            "steps": args.accuracy_steps, "oracle_seconds": oracle_s,
            "spacing_ratio": {"fp32": {k: v for k, v in stats["fp32"].items() if k != "hist"},
                              "oracle": {k: v for k, v in stats["oracle"].items() if k != "hist"},
                              "hist_bins": "40 bins over [0, 2)", "hist_fp32": stats["fp32"]["hist"],
                              "hist_oracle": stats["oracle"]["hist"]},
            "fp32_vs_oracle_rel_diff": dif}


def run_mrsph(args, ws, rank, local, dist):
    import numpy as np
    from mrsph import SPHMeshGeneration
    from mrsph import build as mbuild
    from mrsph import cases as mcases
    from mrsph import roofline
    mbuild.build()
    # the batched leg's geometries, built in spawned processes before this
    # process touches the GPU
    t0 = time.perf_counter()
    batch_geoms = mcases.star_batch(args.batch_geoms, workers=min(16, os.cpu_count() or 1)) \
        if args.batch_geoms > 0 else None
    batch_gen_s = time.perf_counter() - t0
    dev = local
    case = workload(args.workload, "fp32")
    n = case.n_particles
    dim = case.params["dim"]
    warm = max(args.warmup, 3)
    gpu = SPHMeshGeneration(case, precision="fp32", device=dev)
    gpu.Initialize_case(n)
    gpu.SPH_run_mesh_generation(warm)
    gpu.sync()
    st0 = gpu.stats()
    gpu.sync()
    barrier(dist)
    clk = ClockSampler(dev)
    ms = gpu.step_timed(args.steps)
    clocks = clk.stop()
    barrier(dist)
    ms = max_over_ranks(ms, dist)
    st1 = gpu.stats()
    window = f"steps {warm + 1}..{warm + args.steps} after seeding"
    prof = gpu.profile_steps(3)  # per-phase device times of the three steps after the window
    pairs = st1["pairs_total"] - st0["pairs_total"]
    value = ws * n * args.steps / (ms / 1000.0)
    pair_rate = ws * 3.0 * pairs / (ms / 1000.0)
    ms_step = ms / args.steps

    # roofline of the dominant phase (device-timed per phase, eager launches)
    bytes_ = roofline.step_bytes(dim, "fp32", n, st1["num_cells"])
    top = max(prof, key=prof.get)
    peak, peak_kind = peaks()
    ach = bytes_[top] / (prof[top] / 1000.0) / 1e9
    step_ach = sum(bytes_.values()) / (ms_step / 1000.0) / 1e9
    ns = ncu_summary(top, "fp32", dim)
    tr = ns.get("dram_bytes_per_particle")
    roof = {"bound": "hbm", "kernel": top, "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind,
            "traffic": (tr * n if tr is not None else None),
            "issue": {"issue_active_frac": ns.get("issue_active_pct", 0.0) / 100.0 or None,
                      "fp32_fma_pipe_frac": ns.get("fma_pipe_pct", 0.0) / 100.0 or None,
                      "source": "ncu --set full of the same kernel on the 301,270-particle torus "
                                "(profiles/density_torus_3d_small.md): the kernel is issue-bound, so its "
                                "instruction-issue and FP32-pipe fractions bound it, not HBM"},
            "algorithmic_bytes_per_launch": bytes_[top],
            "step_achieved": step_ach, "step_frac": step_ach / peak,
            "step_bytes_per_particle": roofline.total_bytes_per_particle(dim, "fp32")}

    flags = st1["flags"]
    # CVP partition of the relaxed particles (256 cells, 50 Lloyd iterations)
    cvp = None
    if args.cvp_vps > 0:
        xyz_now = gpu.particles(("xyz",))["xyz"]
        rng = np.random.default_rng(0)
        vp0 = xyz_now[rng.choice(n, args.cvp_vps, replace=False)].copy()
        gpu.sync()
        t0 = time.perf_counter()
        _, labels, vmass, cres = gpu.Partitioning(vp0, max_iter=args.cvp_iters - 1)
        cvp_s = time.perf_counter() - t0
        cvp = {"num_vp": args.cvp_vps, "iterations": cres["iterations"], "seconds": cvp_s,
               "ms_per_iteration": 1000.0 * cvp_s / max(cres["iterations"], 1), "error_max": cres["error_max"],
               "points": n, "timer": "host wall clock around mrsph_cvp (FP64, bit-exact vs the oracle)"}
    # 2D: neighbour-graph triangulation of the relaxed particles
    tri = None
    if dim == 2:
        gpu.sync()
        t0 = time.perf_counter()
        tris, q = gpu.Reconstruct_tris()
        tri_s = time.perf_counter() - t0
        tri = {"seconds": tri_s, "timer": "host wall clock around mrsph_triangulate (incl. copies)",
               "triangles": int(q["ntri"]), "edges": int(q["nedge"]), "deleted_edges": int(q["ndeleted"]),
               "error_edges": int(q["nerror"]), "min_angle": q["min_angle"], "min_angle_avg": q["min_angle_avg"],
               "max_aspect": q["max_aspect"], "G_avg": q["G_avg"], "theta_30": q["theta_30"],
               "total_area": q["total_area"], "angle_hist_4deg": [int(v) for v in q["hist"]]}
    # cut-cell volume, surface area and particle count of the finest level
    # (Calculate_total_volume_mass + Get_num_particles), device-timed, and
    # the set-up of a fresh handle (level-set copy and build on the GPU)
    vm = None
    if not args.no_volume_mass:
        gpu.sync()
        t0 = time.perf_counter()
        g_setup = SPHMeshGeneration(case, precision="fp32", device=dev)
        setup_s = time.perf_counter() - t0
        g_setup.close()
        gpu.sync()
        t0 = time.perf_counter()
        r = gpu.volume_mass(-1)  # raises (with the engine's message) on a device error
        vm_wall = time.perf_counter() - t0
        vm = {k: r[k] for k in ("total_mass", "total_mass_surface", "total_volume", "total_area",
                                "num_interface_cell", "num_particle_mesh", "num_particle_surface", "num_particle")}
        vm.update(device_ms=r["device_ms"], wall_s=vm_wall, level_cells=int(case.levels[-1].phi.size),
                  handle_setup_s=setup_s, levelset_cells=int(sum(lv.phi.size for lv in case.levels)),
                  timer="CUDA events around the pass on the handle's stream; wall clock incl. scratch "
                        "allocation and copies; handle_setup_s: host wall clock of mrsph_create + "
                        "mrsph_set_levelset (phi copied in, every level built on the GPU)")
    gpu.close()

    # e2e through the C ABI with host buffers (pinned when torch is available):
    # a second handle seeded identically replays the untimed steps, then runs
    # the timed steps again with every step's positions uploaded from and
    # downloaded to host memory and the stats read back
    e2e_steps = args.steps if args.e2e_steps < 0 else args.e2e_steps
    try:
        import torch
        host_in = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        host_out = torch.empty((n, 3), dtype=torch.float64, pin_memory=True).numpy()
        pinned = True
    except Exception:
        host_in = np.empty((n, 3))
        host_out = np.empty((n, 3))
        pinned = False
    g2 = SPHMeshGeneration(case, precision="fp32", device=dev)
    g2.Initialize_case(n)
    g2.SPH_run_mesh_generation(warm)
    g2.download_positions(host_in)
    g2.sync()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        g2.upload_positions(host_in)
        g2.SPH_run_mesh_generation(1)
        g2.download_positions(host_out)
        s = g2.stats()
        host_in, host_out = host_out, host_in
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e = {"value": ws * n * e2e_steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": int(host_in.nbytes), "d2h_bytes_per_step": int(host_out.nbytes) + 96,
           "steps": e2e_steps, "pinned": pinned, "timer": "host wall clock, synchronised",
           "steps_replayed": "the device-timed steps, from an identically seeded state"}
    flags |= s["flags"]
    g2.close()
    # FP64-plain path on the same workload: the FP64 path is ~30x slower, so
    # both precisions are timed over the same short window (steps 2 to
    # 1 + fp64_steps after seeding, the densest steps), which is also the
    # window of the CPU sample
    fp64 = None
    if not args.no_fp64:
        win = {}
        for prec in ("fp32", "fp64"):
            g = SPHMeshGeneration(case, precision=prec, device=dev)
            g.Initialize_case(n)
            g.SPH_run_mesh_generation(1)
            g.sync()
            ms_w = max_over_ranks(g.step_timed(args.fp64_steps), dist)
            win[prec] = {"value": ws * n * args.fp64_steps / (ms_w / 1000.0), "ms_per_step": ms_w / args.fp64_steps}
            g.close()
        fp64 = {"value": win["fp64"]["value"], "unit": "particle-steps/s", "steps": args.fp64_steps,
                "ms_per_step": win["fp64"]["ms_per_step"], "window": f"steps 2..{1 + args.fp64_steps} after seeding",
                "fp32_same_window": win["fp32"]}

    batched = run_batched(args, dev, dist, batch_geoms) if args.batch_geoms > 0 else None
    if batched is not None:
        batched["generation_s"] = batch_gen_s
    accuracy = run_accuracy(args, dev) if (args.accuracy_steps > 0 and rank == 0) else None

    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        r = cpu_oracle_run(case, args.cpu_steps)
        cpu = {"value": n * r["steps"] / r["seconds"], "unit": "particle-steps/s", "cores": r["threads"],
               "kind": "port",
               "sample": f"{r['steps']} relaxation step(s) of the full workload (N={n}) from step 2 after "
                         f"seeding, FP64 oracle (restatement of the reference, OpenMP {r['threads']} threads)",
               "gpu_same_window": fp64["fp32_same_window"] if fp64 else None}
    if vm is not None and not args.no_cpu:
        r = cpu_volume_mass(case)  # the oracle (CPU), beside the device pass
        ref = r["result"]
        vm["cpu"] = {"seconds": r["seconds"], "threads": r["threads"], "kind": "port",
                     "num_particle": ref["num_particle"],
                     "counts_equal": all(ref[k] == vm[k] for k in ("num_interface_cell", "num_particle_mesh",
                                                                   "num_particle_surface")),
                     "total_mass_rel_diff": abs(ref["total_mass"] - vm["total_mass"]) / abs(ref["total_mass"]),
                     "levelset_build_s": r["levelset_s"]}
        vm["speedup_vs_cpu"] = r["seconds"] / (vm["device_ms"] / 1000.0)
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "window": window, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": config_of(case, args.workload),
            "pair_interactions_per_s": pair_rate, "pairs_per_particle": pairs / (n * args.steps),
            "fp64_plain": fp64,
            "fp32_over_fp64": (fp64["fp32_same_window"]["value"] / fp64["value"]) if fp64 else None,
            "phase_ms": prof, "cvp": cvp, "triangulation": tri, "volume_mass": vm, "batched": batched, "accuracy": accuracy, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": 12 * args.steps, "clocks": clocks, "device_flags": flags}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local, dist = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank, dist)
    else:
        run_mrsph(args, ws, rank, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
