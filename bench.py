#!/usr/bin/env python
"""Benchmark of the GB300 WCSPH hot path (one JSON line on rank 0).

Workload (default, ``--config c4``): the 3D dam break, H = 1, column
2H x H x H at dx = H/200 (16,000,000 fluid particles at dx (i+1, j+1, k+1))
in a 5.366H x 3H x (H + dx) tank with three layers of fixed wall particles,
Wendland C2 kernel (h = 1.3dx), Tait EOS (rho0 = 1000, xi = 7,
cs0 = 10 sqrt(gH)), hydrostatic start, Monaghan alpha = 0.02, delta-SPH
delta = 0.1, SSPRK3 at CFL 0.25.  A step is one full SSPRK3 step (three
neighbour rebuilds, three fused force passes).

* ``value``: FP32-compensated form, particle-updates/s = fluid particles x
  steps / device time, state resident in HBM (working set > L2), CUDA-graph
  replay, timed with CUDA events on the library's stream.
* ``forms.fp64``: the plain FP64 form on the same workload.
* ``l2_error_vs_fp64``: relative L2 error of rho, r and v (field-relative,
  and r also against the displacement from the start), the drift of total
  momentum (|sum m v32 - sum m v64| / sum m |v64|), FP32C against FP64
  after ``--err-steps`` (1000) steps from the same start, run outside the
  timed region on ``--err-config`` (for the 3D workloads the 3D dam break at
  dx = H/100, 2,000,000 fluid: 1000 plain-FP64 steps of the 16M workload
  would take eleven minutes).
* ``e2e``: the same metric through the C ABI with host buffers: every step
  uploads r, v, rho, dv/dt from pinned host memory, steps, and downloads
  them again (tg_particles_update / tg_step / tg_particles_download_state).
* ``roofline``: the fused force kernel (k_forces): algorithmic bytes per
  launch = fluid particles x 3S (S = state bytes per particle) over its mean
  launch time from a profiled pass with CUDA events on the same stream.
  The kernel is not HBM-bound; ``compute`` gives its FP32 work per launch
  (FLOPs per neighbour pair counted from the kernel source, pairs counted
  live) against the FP32 pipe and the recorded instruction count against
  the issue rate, and ``ncu_working_ceiling`` the recorded ncu capture's
  busiest unit.
* ``extra_workloads``: the 2D dam break at scale (c1), the 512 batched 2D
  tanks (c3) and 64 batched 3D tanks (c5), both forms, and c3's FP32C error
  after 500 steps.
* ``cpu_baseline``: the oracle (the C++ restatement of the reference's CPU
  path) on the host cores, on a bounded sample of the same workload.

Other workloads (``--config``): c0, c1, c3, c4q, c4half, c5 (2D / 3D /
batched dam breaks, the same report), c2 (point-cloud search + summation
density), f2 and f3 (the reference's face-wall mode: the titwcsph pool in
2D, a triangulated 3D pool; reference physics with shifting; device time
per step of each form: fp32c with FP64 face integrals, fp32c_face32 with
tg_params.face_fp32, fp64; each compensated form's drift from fp64; and the
oracle's rate on the same workload on the host cores).

``--impl reference`` times that CPU path alone on a sample of the same
workload (the reference itself needs C++26 / GCC 16 and cannot be built
here).  ``--gpus N`` under torch.distributed.run runs N independent replicas
(the path does not shard across GPUs) and reports their summed throughput
over the slowest rank.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "particle-updates/s: FP32-comp vs plain FP64 WCSPH, 1 GB300, at stated L2 error"
UNIT = "particle-updates/s"


def _peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def state_bytes(dim: int, form: str) -> int:
    """S: algorithmic state bytes per particle (positions, velocity, density)."""
    if form == "fp64":
        return 8 * (2 * dim + 1)
    return 8 * dim + 4 * dim + 4


def bytes_per_update(dim: int, form: str) -> int:
    """Algorithmic bytes per particle-update: 3 (3S + 8d + 16)."""
    return 3 * (3 * state_bytes(dim, form) + 8 * dim + 16)


def make_config(name: str):
    from titsolver_gb300 import scenarios

    if name == "c1":
        return ("2D dam break H=1, dx=H/800 (1,280,000 fluid + 3-layer walls), "
                "Wendland C2 h=2dx, Tait rho0=1000 xi=7 cs0=10sqrt(gH), alpha=0.02, "
                "delta-SPH 0.1, SSPRK3 CFL 0.25"), lambda: scenarios.dam_break_2d(nx_per_H=800)
    if name == "c2":
        return ("3D point cloud, 4,000,000 points in the unit box: 70% jittered lattice "
                "(+-0.25dx), 30% in 8 Gaussian clusters (sigma 0.05), seed 20261203; "
                "Wendland C2 h=1.3dx; neighbour search + summation density"), \
            lambda: scenarios.cloud_3d(n_total=4_000_000)
    if name == "c0":
        return ("2D dam break H=1, dx=H/80 (12,800 fluid + 3-layer walls), same physics"), \
            lambda: scenarios.dam_break_2d(nx_per_H=80)
    if name == "c3":
        return ("512 independent 2D dam breaks, column N~U{20..120} particles, aspect "
                "U[0.5,2], dx=1/80, same physics"), lambda: scenarios.batched_tanks(512)
    if name == "c4":
        return ("3D dam break 2Hx1Hx1H, dx=H/200 (16,000,000 fluid + 3-layer walls), "
                "Wendland C2 h=1.3dx, same physics"), lambda: scenarios.dam_break_3d(nx_per_H=200)
    if name == "c4q":
        return ("3D dam break 2Hx1Hx1H, dx=H/100 (2,000,000 fluid + 3-layer walls), "
                "Wendland C2 h=1.3dx, same physics"), lambda: scenarios.dam_break_3d(nx_per_H=100)
    if name == "c5":
        return ("64 independent 3D dam breaks, column height N~U{12..40} particles, "
                "length and depth U[0.5,2] N, dx=1/100, Wendland C2 h=1.3dx, same physics"), \
            lambda: scenarios.batched_tanks_3d(64)
    if name == "f2":
        return ("titwcsph 2D pool with the reference's face walls: H=0.6, column 2HxH at "
                "dx=H/80 (12,800 fluid), pool 5.366Hx4H tessellated at dx (one fixed "
                "particle per vertex), Wendland C4 h=2dx, cs0=20sqrt(gH), Ferrari + Morris "
                "mu=0.001, SSPRK3 CFL 0.4, shifting"), \
            lambda: scenarios.dam_break_2d_faces(nx_per_H=80)
    if name == "f3":
        return ("3D pool with triangle face walls: column 2HxHxH at dx=H/20 (16,000 fluid), "
                "pool 3Hx1.5Hx(H+dx) triangulated at dx (7,382 vertices, 14,760 triangles), "
                "box containment, Wendland C4 h=1.3dx, reference physics, shifting"), \
            lambda: scenarios.dam_break_3d_faces(nx_per_H=20, tank=(3.0, 1.5))
    if name == "c4half":
        return ("3D dam break 2Hx1HxH/2, dx=H/200 (8,000,000 fluid + 3-layer walls), "
                "Wendland C2 h=1.3dx, same physics"), \
            lambda: scenarios.dam_break_3d(nx_per_H=200, column=(2.0, 1.0, 0.5))
    raise SystemExit(f"unknown config {name}")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.tmp = None

    def start(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.device)],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4:]))
                except ValueError:
                    continue
        os.unlink(self.tmp.name)
        if not rows:
            return None
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[3][1:]) if v == "Active"})
        loaded = [r for r in rows if r[2] > 200.0] or rows
        return {"sm_mhz": statistics.median(r[0] for r in loaded),
                "sm_max_mhz": max(r[1] for r in rows),
                "power_w_max": max(r[2] for r in rows),
                "samples": len(rows), "reasons": reasons}


def _forces_profile(dim: int, form: str) -> dict | None:
    p = ROOT / "profiles" / "forces_traffic.json"
    if not p.exists():
        return None
    return json.loads(p.read_text()).get(f"{form}_{dim}d")


def forces_traffic(dim: int, form: str, n_fluid: int):
    d = _forces_profile(dim, form)
    return None if d is None else float(d["dram_bytes_per_fluid_particle"]) * n_fluid


def forces_traffic_source(dim: int, form: str) -> str | None:
    d = _forces_profile(dim, form)
    if d is None:
        return None
    return (f"recorded, not measured in this run: DRAM bytes per fluid particle of one ncu "
            f"capture of {d['kernel']} ({d['source']}) x the fluid count")


# FP32 floating-point operations of the compensated force pass, counted from
# the kernel source (fluid.cuh, PairF32::add with the textbook terms:
# Wendland C2, delta-SPH diffusion, Monaghan viscosity; an FMA counts 2, a
# reciprocal square root or reciprocal 1).  Per accepted pair: rsqrt 1,
# r and q 2, kernel gradient factor 6, v_ab . r_ab 3d - 1, density
# difference 1, diffusion 3, continuity term 2, Monaghan term 9, momentum
# coefficient 4, sums 1 + 2d.  Per candidate: r_ab d (plus the 3D row
# shift 2) and |r_ab|^2 2d - 1.
FLOPS_PER_PAIR = {2: 38, 3: 43}
FLOPS_PER_CANDIDATE = {2: 5, 3: 10}
SM_COUNT = 152
FP32_LANES_PER_SM = 128
ISSUE_PER_SM_CLK = 4


def forces_compute(dim: int, n_fluid: int, pairs: int, avg_ms: float,
                   clk: dict | None, cells_per_radius: int | None = None) -> dict:
    """Compute-side roofline of the compensated force pass: FP32 work per
    launch (pairs counted live in this run, the per-pair FLOPs from the
    source) against the FP32 pipe's nominal rate at the sampled SM clock,
    and the recorded ncu instruction count (per fluid particle, captured at
    the cell size the record names; this run's cell size beside it) against
    the issue rate."""
    mhz = float(clk["sm_mhz"]) if clk and clk.get("sm_mhz") else 2070.0
    sec = avg_ms / 1e3
    flops = pairs * FLOPS_PER_PAIR[dim]
    fp32_peak = SM_COUNT * FP32_LANES_PER_SM * 2 * mhz * 1e6
    out = {"pairs_per_launch": pairs, "pairs_per_fluid_particle": pairs / max(n_fluid, 1),
           "flops_per_pair": FLOPS_PER_PAIR[dim],
           "flops_per_candidate": FLOPS_PER_CANDIDATE[dim],
           "pair_flops_per_launch": flops,
           "fp32_tflops": flops / sec / 1e12,
           "fp32_peak_tflops": fp32_peak / 1e12,
           "fp32_frac": flops / sec / fp32_peak,
           "fp32_peak_source": (f"nominal: {SM_COUNT} SMs x {FP32_LANES_PER_SM} FP32 lanes x "
                                f"2 (FMA) x {mhz:.0f} MHz (median SM clock of this run)")}
    d = _forces_profile(dim, "fp32c")
    if d is not None and "warp_inst_per_fluid_particle" in d:
        inst = d["warp_inst_per_fluid_particle"] * n_fluid
        issue_peak = SM_COUNT * ISSUE_PER_SM_CLK * mhz * 1e6
        rec = d.get("cells_per_radius")
        at = f" at {rec} cells per radius" if rec else ""
        run = f" (this run: {cells_per_radius})" if cells_per_radius else ""
        out.update({"warp_inst_per_launch": inst,
                    "thread_inst_per_pair": 32.0 * inst / max(pairs, 1),
                    "issue_frac": inst / sec / issue_peak,
                    "inst_source": (f"recorded: smsp__inst_executed.sum of {d['source']}{at}"
                                    f"{run}, scaled by the fluid count")})
    return out


def forces_ceiling(dim: int, form: str) -> dict | None:
    """The unit that bounds k_forces in its ncu capture (issue slots for the
    compensated form, the FP64 pipe for the plain one) and how busy it was:
    a recorded capture, beside the live HBM fraction."""
    d = _forces_profile(dim, form)
    if d is None or "working_ceiling" not in d:
        return None
    return {**d["working_ceiling"], "source": d["source"]}


def sample_scenario(dim: int, nx: int, cfg: str | None = None):
    """A dam break of the workload's dimension at resolution dx = H/nx (the
    2D and 3D workloads' own geometry and physics at a coarser lattice)."""
    from titsolver_gb300 import scenarios

    if cfg == "c4half":
        return scenarios.dam_break_3d(nx_per_H=nx, column=(2.0, 1.0, 0.5))
    if dim == 3:
        return scenarios.dam_break_3d(nx_per_H=nx)
    return scenarios.dam_break_2d(nx_per_H=nx)


def cpu_sample(budget_s: float, steps: int, threads: int, dim: int = 2,
               workload: dict | None = None, warmup: int = 0,
               cfg: str | None = None) -> dict:
    """Time the oracle (CPU restatement of the reference path) on a dam
    break of the workload's dimension sized so that warmup + steps steps take
    about budget_s seconds; the warm-up steps run untimed.  A one-tank
    workload without faces that is no larger than that size is timed itself
    (nx_per_H = 0 in the result).  One step at a small calibration size
    gives the host time per particle (fluid and walls), which picks the
    size."""
    import oracle
    from titsolver_gb300 import physics

    P = physics.baseline_params(dim)
    nx_cal, nx_max = (40, 800) if dim == 2 else (16, 200)
    cal = sample_scenario(dim, nx_cal, cfg)
    st = oracle.State(cal)
    oracle.step(P, st, 1, nthreads=threads)  # thread pool start-up
    t0 = time.perf_counter()
    oracle.step(P, st, 1, nthreads=threads)
    per_particle = max(time.perf_counter() - t0, 1e-6) / cal["r"].shape[0]
    want = budget_s / max(steps + warmup, 1) / per_particle  # particles per sample
    scale = (want / cal["r"].shape[0]) ** (1.0 / dim)
    nx = int(max(nx_cal, min(nx_max, nx_cal * scale)))
    scn = sample_scenario(dim, nx, cfg)
    if (workload is not None and workload["dim"] == dim and len(workload["tanks"]) == 1
            and not any(workload.get("faces") or [])
            and workload["r"].shape[0] <= scn["r"].shape[0]):
        scn, nx = workload, 0
    st = oracle.State(scn)
    nf = scn["tanks"][0]["n_fluid"]
    if warmup:
        oracle.step(P, st, warmup, nthreads=threads)
    t0 = time.perf_counter()
    oracle.step(P, st, steps, nthreads=threads)
    sec = time.perf_counter() - t0
    return {"value": nf * steps / sec, "seconds": sec, "fluid": nf,
            "walls": scn["tanks"][0]["n_wall"], "nx_per_H": nx, "steps": steps,
            "warmup": warmup, "threads": threads}


def sample_text(res: dict, dim: int) -> str:
    what = (f"the workload itself ({res['fluid']} fluid)" if res["nx_per_H"] == 0 else
            f"{dim}D dam break of the same geometry at dx=H/{res['nx_per_H']} "
            f"({res['fluid']} fluid, {res['walls']} walls)")
    return (f"{what}, same physics, {res['warmup']} untimed + {res['steps']} timed SSPRK3 "
            f"steps ({res['seconds']:.1f} s), oracle built g++ -O3 -ffp-contract=off")


def describe(scn: dict, workload: str) -> dict:
    """The workload part of the bench line's config: the same dictionary in
    both arms."""
    from titsolver_gb300 import scenarios

    nf = scenarios.n_fluid(scn)
    nw = int(sum(t["n_wall"] for t in scn["tanks"]))
    ws = scn["r"].shape[0] * (200 if scn["dim"] == 2 else 270)
    l2 = (f"inputs larger than L2 (working set ~{ws / 1e6:.0f} MB > 129 MB)" if ws > 129e6 else
          f"inputs smaller than L2 (working set ~{ws / 1e6:.0f} MB < 129 MB): L2-resident")
    return {"workload": workload, "fluid_particles": nf, "wall_particles": nw,
            "tanks": len(scn["tanks"]), "parallelism": "replicas (no exchange between GPUs)",
            "l2": l2}


def run_reference(args, ranks) -> dict:
    import oracle

    threads = oracle.default_threads()
    workload, make = make_config(args.config)
    scn = make()
    dim = scn["dim"]
    # Each timed step is one SSPRK3 step of a dam break of the workload's
    # dimension sized so that the warm-up and timed steps take about
    # --ref-budget seconds of host time.
    res = cpu_sample(args.ref_budget, args.steps, threads, dim=dim, workload=scn,
                     warmup=args.warmup, cfg=args.config)
    sample = sample_text(res, dim)
    return {
        "metric": METRIC, "value": res["value"], "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * res["seconds"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded dam-break lattice, hydrostatic start)",
        "config": describe(scn, workload),
        "impl": "reference",
        "cpu_baseline": {"value": res["value"], "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": res["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def tune(P, args) -> None:
    if args.cells_per_radius is not None:
        P.cells_per_radius = args.cells_per_radius
    P.kahan = args.kahan
    P.staging = args.staging
    P.resort = args.resort


def gpu_leg(scn, params, warmup: int, steps: int, profile_steps: int, ranks,
            autotune: bool = False, tuning: dict | None = None):
    from titsolver_gb300 import _abi

    ctx = _abi.Context(params)
    ctx.upload(scn["tanks"], scn["r"], scn["v"], scn["rho"])
    for t, fc in enumerate(scn.get("faces") or []):
        if fc is not None:
            ctx.set_faces(t, fc["face_verts"], fc["poly"])
    if tuning is not None:
        ctx.set_tuning(tuning["cells_per_radius"], tuning["block_size"],
                       tuning["lanes_per_particle"])
    elif autotune:
        # Untimed setup: the autotuner times a few steps per launch shape and
        # leaves the context at the fastest, with the uploaded state.
        ctx.autotune(3)
    if warmup:
        ctx.step(warmup)
    ranks.barrier()
    l0 = ctx.launch_count()
    ctx.timer_start()
    ctx.step(steps)
    ms = ctx.timer_stop()
    launches = ctx.launch_count() - l0
    ranks.barrier()
    prof = None
    if profile_steps:
        ctx.profile_enable(True)
        ctx.step(profile_steps)
        prof = ctx.profile_read()
        ctx.profile_enable(False)
    return ctx, ms, launches, prof


def fluid_mask(scn: dict) -> np.ndarray:
    return np.concatenate([np.r_[np.ones(t["n_fluid"], bool), np.zeros(t["n_wall"], bool)]
                           for t in scn["tanks"]])


def form_errors(scn: dict, ctx32, ctx64, steps: int) -> dict:
    """FP32C against FP64 on the fluid after the same number of steps from
    the same start: relative L2 of rho, r, v (field-relative), r against the
    displacement and rho against its deviation from rho0, the drift of total
    momentum and the time offset; total mass is exact (constant masses)."""
    from titsolver_gb300 import _abi

    f = fluid_mask(scn)
    r32, r64 = ctx32.download(_abi.TG_FIELD_R)[f], ctx64.download(_abi.TG_FIELD_R)[f]
    d32, d64 = ctx32.download(_abi.TG_FIELD_RHO)[f], ctx64.download(_abi.TG_FIELD_RHO)[f]
    v32, v64 = ctx32.download(_abi.TG_FIELD_V)[f], ctx64.download(_abi.TG_FIELD_V)[f]
    t32, t64 = ctx32.time(), ctx64.time()
    r0 = scn["r"][f]
    rho0 = np.concatenate([np.full(t["n_fluid"], t["rho0"]) for t in scn["tanks"]])
    # Equal masses within a tank: total momentum is m * sum(v) per tank.
    m = np.concatenate([np.full(t["n_fluid"], t["m"]) for t in scn["tanks"]])[:, None]
    p32, p64 = (m * v32).sum(axis=0), (m * v64).sum(axis=0)
    return {"steps": steps,
            "rho": float(np.linalg.norm(d32 - d64) / np.linalg.norm(d64)),
            "r": float(np.linalg.norm(r32 - r64) / np.linalg.norm(r64)),
            "v": float(np.linalg.norm(v32 - v64) / max(np.linalg.norm(v64), 1e-300)),
            "r_vs_displacement": float(np.linalg.norm(r32 - r64) /
                                       max(np.linalg.norm(r64 - r0), 1e-300)),
            "rho_vs_deviation": float(np.linalg.norm(d32 - d64) /
                                      max(np.linalg.norm(d64 - rho0), 1e-300)),
            "momentum_drift": float(np.linalg.norm(p32 - p64) /
                                    max(float((m * np.linalg.norm(v64, axis=1)[:, None]).sum()),
                                        1e-300)),
            "time_rel_diff": float(np.max(np.abs(t32 - t64) / np.maximum(t64, 1e-300))),
            "mass_exact": True,
            "normalisation": "field-relative ||x32 - x64|| / ||x64|| for r, rho and v; "
                             "r_vs_displacement divides by ||r64 - r0||"}


def error_leg(name: str, steps: int, tuning32: dict, tuning64: dict, dev: int) -> dict:
    """Both forms for `steps` steps from the start of workload `name` at the
    headline's launch shapes (untimed), and the FP32C error against FP64."""
    from titsolver_gb300 import _abi, physics

    workload, make = make_config(name)
    scn = make()
    ctxs = []
    for prec, tn in ((_abi.TG_FP32C, tuning32), (_abi.TG_FP64, tuning64)):
        P = physics.baseline_params(scn["dim"], precision=prec)
        P.device = dev
        ctx = _abi.Context(P)
        ctx.upload(scn["tanks"], scn["r"], scn["v"], scn["rho"])
        ctx.set_tuning(tn["cells_per_radius"], tn["block_size"], tn["lanes_per_particle"])
        ctx.step(steps)
        ctxs.append(ctx)
    err = form_errors(scn, ctxs[0], ctxs[1], steps)
    for c in ctxs:
        c.close()
    err["workload"] = workload
    err["fluid_particles"] = int(sum(t["n_fluid"] for t in scn["tanks"]))
    return err


def shares(p: dict) -> dict:
    """Share of the step's device time per kernel group (fractions)."""
    keys = (("sort", "sort_ms"), ("reorder", "reorder_ms"), ("walls", "walls_ms"),
            ("forces", "forces_ms"))
    tot = sum(p[k] for _, k in keys)
    return {n: round(p[k] / tot, 4) for n, k in keys}


def extra_workload(name: str, args, ranks, err_steps: int) -> dict:
    """Both forms on another workload (autotuned, warm-up, timed steps) and,
    with err_steps, the FP32C error against FP64 after err_steps steps (the
    contexts continue from the timed steps; untimed)."""
    from titsolver_gb300 import _abi, physics, scenarios

    workload, make = make_config(name)
    scn = make()
    nf = scenarios.n_fluid(scn)
    out = {"workload": workload, "fluid_particles": nf, "tanks": len(scn["tanks"])}
    ctxs = {}
    k = min(args.steps, 20)
    for form, prec in (("fp32c", _abi.TG_FP32C), ("fp64", _abi.TG_FP64)):
        P = physics.baseline_params(scn["dim"], precision=prec)
        P.device = ranks.local_rank
        ctx, ms, _, prof = gpu_leg(scn, P, args.warmup, k, 5, ranks, True)
        out[form] = {"value": nf * k / (ms / 1e3), "ms_per_step": ms / k, "steps": k,
                     "kernel_shares": shares(prof), "launch_shape": ctx.get_tuning()}
        ctxs[form] = ctx
    out["speedup_fp32c_over_fp64"] = out["fp32c"]["value"] / out["fp64"]["value"]
    done = args.warmup + k + 5
    if err_steps > done:
        for ctx in ctxs.values():
            ctx.step(err_steps - done)
        out["l2_error_vs_fp64"] = form_errors(scn, ctxs["fp32c"], ctxs["fp64"], err_steps)
    for ctx in ctxs.values():
        ctx.close()
    return out


def err_config(name: str) -> str:
    """Workload of the error leg: 1000 plain-FP64 steps of the 3D workloads
    at dx = H/200 take over ten minutes, so they use the 2M-fluid 3D dam
    break at dx = H/100; the others their own workload."""
    return "c4q" if name in ("c4", "c4half") else name


def run_gpu(args, ranks) -> dict | None:
    from titsolver_gb300 import _abi, physics, scenarios

    workload, make = make_config(args.config)
    scn = make()
    dim = scn["dim"]
    nf = scenarios.n_fluid(scn)
    dev = ranks.local_rank
    peaks = _peaks()

    # FP32-compensated form: the headline.
    P32 = physics.baseline_params(dim, precision=_abi.TG_FP32C)
    P32.device = dev
    tune(P32, args)
    clocks = ClockSampler(dev)
    clocks.start()
    auto = args.cells_per_radius is None and args.autotune == 1
    ctx32, ms32, launches, prof32 = gpu_leg(scn, P32, args.warmup, args.steps,
                                            min(args.steps, 20), ranks, auto)
    tuning32 = ctx32.get_tuning()
    clk = clocks.stop()
    sec32 = ms32 / 1e3
    value, t_max = (nf * args.steps / sec32, sec32)
    if ranks.world_size > 1:
        from titsolver_gb300.replicas import aggregate
        value, t_max = aggregate(nf * args.steps, sec32, ranks)

    # Plain FP64 form on the same workload and the same number of steps.
    P64 = physics.baseline_params(dim, precision=_abi.TG_FP64)
    P64.device = dev
    tune(P64, args)
    k64 = args.steps if args.fp64_steps is None else args.fp64_steps
    ctx64, ms64, _, prof64 = gpu_leg(scn, P64, args.warmup, k64, min(k64, 5), ranks, auto)
    tuning64 = ctx64.get_tuning()
    value64 = nf * k64 / (ms64 / 1e3)
    ctx64.close()

    # Live pair count of the compensated state (fluid targets, self excluded)
    # for the compute-side roofline.
    cnt, _ = ctx32.neighbour_counts()
    pairs = int(cnt[fluid_mask(scn)].sum()) - nf

    # End to end through the C ABI with pinned host buffers.
    n = scn["r"].shape[0]
    pin = {k: _abi.PinnedArray(shape) for k, shape in
           (("r", (n, dim)), ("v", (n, dim)), ("rho", (n,)), ("dv", (n, dim)))}
    ctx32.download(_abi.TG_FIELD_R, pin["r"].array)
    ctx32.download(_abi.TG_FIELD_V, pin["v"].array)
    ctx32.download(_abi.TG_FIELD_RHO, pin["rho"].array)
    ctx32.download(_abi.TG_FIELD_DV_DT, pin["dv"].array)
    ke = max(1, min(args.steps, args.e2e_steps))

    def e2e_step():
        ctx32.update(pin["r"].array, pin["v"].array, pin["rho"].array, pin["dv"].array)
        ctx32.step(1)
        ctx32.download_state(r=pin["r"].array, v=pin["v"].array, rho=pin["rho"].array,
                             dv_dt=pin["dv"].array)

    for _ in range(2):
        e2e_step()
    ranks.barrier()
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e_step()
    te = time.perf_counter() - t0
    e2e_value = nf * ke / te
    if ranks.world_size > 1:
        from titsolver_gb300.replicas import aggregate
        e2e_value, _ = aggregate(nf * ke, te, ranks)
    hd_bytes = n * 8 * (3 * dim + 1)
    ctx32.close()
    del pin

    # Error of the compensated form against FP64 (untimed).
    err = None
    if args.err_steps > 0:
        err = error_leg(args.err_config or err_config(args.config), args.err_steps,
                        tuning32, tuning64, dev)

    # Roofline of the fused force kernel.
    forces_avg_ms = prof32["forces_ms"] / max(prof32["forces_launches"], 1)
    alg = nf * 3 * state_bytes(dim, "fp32c")
    achieved = alg / (forces_avg_ms / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_forces (fused continuity+momentum+RK update)",
                "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"],
                "traffic": forces_traffic(dim, "fp32c", nf),
                "traffic_source": forces_traffic_source(dim, "fp32c"),
                "peak_source": f"{peaks['source']} hbm_gbs",
                "alg_bytes_per_launch": alg, "avg_launch_ms": forces_avg_ms,
                "compute": forces_compute(dim, nf, pairs, forces_avg_ms, clk,
                                          tuning32.get("cells_per_radius")),
                "ncu_working_ceiling": forces_ceiling(dim, "fp32c")}

    extras = {}
    for name in [x for x in args.extra.split(",") if x and x != args.config]:
        extras[name] = extra_workload(name, args, ranks,
                                      args.extra_err_steps if name == "c3" else 0)

    out = None
    if ranks.rank == 0:
        cpu = None
        if ranks.world_size == 1 and not args.no_cpu:
            import oracle
            threads = oracle.default_threads()
            c = cpu_sample(args.cpu_budget, 3, threads, dim=dim, workload=scn, warmup=1,
                           cfg=args.config)
            cpu = {"value": c["value"], "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": sample_text(c, dim)}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated sums; f64 positions and time)",
            "data": "synthetic (seeded dam-break lattice, hydrostatic start)",
            "config": describe(scn, workload),
            "form": {"name": "fp32c", "kahan": bool(P32.kahan)},
            "forms": {
                "fp32c": {"value": value, "ms_per_step": ms32 / args.steps,
                          "kernel_shares": shares(prof32), "launch_shape": tuning32},
                "fp64": {"value": value64, "ms_per_step": ms64 / k64, "steps": k64,
                         "kernel_shares": shares(prof64), "launch_shape": tuning64},
                "speedup_fp32c_over_fp64": value / value64 if value64 > 0 else None,
            },
            "l2_error_vs_fp64": err,
            "bytes_per_update": {"fp32c": bytes_per_update(dim, "fp32c"),
                                 "fp64": bytes_per_update(dim, "fp64")},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": hd_bytes,
                    "d2h_bytes_per_step": hd_bytes, "steps": ke},
            "gpu_launches": launches,
            "clocks": clk,
            "extra_workloads": extras,
        }
    return out


def run_cloud(args, ranks) -> dict | None:
    """Search + summation density over the point cloud (one pass per step),
    FP64 and FP32 positions; points/s."""
    import oracle
    from titsolver_gb300 import _abi, physics

    workload, make = make_config(args.config)
    scn = make()
    n = scn["r"].shape[0]
    t = scn["tanks"][0]
    P = physics.baseline_params(3)
    P.device = ranks.local_rank
    tune(P, args)
    ctx = _abi.Context(P)
    ctx.upload(scn["tanks"], scn["r"], scn["v"], scn["rho"])
    res = {}
    for prec, name in ((_abi.TG_POS_FP32, "fp32"), (_abi.TG_POS_FP64, "fp64")):
        for _ in range(args.warmup):
            ctx.summation_density_resident(prec)
        ctx.synchronize()
        ranks.barrier()
        l0 = ctx.launch_count()
        ctx.timer_start()
        for _ in range(args.steps):
            ctx.summation_density_resident(prec)
        ms = ctx.timer_stop()
        res[name] = {"value": n * args.steps / (ms / 1e3), "ms_per_pass": ms / args.steps,
                     "launches": ctx.launch_count() - l0}
    # Parity on a bounded sample: full oracle search + density, compared
    # on every point (counts and hashes bit-exact, rho within tolerance).
    rho, cnt, hs = ctx.summation_density(_abi.TG_POS_FP64)
    ctx.close()
    parity = None
    if ranks.rank == 0 and not args.no_cpu:
        t0 = time.perf_counter()
        orho, ocnt, ohs = oracle.summation_density(scn["r"], t["h"], t["m"], 3, 0)
        cpu_s = time.perf_counter() - t0
        parity = {"counts_equal": bool(np.array_equal(cnt, ocnt)),
                  "hashes_equal": bool(np.array_equal(hs, ohs)),
                  "rho_max_rel_err": float(np.max(np.abs(rho - orho) / orho)),
                  "neighbour_entries": int(ocnt.sum()), "oracle_seconds": cpu_s}
    if ranks.rank != 0:
        return None
    out = {"metric": "points/s: 3D neighbour search + summation density", "value": res["fp32"]["value"],
           "unit": "points/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": res["fp32"]["ms_per_pass"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 positions (and f64)",
           "data": "synthetic (seeded jittered lattice + Gaussian clusters)",
           "config": {"workload": workload, "points": n, "cells_per_radius": P.cells_per_radius},
           "forms": res, "parity_vs_oracle_fp64": parity,
           "bytes_per_point": {"fp64": 48, "fp32": 36}}
    if parity is not None:
        out["cpu_baseline"] = {"value": n / parity["oracle_seconds"], "unit": "points/s",
                               "cores": oracle.default_threads(), "kind": "port",
                               "sample": "the full cloud, one search + summation pass, FP64"}
    return out


def run_faces(args, ranks) -> dict | None:
    """The reference's face-wall mode (configs f2, f3): reference physics
    with shifting, both forms (or --only one), device time per step."""
    from titsolver_gb300 import _abi, physics, scenarios

    workload, make = make_config(args.config)
    scn = make()
    nf = scenarios.n_fluid(scn)
    # fp32c: FP64 face integrals (the default); fp32c_face32: tg_params.face_fp32.
    forms = [args.only] if args.only else ["fp32c", "fp32c_face32", "fp64"]
    res, launches, state = {}, 0, {}
    f = np.concatenate([np.r_[np.ones(t["n_fluid"], bool), np.zeros(t["n_wall"], bool)]
                        for t in scn["tanks"]])
    for form in forms:
        P = physics.reference_params(
            scn["dim"], precision=_abi.TG_FP64 if form == "fp64" else _abi.TG_FP32C)
        P.face_fp32 = 1 if form == "fp32c_face32" else 0
        P.post_integrate = _abi.TG_POST_SHIFTING
        P.device = ranks.local_rank
        ctx, ms, n_launch, _ = gpu_leg(scn, P, args.warmup, args.steps, 0, ranks, False)
        state[form] = {k: ctx.download(fld)[f] for k, fld in
                       (("r", _abi.TG_FIELD_R), ("v", _abi.TG_FIELD_V),
                        ("rho", _abi.TG_FIELD_RHO))}
        ctx.close()
        res[form] = {"value": nf * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps}
        launches += n_launch
    if ranks.rank != 0:
        return None
    err = None
    if "fp64" in state and len(state) > 1:
        b = state["fp64"]
        err = {"steps": args.warmup + args.steps}
        for form, a in state.items():
            if form != "fp64":
                err[form] = {k: float(np.linalg.norm(a[k] - b[k]) /
                                      max(np.linalg.norm(b[k]), 1e-300))
                             for k in ("rho", "r", "v")}
    cpu = None
    if ranks.world_size == 1 and not args.no_cpu:
        # The oracle on the same workload and physics (plain FP64, face walls,
        # shifting): one untimed step, then as many steps as fill the budget.
        import oracle
        threads = oracle.default_threads()
        P = physics.reference_params(scn["dim"], precision=_abi.TG_FP64)
        P.post_integrate = _abi.TG_POST_SHIFTING
        st = oracle.State(scn)
        t0 = time.perf_counter()
        oracle.step(P, st, 1, nthreads=threads)
        one = max(time.perf_counter() - t0, 1e-6)
        k = int(max(2, min(200, args.cpu_budget / one)))
        t0 = time.perf_counter()
        oracle.step(P, st, k, nthreads=threads)
        sec = time.perf_counter() - t0
        cpu = {"value": nf * k / sec, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": (f"the workload itself ({nf} fluid), reference physics with face "
                          f"walls and shifting, 1 untimed + {k} timed SSPRK3 steps "
                          f"({sec:.1f} s), oracle built g++ -O3 -ffp-contract=off")}
    head = res[forms[0]]
    return {"metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms_per_step"],
            "higher_is_better": True, "forms": res, "l2_error_vs_fp64": err,
            "faces": int(sum(fc["face_verts"].shape[0] for fc in scn["faces"] if fc)),
            "config": describe(scn, workload), "cpu_baseline": cpu,
            "gpu_launches": launches}


def run_single_form(args, ranks) -> dict | None:
    """One form on the configured workload (used under ncu)."""
    from titsolver_gb300 import _abi, physics, scenarios

    workload, make = make_config(args.config)
    scn = make()
    nf = scenarios.n_fluid(scn)
    form = _abi.TG_FP64 if args.only == "fp64" else _abi.TG_FP32C
    P = physics.baseline_params(scn["dim"], precision=form)
    P.face_fp32 = 1 if args.only == "fp32c_face32" else 0
    P.device = ranks.local_rank
    tune(P, args)
    auto = args.cells_per_radius is None and args.autotune == 1
    ctx, ms, launches, prof = gpu_leg(scn, P, args.warmup, args.steps, 0, ranks, auto)
    shape = ctx.get_tuning()
    ctx.close()
    if ranks.rank != 0:
        return None
    return {"metric": METRIC, "value": nf * args.steps / (ms / 1e3), "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "form": args.only, "launch_shape": shape,
            "cells_per_radius": shape["cells_per_radius"], "kahan": P.kahan,
            "staging": P.staging,
            "config": {"workload": workload}, "gpu_launches": launches}


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gpu", "reference"), default="gpu")
    ap.add_argument("--config", default="c4")
    ap.add_argument("--err-steps", type=int, default=1000,
                    help="steps of the FP32C-vs-FP64 error leg (0: skip)")
    ap.add_argument("--err-config", default=None,
                    help="workload of the error leg (default: c4q for c4/c4half, else --config)")
    ap.add_argument("--extra", default="c1,c3,c5",
                    help="further workloads timed in both forms (comma-separated)")
    ap.add_argument("--extra-err-steps", type=int, default=500,
                    help="steps after which c3's FP32C error is taken (0: skip)")
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="host seconds of the reference arm (warm-up + timed steps)")
    ap.add_argument("--fp64-steps", type=int, default=None,
                    help="FP64 timed steps (default: --steps)")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cells-per-radius", type=int, default=None,
                    help="grid cells per support radius (default: library default)")
    ap.add_argument("--kahan", type=int, choices=(0, 1), default=1)
    ap.add_argument("--autotune", type=int, choices=(0, 1), default=1,
                    help="pick the launch shape with tg_autotune before warm-up "
                         "(skipped when --cells-per-radius is given)")
    ap.add_argument("--staging", type=int, choices=(0, 1), default=0)
    ap.add_argument("--resort", type=int, choices=(0, 1), default=1,
                    help="re-sort only the particles whose cell changed (1) or a full "
                         "radix sort every stage (0)")
    ap.add_argument("--only", choices=("fp32c", "fp64", "fp32c_face32"), default=None,
                    help="time one form only (profiling runs); prints its value; "
                         "fp32c_face32 = fp32c with FP32 face integrals")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    from titsolver_gb300.replicas import init_from_env

    ranks = init_from_env()
    try:
        if args.impl == "reference":
            if ranks.rank != 0:
                return 0
            print(json.dumps(run_reference(args, ranks)), flush=True)
            return 0
        from titsolver_gb300 import build as gpu_build
        if ranks.rank == 0:
            gpu_build.build()
        ranks.barrier()
        if args.config == "c2":
            out = run_cloud(args, ranks)
        elif args.config in ("f2", "f3"):
            out = run_faces(args, ranks)
        elif args.only is not None:
            out = run_single_form(args, ranks)
        else:
            out = run_gpu(args, ranks)
        if out is not None:
            print(json.dumps(out), flush=True)
        return 0
    finally:
        ranks.close()


if __name__ == "__main__":
    sys.exit(main())
