"""Benchmark of the DFSPH step: particle-steps/s on the 1M-particle viscous dam break.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
python bench.py --profile-case N_SIDE [--lanes L]   (a short run for ncu to capture)

Workload (the 1M-particle high-viscosity dam break): 100^3 jittered lattice (r = 0.005, a 1 m block) in
a 2 x 1.5 x 1 m box (volume-map boundary), dynamic viscosity 50 Pa s with the
implicit CG solve (relative tolerance 1e-4), surface tension 0.05, CFL time
steps, pressure solve to <= 0.1 % mean density error. Synthetic seeded data.

value : particle-steps/s with the state resident in HBM (whole step as one
        CUDA graph, timed with CUDA events on the library's stream).
e2e   : the same metric through the C-ABI with host buffers: each step uploads
        positions and velocities from pinned host memory, steps, and reads back
        positions, velocities and accelerations.
roofline: the kernel with the largest share of the step, timed per launch with
        CUDA events (eager launches), against the measured HBM copy bandwidth.
cpu_baseline: the CPU restatement of the reference method (oracle, FP32, all
        host threads) on a 64k-particle sample of the same configuration.
--impl reference: that CPU restatement alone (the reference has no CPU DFSPH and
        its CUDA path needs Windows headers and a missing glm submodule).
Multi-GPU: replicas of the 1M scene (one per rank, weak scaling); the batched form splits
its 256 scenes across the ranks by particle count.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @1M, ≤0.1% density err: plain vs batched vs fwd+adjoint"
UNIT = "particle-steps/s"

# Algorithmic bytes per particle of each kernel, from the per-phase table of compulsory
# FP32 SoA traffic (each field counted once per synchronisation phase, neighbour-field
# gathers cache-served, neighbour-list and index traffic not counted), phase by phase
# onto the kernels that carry it. Kernels outside that table count the fields they must
# read and write once.
ALGO_BYTES = {
    "k_boundary": 28,                       # K1
    "k_density_factor": 32 + 32 + 56,       # K2 + K3, and K4 (the bench scene runs the divergence solve)
    "k_pressure_accel": 44,                 # K5 / K18
    "k_jacobi_iter": 60 + 4,                # K6 / K19 + the residual reduction
    "k_div_finish": 64 + 12,                # K7 + K8
    "k_visc_precond": 68 + 68,              # K12 + K13
    "k_visc_setup": 68,                     # r0
    "k_cg_p0": 60,                          # z0
    "k_cg_spmv": 56,                        # SpMV + dot
    "k_cg_update": 120,                     # alpha update
    "k_cg_p": 36,                           # beta update
    "k_visc_finish": 60 + 24,               # K15 + T1
    "k_velocity": 36,                       # K16
    "k_pres_init": 60,                      # K17
    "k_pres_finish": 56 + 36,               # K20 + K21
    "k_st_classify": 28,                    # surface tension, classification
    "k_st_smooth": 44,                      # surface tension, smoothing
    "k_st_blend": 60,                       # surface tension, blend
    "k_keys": 20,                           # search: key generation
    "k_slots": 4,                           # search: cell table
    "k_rank_gather": 48,                    # search: reorder of x, v
    "k_minmax": 12,                         # x -> grid bounds (outside the table)
    "k_neighbors": 12 + 4,                  # x -> count (outside the table; the list excluded)
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo, else the machine type)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().lower().startswith("model name"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines: list[str] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, fl in rows for k, v in enumerate(fl) if v.lower().startswith("active")})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


def dam_break_config(n_side: int) -> dict:
    edge = n_side * 0.01
    return {"workload": f"viscous dam break, {n_side ** 3} particles ({n_side}^3 lattice, r=0.005)",
            "particles": n_side ** 3, "box_m": [round(2 * edge + 0.02, 4), round(1.5 * edge + 0.02, 4),
                                                 round(edge + 0.02, 4)],
            "dynamic_viscosity_pa_s": 50.0, "cg_relative_tolerance": 1e-4, "surface_tension": 0.05,
            "pressure_error_bound": "0.1% of rho0 (MaxPressureSolverError=10)", "min_solver_iterations": 2,
            "boundary": "volume map (GPU-built, 40x30x20 cells)", "parallelism": "replicas",
            "l2": "inputs larger than L2 (device state ~1.3 GB for 1M particles, L2 129 MB)"}


def batched_form(V, scenes, steps: int, warmup: int, plain_every: int, ws: int = 1, rank: int = 0):
    """The uneven-scene batch (256 scenes, 2k-64k particles each) advanced as one
    simulation, against the plain step run scene by scene on every `plain_every`-th
    scene, each autotuned first. Both in particle-steps/s, timed with CUDA events on the
    library's stream.
    With several ranks the scenes are split by particle count (vfd_gb300.partition),
    each rank advances its share as one batch, and the whole batch's particle-steps are
    divided by the slowest rank's time."""
    import torch
    from vfd_gb300 import partition
    full = scenes.uneven_batch()
    costs = [len(s["x"]) for s in full]
    idx, batch = partition.local_scenes(full, rank, ws, costs)
    counts = [len(s["x"]) for s in batch]
    maps = [[V.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"],
                             s["desc"]["ParticleRadius"]) for b in s["boxes"]] for s in batch]

    def run(sim, k):
        stream = torch.cuda.ExternalStream(sim.GetStream())
        sim.Steps(warmup)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        sim.StepsAsync(k)
        e1.record(stream)
        sim.Synchronize()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1)

    # both sides autotuned (lanes, forms, block sizes), as the main form is
    sim = V.batch_simulation(batch, maps)
    sim.Steps(2)
    sim.Autotune(2)
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    ms_b = run(sim, steps)
    errs = [sim.GetDebugInfo(scene=k)["PressureSolverError"] for k in range(len(batch))]
    del sim
    if ws > 1:
        t = torch.tensor([ms_b, max(errs)], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        parts = partition.assign(costs, ws)
        return {"workload": f"{len(full)} uneven scenes over {ws} ranks ({sum(costs)} particles)", "steps": steps,
                "batched": sum(costs) * steps / (float(t[0]) / 1e3), "batched_ms_per_step": float(t[0]) / steps,
                "rank_imbalance": partition.imbalance(costs, parts), "max_pressure_error": float(t[1])}
    plain_n, plain_ms = 0, 0.0
    for k in range(0, len(batch), plain_every):
        one = V.scene_simulation(batch[k], maps=maps[k])
        one.Steps(2)
        one.Autotune(2)
        plain_ms += run(one, steps)
        plain_n += counts[k]
        del one
    batched = sum(counts) * steps / (ms_b / 1e3)
    plain = plain_n * steps / (plain_ms / 1e3)
    return {"workload": f"{len(batch)} uneven scenes (dam breaks and drops, 2k-64k particles, "
                        f"mu log-uniform 0.01-100 Pa s), {sum(counts)} particles in all",
            "steps": steps, "batched": batched, "batched_ms_per_step": ms_b / steps,
            "plain_scene_by_scene": plain, "plain_sample": f"every {plain_every}th scene run alone "
                                                          f"({plain_n} particles)",
            "batched_over_plain": batched / plain, "max_pressure_error": max(errs)}


def adjoint_form(V, scenes, steps: int = 60, every: int = 10, analytic_check: bool = True, eps: float = 1e-3,
                 check_overrides: dict | None = None):
    """The viscous drop (32k particles, mu = 10 Pa s), `steps` steps: the plain forward
    run, then the forward run with checkpoints every `every` steps plus the adjoint,
    both from the same initial state and timed on the host around synchronised calls.
    Loss = mean |x_T - y|^2, y a jittered copy of the drop moved by (0.05, -0.2, 0);
    its gradient is checked against central differences (relative step 1e-3) in the
    viscosity and along one random initial-velocity direction."""
    s = scenes.viscous_drop_33k()
    n = len(s["x"])
    rng = np.random.default_rng(scenes.config_seed(4))
    target = s["x"].astype(np.float64) + np.array([0.05, -0.2, 0.0]) + 0.25 * s["desc"]["ParticleRadius"] * \
        rng.standard_normal(s["x"].shape)
    sim = V.scene_simulation(s)
    sim.Steps(2)  # builds the step graphs
    sim.Autotune(2)  # lanes and block sizes for this scene size, as for the main form

    def restart(x=None, v=None, nu=None):
        d = dict(s["desc"])
        if nu is not None:
            d["Viscosity"] = d["BoundaryViscosity"] = nu
        sim.SetDescription(d)
        sim.SetFluidObjects(s["x"] if x is None else x, s["v"] if v is None else v)

    def loss(**kw):
        restart(**kw)
        sim.Steps(steps)
        x, _, _ = sim.GetState()
        return float(np.mean(np.sum((x.astype(np.float64) - target) ** 2, axis=1)))

    loss()  # warm-up of the forward path at this size
    restart()
    t0 = time.perf_counter()
    sim.Steps(steps)
    t_fwd = time.perf_counter() - t0
    restart()  # warm-up of the adjoint (its tape, checkpoints and graphs are allocated once)
    sim.AdjointForward(steps, every)
    x, v, _ = sim.GetState()
    sim.AdjointBackward(np.zeros_like(x), np.zeros_like(v))
    restart()
    t0 = time.perf_counter()
    sim.AdjointForward(steps, every)
    t_rec = time.perf_counter() - t0  # the forward run with its checkpoints and tape (synchronous)
    x, v, _ = sim.GetState()
    xb = (2.0 / n) * (x.astype(np.float64) - target)
    x0b, v0b, pb = sim.AdjointBackward(xb.astype(np.float32), np.zeros_like(v))
    t_adj = time.perf_counter() - t0
    adj_stats = sim.AdjointStats()
    # the same run with every step recorded in the forward pass (no segment replays):
    # what 280 GB of HBM allows at this size
    restart()
    sim.AdjointForward(steps, steps)
    sim.AdjointBackward(np.zeros_like(x), np.zeros_like(v))
    restart()
    t0 = time.perf_counter()
    sim.AdjointForward(steps, steps)
    x2, v2, _ = sim.GetState()
    sim.AdjointBackward(((2.0 / n) * (x2.astype(np.float64) - target)).astype(np.float32), np.zeros_like(v2))
    t_all = time.perf_counter() - t0

    # Gradient check by central differences on the smooth variant of the same scene.
    # The method has kinks a finite difference straddles: the adaptive time step follows
    # the fastest particle (an argmax), the divergence solve clamps its residual at zero,
    # the Jacobi loops stop at a tolerance, and the reference's kernel tables are
    # piecewise constant in |r|. The check therefore runs with a fixed time step of 1 ms,
    # the divergence solve off, the pressure iterations pinned (min = max = 3) and the
    # analytic kernel mode, with its own adjoint run; the viscosity CG keeps its tolerance.
    smooth = dict(MinPressureSolverIterations=3, MaxPressureSolverIterations=3, EnableDivergenceSolverError=0,
                  TimeStepSize=0.001, MinTimeStepSize=0.001, MaxTimeStepSize=0.001)
    smooth.update(check_overrides or {})
    nu = s["desc"]["Viscosity"]
    if analytic_check:
        sim.SetKernelMode(True)
        sim.SetFluidObjects(s["x"], s["v"])

    def restart_smooth(v=None, nu_=None):
        d = dict(s["desc"], **smooth)
        if nu_ is not None:
            d["Viscosity"] = d["BoundaryViscosity"] = nu_
        sim.SetDescription(d)
        sim.SetFluidObjects(s["x"], s["v"] if v is None else v)

    def loss_smooth(**kw):
        restart_smooth(**kw)
        sim.Steps(steps)
        x, _, _ = sim.GetState()
        return float(np.mean(np.sum((x.astype(np.float64) - target) ** 2, axis=1)))

    restart_smooth()
    sim.AdjointForward(steps, every)
    x, v, _ = sim.GetState()
    xb = (2.0 / n) * (x.astype(np.float64) - target)
    _, v0b_s, pb_s = sim.AdjointBackward(xb.astype(np.float32), np.zeros_like(v))
    fd_nu = (loss_smooth(nu_=nu * (1 + eps)) - loss_smooth(nu_=nu * (1 - eps))) / (2 * eps * nu)
    g_nu = float(pb_s[0] + pb_s[1])
    # along the gradient (unit RMS per component), where the change of the loss stands
    # far above FP32 rounding
    g64 = v0b_s.astype(np.float64)
    d = (g64 / np.sqrt(np.mean(g64 * g64))).astype(np.float32)
    fd_v = (loss_smooth(v=s["v"] + eps * d) - loss_smooth(v=s["v"] - eps * d)) / (2 * eps)
    g_v = float(np.sum(g64 * d))
    return {"workload": f"viscous drop, {n} particles (sphere r = 0.1 m), mu = 10 Pa s, {steps} steps, "
                        f"checkpoint every {every}",
            "forward": n * steps / t_fwd, "fwd_adjoint": n * steps / t_adj, "adjoint_over_forward": t_adj / t_fwd,
            "forward_s": t_fwd, "fwd_adjoint_s": t_adj,
            # the two passes apart: the recording forward run, and the reverse pass (replays included)
            "recording_forward_s": t_rec, "backward_s": t_adj - t_rec, "backward_over_forward": (t_adj - t_rec) / t_fwd,
            "every_step_recorded": {"fwd_adjoint_s": t_all, "adjoint_over_forward": t_all / t_fwd},
            "backward": {"replayed_steps": adj_stats["ReplayedSteps"],
                         "viscosity_cg_iterations": adj_stats["ViscositySolverIterations"],
                         "max_viscosity_cg_iterations": adj_stats["MaxViscositySolverIterations"]},
            "grad_check": {"variant": "same scene, fixed dt 1 ms, divergence solve off, pressure iterations "
                                      "pinned to 3, analytic kernel" if analytic_check else
                                      "same scene, fixed dt 1 ms, divergence solve off, pressure iterations "
                                      "pinned to 3, table kernel",
                           "dL_dmu_adjoint": g_nu, "dL_dmu_central_difference": fd_nu,
                           "rel_err_mu": abs(g_nu - fd_nu) / abs(fd_nu),
                           "dL_dv0_along_gradient_adjoint": g_v, "dL_dv0_along_gradient_central_difference": fd_v,
                           "rel_err_v0": abs(g_v - fd_v) / abs(fd_v), "step": eps}}


def jet_form(V, scenes, steps: int = 8, warmup: int = 2):
    """The jet-coiling scene: the viscous jet onto an 8M-particle pool, the inflow emitter adding a disk
    layer each time the flow has covered one spacing, run with FP32 absolute and with
    cell-relative positions. Reports particle-steps/s (host clock around synchronous
    steps, emission included), the mean density error of every step, the solver
    iterations and the step's algorithmic HBM bytes over its kernel time. The surface
    tension coefficient is scaled by (r / 25 mm)^3: at 0.07 and r = 1.5 mm the reference's
    surface-tension model accelerates the free surface to ~50 m/s within a few steps
    (the oracle and the GPU agree), which pins the time step to its minimum."""
    import torch
    from vfd_gb300 import emitter
    out = {}
    peak, _ = measured_peaks()
    for mode in ("absolute", "cell_relative"):
        s = scenes.jet_coiling_8m()
        r = s["desc"]["ParticleRadius"]
        sigma = 0.07 * (r / 0.025) ** 3
        s["desc"]["SurfaceTension"] = sigma
        sim = V.scene_simulation(s)
        if mode == "cell_relative":
            sim.SetPositionMode(True)
            sim.SetFluidObjects(s["x"], s["v"])
        f = s["inflow"]
        em = emitter.InflowEmitter(f["center"], f["direction"], f["radius"], f["speed"], r)
        em.run(sim, warmup)
        sim.Autotune(2)  # lanes, forms and block sizes for this scene, as for the main form (state restored)
        torch.cuda.synchronize()
        errs, its = [], []
        t0 = time.perf_counter()
        st = em.run(sim, steps, on_step=lambda k, st: (errs.append(100.0 * st["PressureSolverError"] / 1000.0),
                                                      its.append(st["ViscositySolverIterationCount"])))
        el = time.perf_counter() - t0
        n = sim.GetParticleCount()
        prof = sim.ProfileKernels(2)
        tot = sum(v[1] for v in prof.values())
        step_bytes = sum(ALGO_BYTES.get(k, 0) * n * c for k, (c, _) in prof.items())
        achieved = step_bytes / (tot / 1e3) / 1e9
        out[mode] = {"particles": n, "emitted": em.emitted, "particle_steps_per_s": n * steps / el,
                     "ms_per_step": 1e3 * el / steps, "mean_density_error_pct_per_step": errs,
                     "viscosity_iterations": its, "flags": st["Flags"], "time_step_s": st["TimeStepSize"],
                     "step_roofline": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak}}
        sim.close()
        del sim
    out["workload"] = (f"jet (inflow r 0.02 m, 1 m/s, 0.5 m above the floor) onto a pool of "
                       f"{out['absolute']['particles'] - out['absolute']['emitted']} particles, r = 1.5 mm, "
                       f"viscosity 0.2 (200 Pa s), surface tension {sigma:.3g} (0.07 x (1.5/25)^3), "
                       f"{warmup} + {steps} steps per mode")
    return out


def fp64_precision_form(V, scenes, steps: int = 10, pool=(400, 50, 400), sigma: float | None = None,
                        far: bool = True, compare_every: int = 0):
    """Precision of the FP32 step against the FP64 GPU path on the jet-coiling scene: the
    8M-particle pool with the jet column already flowing (no emitter, so all modes keep
    the same particles). FP64 (vfd_set_precision), FP32 absolute and FP32 cell-relative
    positions run `steps` steps in lockstep from the same FP32 inputs, and again with the
    scene translated by (1000, 200, -300) m unless `far` is off. Per step and mode: the
    mean density error at the pressure solve's exit (-rho0 sum(res)/N, % of rho0), the
    solver iteration counts and the viscosity CG's relative residual |r|/|b| where it
    stopped. Every `compare_every` steps (and after the last): each FP32 mode's position
    difference from the FP64 trajectory (mean, p99, max). Surface tension sigma, by
    default the jet form's 0.07 x (r / 25 mm)^3."""
    out = {}
    far_offset = (1000.0, 200.0, -300.0)
    modes = ("fp64", "fp32_absolute", "fp32_cell_relative")
    for suffix, offset in (("", (0.0, 0.0, 0.0)), ("_far", far_offset))[:2 if far else 1]:
        s = scenes.jet_column_8m(pool=pool, offset=offset)
        r = s["desc"]["ParticleRadius"]
        s["desc"]["SurfaceTension"] = 0.07 * (r / 0.025) ** 3 if sigma is None else sigma
        n = len(s["x"])
        sims = {}
        for mode in modes:
            sim = V.scene_simulation(s)
            if mode == "fp64":
                sim.SetPrecision(True)
            elif mode == "fp32_cell_relative":
                sim.SetPositionMode(True)
                sim.SetFluidObjects(s["x"], s["v"])
            sims[mode] = sim
        recs = {m: {"mean_density_error_pct_per_step": [], "iterations_per_step": [],
                    "viscosity_residual_per_step": [], "_s": 0.0} for m in modes}
        for m in modes[1:]:
            recs[m]["position_error_m_by_step"] = []
        for k in range(steps):
            for m in modes:
                t0 = time.perf_counter()
                st = sims[m].OnUpdate()
                recs[m]["_s"] += time.perf_counter() - t0
                recs[m]["mean_density_error_pct_per_step"].append(100.0 * st["PressureSolverError"] / 1000.0)
                recs[m]["iterations_per_step"].append([st["DivergenceSolverIterationCount"],
                                                       st["PressureSolverIterationCount"],
                                                       st["ViscositySolverIterationCount"]])
                recs[m]["viscosity_residual_per_step"].append(st["ViscositySolverError"])
            if (compare_every and (k + 1) % compare_every == 0) or k + 1 == steps:
                ref, _ = sims["fp64"].GetStateF64()  # the FP64 trajectory of the same (FP32) inputs
                for m in modes[1:]:
                    x, _, _ = sims[m].GetState()
                    e = np.linalg.norm(x.astype(np.float64) - ref, axis=1)
                    recs[m]["position_error_m_by_step"].append(
                        [k + 1, float(e.mean()), float(np.quantile(e, 0.99)), float(e.max())])
        for m in modes:
            rec = recs[m]
            rec["particle_steps_per_s"] = n * steps / rec.pop("_s")
            if m != "fp64":
                _, mean, p99, mx = rec["position_error_m_by_step"][-1]
                rec.update(mean_position_error_m=mean, p99_position_error_m=p99, max_position_error_m=mx)
                if not compare_every:
                    del rec["position_error_m_by_step"]
            out[m + suffix] = rec
            sims[m].close()
        del sims
    out["workload"] = (f"jet column onto a pool: {n} particles (pool {pool[0]}x{pool[1]}x{pool[2]}, r = 1.5 mm), "
                       f"surface tension {s['desc']['SurfaceTension']:.3g}, {steps} steps per mode in lockstep; "
                       f"FP32 modes against the FP64 GPU path" +
                       (", also translated by (1000, 200, -300) m" if far else ""))
    return out


def config_table(V, scenes):
    """Step rates of each benchmark scene on the GPU (FP32 graph step and FP64 path) and on
    the host (FP32 and FP64 oracle, all host threads), for the per-scene comparison table.
    Each rate is particles x steps / host wall time around synchronised step calls, after
    two warm-up steps; the 1M dam break runs on the host as its 64k (40^3) sample with
    the same parameters."""
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    cases = [
        ("c1_dam_break_8k", scenes.dam_break_8k(), 200, 20),
        ("c1b_dam_break_8k_2x1x1", scenes.dam_break_8k(box_scale=(2.0, 1.0, 1.0)), 200, 20),
        ("c2_viscous_dam_break_1M", scenes.viscous_dam_break(), 50, 0),
        ("c2_sample_viscous_dam_break_64k", scenes.viscous_dam_break(n_side=40), 50, 5),
        ("c4_viscous_drop_33k", scenes.viscous_drop_33k(), 60, 10),
    ]
    out = {"cpu": {"cores": O.get_threads(), "cpu_model": cpu_model()}}

    def rate(steps, n, k):
        steps(2)
        t0 = time.perf_counter()
        steps(k)
        return n * k / (time.perf_counter() - t0)

    def oracle_steps(orc):
        def run(k):
            for _ in range(k):
                orc.step()
        return run

    for name, s, gpu_steps, cpu_steps in cases:
        n = len(s["x"])
        rec = {"particles": n}
        for prec in ("fp32", "fp64"):
            sim = V.scene_simulation(s)
            if prec == "fp64":
                sim.SetPrecision(True)
            k = gpu_steps if prec == "fp32" else max(5, gpu_steps // 5)
            rec[f"gpu_{prec}"] = rate(sim.Steps, n, k)
            sim.close()
            del sim
        if cpu_steps:
            for bits in (32, 64):
                orc = O.scene_oracle(s, bits)
                rec[f"cpu_fp{bits}"] = rate(oracle_steps(orc), n, cpu_steps)
                del orc
        out[name] = rec
    return out


def legacy_sph_form(steps: int = 100, warmup: int = 5):
    """The reference's legacy SPH pipeline (vfd_sph_*): a 100^3 block (1M particles,
    r = 4 mm, h = 1 cm) falling in a 1.6 x 1.2 x 1.6 m world box, `steps` steps with the
    state on the device, host clock around synchronous calls; and the FP32 oracle (one
    thread) on a 20^3 block for 10 steps as its CPU sample."""
    from oracle import oracle as O
    from vfd_gb300 import scenes, sph
    d = sph.make_sph_desc(WorldMin=(-0.8, -0.6, -0.8), WorldMax=(0.8, 0.6, 0.8))
    x = scenes.lattice_block((100, 100, 100), 0.004, (-0.4, -0.5, -0.4), 0.05, scenes.SplitMix64(7))
    sim = sph.SPHSimulation(d, x)
    sim.Steps(warmup)
    t0 = time.perf_counter()
    sim.Steps(steps)
    el = time.perf_counter() - t0
    sim.close()
    xs = scenes.lattice_block((20, 20, 20), 0.004, (-0.05, -0.5, -0.05), 0.05, scenes.SplitMix64(7))
    o = O.SphOracle(d, xs)
    t1 = time.perf_counter()
    o.steps(10)
    cpu = len(xs) * 10 / (time.perf_counter() - t1)
    return {"workload": f"legacy SPH, {len(x)} particles (100^3 block, r = 4 mm, h = 1 cm), {steps} steps",
            "particle_steps_per_s": len(x) * steps / el, "ms_per_step": 1e3 * el / steps,
            "cpu_oracle_particle_steps_per_s": cpu, "cpu_sample": "FP32 oracle, one thread, 8000 particles, 10 steps"}


def precision_form(V, scenes, n_side: int = 40, steps: int = 20):
    """The 1M configuration's parameters at n_side^3 particles: positions after `steps`
    steps in FP32 with absolute and with cell-relative positions against the FP64
    oracle from the same FP32 inputs and volume map (the oracle uses all host threads)."""
    from oracle import oracle as O
    s = scenes.viscous_dam_break(n_side=n_side)
    r = s["desc"]["ParticleRadius"]
    maps = [O.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r) for b in s["boxes"]]
    O.set_threads(os.cpu_count() or 1)
    orc = O.scene_oracle(s, 64, maps=maps)
    for _ in range(steps):
        orc.step()
    xo, _, _ = orc.state()
    out = {"workload": f"viscous dam break parameters, {len(s['x'])} particles, {steps} steps, FP64 oracle "
                       f"from the same FP32 inputs"}
    for name, rel in (("absolute", False), ("cell_relative", True)):
        sim = V.DFSPHSimulation(V.make_desc(**s["desc"]))
        sim.SetPositionMode(rel)
        sim.SetFluidObjects(s["x"], s["v"])
        for m in maps:
            sim.AddRigidBody(m)
        st = sim.Steps(steps)
        x, _, _ = sim.GetState()
        e = np.linalg.norm(x.astype(np.float64) - xo, axis=1)
        out[name] = {"max_position_error_m": float(e.max()), "mean_position_error_m": float(e.mean()),
                     "mean_density_error_pct": 100.0 * st["PressureSolverError"] / 1000.0}
    return out


def cpu_baseline(n_side: int, steps: int, warmup: int):
    """The oracle (FP32, all host threads) on a sample with the 1M dam break's parameters."""
    from oracle import oracle as O
    from vfd_gb300 import scenes
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    s = scenes.viscous_dam_break(n_side=n_side)
    sim = O.scene_oracle(s, 32)
    for _ in range(warmup):
        sim.step()
    t = time.perf_counter()
    for _ in range(steps):
        sim.step()
    el = time.perf_counter() - t
    n = len(s["x"])
    return n * steps / el, el, n, O.get_threads()


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    n_side = 40
    value, el, n, cores = cpu_baseline(n_side, args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(dam_break_config(100), sample=f"{n} particles ({n_side}^3) with the same parameters"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"1M dam-break parameters at {n} particles, {args.steps} steps after {args.warmup}",
                         "cpu_model": cpu_model(), "nproc": os.cpu_count()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference's DFSPH step (no CPU DFSPH exists in the reference)",
    }
    print(json.dumps(line), flush=True)


def summary(line: dict) -> dict:
    """The forms' headline figures in a few keys at the end of the line, so that a
    reader of a truncated log still sees them."""
    f = line.get("forms", {})
    adj = f.get("fwd_adjoint", {})
    gc = adj.get("grad_check", {})
    out = {"value": line.get("value"), "e2e": (line.get("e2e") or {}).get("value"),
           "mean_density_error_pct": line.get("mean_density_error_pct"),
           "roofline_frac": (line.get("roofline") or {}).get("frac"),
           "roofline_kernel": (line.get("roofline") or {}).get("kernel"),
           "step_roofline_frac": (line.get("step_roofline") or {}).get("frac"),
           "batched_over_plain": f.get("batched", {}).get("batched_over_plain"),
           "adjoint_over_forward": adj.get("adjoint_over_forward"),
           "grad_rel_err_mu": gc.get("rel_err_mu"), "grad_rel_err_v0": gc.get("rel_err_v0"),
           "cpu_baseline": (line.get("cpu_baseline") or {}).get("value")}
    return {k: (round(v, 6) if isinstance(v, float) else v) for k, v in out.items()}


def profile_case(args):
    """The viscous dam break at args.profile_case^3 particles (the 1M configuration's
    parameters), --graph-steps graph steps (lanes per particle from --lanes, else
    autotuned), then --eager-steps steps with every kernel launched from the host."""
    import vfd_gb300 as V
    from vfd_gb300 import scenes
    V.lib().vfd_set_device(0)
    s = scenes.viscous_dam_break(n_side=args.profile_case)
    sim = V.scene_simulation(s)
    sim.Steps(2)
    if args.lanes:
        vals = [int(x) for x in args.lanes.split(",")]
        sim.SetLanes(vals * len(V.TUNED_KERNELS) if len(vals) == 1 else vals)
    else:
        log("lanes", sim.Autotune(1))
    if args.tiles >= 0:
        sim.SetTiles([args.tiles] * len(V.TUNED_KERNELS))
    sim.Steps(args.graph_steps)
    sim.SetGraphMode(False)
    import torch
    torch.cuda.synchronize()
    torch.cuda.profiler.start()  # `ncu --profile-from-start off` records the eager steps only
    st = sim.Steps(args.eager_steps)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    log("particles", len(s["x"]), "stats", st, "tiles", sim.GetTiles())


def adjoint_profile_case(args):
    """The adjoint form's scene and run (the 33k viscous drop, 60 steps, a checkpoint every
    10) with every kernel launched from the host, the forward and backward passes between
    cudaProfilerStart / Stop, for a profiler's launch list (graphs with conditional nodes
    hide their kernels from it)."""
    import numpy as np
    import vfd_gb300 as V
    from vfd_gb300 import scenes
    V.lib().vfd_set_device(0)
    s = scenes.viscous_drop_33k()
    n = len(s["x"])
    rng = np.random.default_rng(scenes.config_seed(4))
    target = s["x"].astype(np.float64) + np.array([0.05, -0.2, 0.0]) + 0.25 * s["desc"]["ParticleRadius"] * \
        rng.standard_normal(s["x"].shape)
    sim = V.scene_simulation(s)
    sim.SetGraphMode(False)
    sim.Steps(2)
    sim.SetFluidObjects(s["x"], s["v"])
    import torch
    torch.cuda.synchronize()
    torch.cuda.profiler.start()
    sim.AdjointForward(60, 10)
    x, v, _ = sim.GetState()
    sim.AdjointBackward(((2.0 / n) * (x.astype(np.float64) - target)).astype(np.float32), np.zeros_like(v))
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    log("particles", n, "adjoint", sim.AdjointStats())


def free_port() -> int:
    import socket
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def relaunch(n: int) -> int:
    """`bench.py --gpus N` outside torchrun: start N ranks on this node (one per GPU) with
    torch.distributed.run and the same arguments; rank 0 prints the line."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), os.path.abspath(__file__)] + sys.argv[1:]
    log("launching", n, "ranks:", " ".join(cmd))
    return subprocess.run(cmd).returncode


def dry_run(args):
    """The replica path of the benchmark on the CPU: a gloo process group, every rank
    advancing its own seeded scene (a 10^3 dam break, the FP32 oracle on one thread),
    barriers around the timed steps, the slowest rank's time, and rank 0's JSON line
    with n_gpus = world size. Tests the multi-rank launcher and reduction only."""
    import torch
    import torch.distributed as dist
    from oracle import oracle as O
    from vfd_gb300 import scenes
    ws, rank, _ = dist_info()
    if ws > 1:
        dist.init_process_group("gloo")
    O.set_threads(1)
    s = scenes.small_dam_break(n_side=10, seed=scenes.config_seed(2) + rank)
    sim = O.scene_oracle(s, 32)
    for _ in range(args.warmup):
        sim.step()
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st = sim.step()
    el = time.perf_counter() - t0
    if ws > 1:
        dist.barrier()
    t = torch.tensor([el], dtype=torch.float64)
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    n = len(s["x"])
    value = n * ws * args.steps / float(t.item())
    if rank == 0:
        print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": 1e3 * float(t.item()) / args.steps,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic", "dry_run": True,
                          "config": {"workload": f"dry run: {n}-particle dam break per rank on the CPU oracle",
                                     "parallelism": f"replicas x{ws}"},
                          "mean_density_error_pct": 100.0 * st["PressureSolverError"] / 1000.0}), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)  # the 1M dam break's 500 steps
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-side", type=int, default=100)
    ap.add_argument("--e2e-steps", type=int, default=0, help="end-to-end steps (default: --steps, the same steps)")
    ap.add_argument("--lanes", default="", help="lanes per particle instead of autotuning: N, or one per tuned "
                    "kernel (comma-separated); profilers use it, as they distort the autotuner's timings")
    ap.add_argument("--cpu-steps", type=int, default=150)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched-scene measurement")
    ap.add_argument("--no-jet", action="store_true", help="skip the 8M-particle jet-coiling form")
    ap.add_argument("--batch-steps", type=int, default=200, help="steps of the uneven-scene batch (the "
                    "configuration's 200)")
    ap.add_argument("--precision-steps", type=int, default=5,
                    help="steps per mode of the FP64-vs-FP32 precision form on the 8M jet scene")
    ap.add_argument("--precision-only", action="store_true",
                    help="run only the FP64-vs-FP32 precision form (with --precision-steps) and print its JSON")
    ap.add_argument("--precision-sigma", type=float, default=None,
                    help="surface tension of the precision form (default 0.07 x (r / 25 mm)^3; 0.07 is the literal value)")
    ap.add_argument("--precision-no-far", action="store_true", help="precision form at the origin only")
    ap.add_argument("--precision-compare-every", type=int, default=0,
                    help="compare positions with the FP64 run every this many steps (default: after the last)")
    ap.add_argument("--config-table", action="store_true",
                    help="print only the per-scene step rates (GPU FP32 and FP64, host oracle FP32 and FP64)")
    ap.add_argument("--eager", action="store_true",
                    help="launch the timed steps kernel by kernel instead of as CUDA graphs (same kernels, same "
                         "results); profilers cannot see the kernels inside graphs with conditional nodes")
    ap.add_argument("--profile-case", type=int, default=0, metavar="N_SIDE",
                    help="profiling run instead of the benchmark: the viscous dam break at N_SIDE^3 particles, "
                         "--graph-steps steps as CUDA graphs, then --eager-steps steps with every kernel launched "
                         "from the host (what a profiler filtering by kernel name captures)")
    ap.add_argument("--tiles", type=int, default=-1, help="form of the three solver-loop passes instead of the "
                    "autotuner's choice: 0 = neighbour rows, 1 = rows with gradW recomputed, 3 = 2x2x2 cell tiles, "
                    "4 = 4x2x2 cell tiles")
    ap.add_argument("--adjoint-profile-case", action="store_true",
                    help="profiling run instead of the benchmark: the adjoint form's run with every kernel launched "
                         "from the host")
    ap.add_argument("--graph-steps", type=int, default=4)
    ap.add_argument("--eager-steps", type=int, default=2)
    ap.add_argument("--dry-run", action="store_true",
                    help="exercise the multi-rank path on the CPU: gloo process group, each rank steps a small "
                         "scene with the FP32 oracle instead of the GPU, same barriers, max-over-ranks timing "
                         "and JSON line (for testing the launcher without GPUs; the numbers are not a benchmark)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return relaunch(args.gpus)
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_case:
        return profile_case(args)
    if args.adjoint_profile_case:
        return adjoint_profile_case(args)
    if args.dry_run:
        return dry_run(args)
    if args.precision_only:
        import vfd_gb300 as V
        from vfd_gb300 import scenes
        V.lib().vfd_set_device(0)
        print(json.dumps({"fp64_precision": fp64_precision_form(
            V, scenes, args.precision_steps, sigma=args.precision_sigma, far=not args.precision_no_far,
            compare_every=args.precision_compare_every)}), flush=True)
        return
    if args.config_table:
        import vfd_gb300 as V
        from vfd_gb300 import scenes
        V.lib().vfd_set_device(0)
        print(json.dumps({"config_table": config_table(V, scenes)}), flush=True)
        return

    import torch
    import torch.distributed as dist

    import vfd_gb300 as V
    from vfd_gb300 import scenes

    ws, rank, local = dist_info()
    if ws > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    V.lib().vfd_set_device(local)

    s = scenes.viscous_dam_break(n_side=args.n_side, seed=scenes.config_seed(2) + rank)
    n = len(s["x"])
    sim = V.scene_simulation(s)
    sim.Steps(1)
    if args.lanes:  # fixed lanes per particle (one value, or one per tuned kernel)
        vals = [int(x) for x in args.lanes.split(",")]
        vals = vals * len(V.TUNED_KERNELS) if len(vals) == 1 else vals
        sim.SetLanes(vals)
        lanes = dict(zip(V.TUNED_KERNELS, vals))
    else:
        lanes = sim.Autotune(2)  # per-kernel lanes per particle and tile sizes, state restored
    if args.tiles >= 0:
        sim.SetTiles([args.tiles] * len(V.TUNED_KERNELS))
    sim.SetGraphMode(not args.eager)
    sim.Steps(args.warmup)
    stream = torch.cuda.ExternalStream(sim.GetStream())

    def timed(k):
        sim.GetLaunchCount(reset=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize()
        if args.eager:  # `ncu --profile-from-start off` then records the timed steps' kernels
            torch.cuda.profiler.start()
        e0.record(stream)
        sim.StepsAsync(k)
        e1.record(stream)
        st = sim.Synchronize()
        torch.cuda.synchronize()
        if args.eager:
            torch.cuda.profiler.stop()
        if ws > 1:
            dist.barrier()
        return e0.elapsed_time(e1), st, sim.GetLaunchCount()

    with ClockSampler(local) as clk:
        try:
            ms, st, launches = timed(args.steps)
        except V.VFDError as e:  # grid grew past the table mid-run: the table was enlarged, time again
            log("retiming after", e)
            sim.Steps(1)
            ms, st, launches = timed(args.steps)
    clocks = clk.summary()
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = n * ws * args.steps / (ms_max / 1e3)

    # end to end through the C-ABI with pinned host buffers, over the same simulated steps
    # as the timed region: the scene restarts and advances to where that region began
    e2e_steps = args.e2e_steps or args.steps
    sim.SetFluidObjects(s["x"], s["v"])
    sim.Steps(1 + args.warmup)
    pin = lambda: torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
    xh, vh, ah = pin(), pin(), pin()
    sim.GetStateInto(xh, vh, ah)
    torch.cuda.synchronize()
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sim.SetState(xh, vh)
        sim.OnUpdate()
        sim.GetStateInto(xh, vh, ah)
    el = time.perf_counter() - t0
    t = torch.tensor([el], dtype=torch.float64, device="cuda")
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e = {"value": n * ws * e2e_steps / float(t.item()), "unit": UNIT, "steps": e2e_steps, "h2d_bytes_per_step": 24 * n,
           "d2h_bytes_per_step": 36 * n}

    # per-kernel event timing of eager launches -> dominant kernel and roofline; by default
    # `ncu --profile-from-start off` records exactly these launches (the kernel shares' list)
    torch.cuda.synchronize()
    if not args.eager:
        torch.cuda.profiler.start()
    prof = sim.ProfileKernels(3)
    torch.cuda.synchronize()
    if not args.eager:
        torch.cuda.profiler.stop()
    tot = sum(v[1] for v in prof.values())
    name, (cnt, kms) = max(prof.items(), key=lambda kv: kv[1][1])
    peak, peak_kind = measured_peaks()
    roof = None
    if name in ALGO_BYTES and cnt:
        bytes_launch = ALGO_BYTES[name] * n
        achieved = bytes_launch / (kms / cnt / 1e3) / 1e9
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic.json")
        if os.path.exists(tp):
            with open(tp) as f:
                tr = json.load(f).get(name)
            if tr:
                traffic = tr["bytes_per_particle"] * n
        roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": bytes_launch, "avg_launch_ms": kms / cnt,
                "share_of_step": kms / tot}
        if traffic:
            # the DRAM rate the measured traffic implies: ncu's bytes per launch (cold
            # cache, scaled from the 512k capture) over this run's launch time
            roof["traffic_gbs"] = traffic / (kms / cnt / 1e3) / 1e9
            roof["traffic_frac"] = roof["traffic_gbs"] / peak
    # the whole step: algorithmic bytes of every launch over the summed kernel time
    step_bytes = sum(ALGO_BYTES.get(k, 0) * n * c for k, (c, _) in prof.items())
    step_achieved = step_bytes / (tot / 1e3) / 1e9
    step_roof = {"achieved": step_achieved, "peak": peak, "unit": "GB/s", "frac": step_achieved / peak,
                 "algorithmic_bytes_per_step": step_bytes / 3, "kernel_ms_per_step": tot / 3}
    shares = {k: round(v[1] / tot, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][1])[:8]}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (f64 reductions)", "data": "synthetic (seeded jittered lattice)",
        "config": dict(dam_break_config(args.n_side), launch="eager" if args.eager else "cuda graph per step"),
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches,
        "roofline": roof, "step_roofline": step_roof, "kernel_shares": shares, "lanes_per_particle": lanes,
        "tile_log2_cells": sim.GetTiles(), "threads_per_block": sim.GetBlocks(),
        "solver": {k: st[k] for k in ("DivergenceSolverIterationCount", "PressureSolverIterationCount",
                                      "ViscositySolverIterationCount", "PressureSolverError", "TimeStepSize",
                                      "MaxNeighborCount", "Flags")},
        "mean_density_error_pct": 100.0 * st["PressureSolverError"] / 1000.0,
    }
    if not args.no_forms:
        line["forms"] = {"batched": batched_form(V, scenes, args.batch_steps, 3, 16, ws, rank)}
        if ws == 1:
            line["forms"]["fwd_adjoint"] = adjoint_form(V, scenes)
            line["forms"]["precision"] = precision_form(V, scenes)
            if not args.no_jet:
                line["forms"]["jet_8m"] = jet_form(V, scenes)
                line["forms"]["fp64_precision"] = fp64_precision_form(V, scenes, args.precision_steps)
            line["forms"]["legacy_sph"] = legacy_sph_form()
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        v, el, nc, cores = cpu_baseline(40, args.cpu_steps, 2)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"oracle FP32 on the 1M dam-break parameters at {nc} particles (40^3), "
                                          f"{args.cpu_steps} steps after 2 ({el:.1f} s)",
                                "cpu_model": cpu_model(), "nproc": os.cpu_count()}
    line["summary"] = summary(line)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
