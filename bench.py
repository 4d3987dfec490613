"""Benchmark: fused LSRK(5,4) advection step, 6D (3x+3v) k=3, 8^3 x 8^3 cells, FP32 storage.

One step = one rk45 time step of the phase-space upwind-DG advection operator
(ECL, Gauss-Lobatto collocation) fused with the stage update: 5 kernel launches
over 1,073,741,824 DoFs.  Metric: GDoF/s in the reference's time-stepping
definition, DoFs * stages * steps / time
(examples/advection/include/application.h:540-543).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
  python bench.py --workload adv2d    (2D k=3 32 x 32, 100 steps, per-step launches vs CUDA graph)
  python bench.py --workload adv4d    (4D k=3 16^2 x 16^2, FP32 and FP64, its own JSON line)
  python bench.py --workload vp2x2v   (the Vlasov-Poisson configuration, its own JSON line)
  python bench.py --workload batch64  (64 batched uneven instances, its own JSON line)

The FP64 form of the same step is timed after the FP32 form (fewer steps) and
the relative L2 difference of the two solutions after the timed steps is
reported.  ``--impl reference`` times the CPU restatement of the reference
operator (the oracle) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "advection GDoF/s (6D k=3) FP32 vs FP64 form at stated L2 err; % HBM roofline"
UNIT = "GDoF/s"
DIM_X = DIM_V = 3
DEGREE = 3
CELLS = 8
VELOCITY = [1.0, 0.8, 0.6, 0.4, 0.3, 0.2]
CFL = 0.2
N_STAGES = 5
# algorithmic passes over the vector per rk45 step of the fused path:
# stage 1 reads U, writes U' and T (3); stages 2-4 read T, U and write U, T' (4 each);
# stage 5 reads T, U and writes U (3)
PASSES_PER_STEP = 18


def workload_config(extra=None):
    cfg = {
        "workload": "6D (3x+3v) upwind DG advection, k=3 Gauss-Lobatto collocation, 8^3 x 8^3 cells "
                    "(262,144 cells, 1,073,741,824 DoFs), periodic unit box, velocity "
                    "(1.0, 0.8, 0.6, 0.4, 0.3, 0.2), fused rk45 LSRK step, FP32 storage",
        "dims": "3x+3v", "degree": DEGREE, "cells": "8^3 x 8^3", "n_dofs": 1073741824, "rk": "rk45",
        "stages": N_STAGES, "initial": "prod_d sin(2 pi x_d + phi_d), phi = default_rng(0).uniform(0, 2 pi, 6)",
        "l2_flush": "inputs larger than L2 (4.3 GB per FP32 vector vs 129 MB L2)",
    }
    if extra:
        cfg.update(extra)
    return cfg


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        if d.get("hbm_gbs"):
            return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per (average) stage launch from the committed ncu summary of the stage kernel (or None)."""
    p = os.path.join(ROOT, "profiles", "ecl_stage_6d_k3_f32.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("dram_bytes_per_avg_launch")
    return None


def cpu_sample(threads: int | None = None):
    """Oracle rk45 step on a 4^3 x 4^3 mesh of the same 6D k=3 problem (16.8M DoFs), all host threads."""
    import numpy as np

    from oracle import oracle as O
    O.build()
    n = os.cpu_count() if threads is None else threads
    cells = 4
    prob = O.Problem(DIM_X, DIM_V, DEGREE, [cells] * 6, [0.0] * 6, [1.0] * 6, VELOCITY, n_threads=n)
    rng = np.random.default_rng(0)
    phi = rng.uniform(0, 2 * math.pi, 6)
    f = O.make_func(2, 1.0, omega=[2 * math.pi] * 6, speed=[0.0] * 6, phase=list(phi))
    u = O.interpolate(prob, f)
    Ki = np.zeros_like(u)
    Ti = np.zeros_like(u)
    dt = 1e-3
    t0 = time.perf_counter()
    O.lsrk_step(prob, "rk45", u, 0.0, dt, Ki, Ti)
    el = time.perf_counter() - t0
    return {"value": prob.n_dofs * N_STAGES / el / 1e9, "unit": UNIT, "cores": n, "kind": "port",
            "sample": "one rk45 step of the oracle (CPU restatement, FP64) on the same 6D k=3 problem with "
                      "4^3 x 4^3 cells (16,777,216 DoFs), %.2f s" % el}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    vals = []
    for _ in range(max(1, args.warmup_cpu)):
        cpu_sample()
    info = None
    for _ in range(args.steps_cpu):
        info = cpu_sample()
        vals.append(info["value"])
    v = sorted(vals)[len(vals) // 2]
    info["value"] = v
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps_cpu,
           "warmup": args.warmup_cpu, "higher_is_better": True, "impl": "reference", "dtype": "f64",
           "data": "synthetic", "config": workload_config({"cpu_sample_mesh": "4^3 x 4^3 cells"}),
           "cpu_baseline": info, "vs_baseline": None,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


VP_DIM_X = 2
VP_CELLS_X, VP_CELLS_V = 16, 32
VP_CFL = 0.05


def vp_config(extra=None):
    cfg = {"workload": "electrostatic Vlasov-Poisson 2x2v, k=3 Gauss-Lobatto collocation, x in [0,4pi]^2 with "
                       "16^2 cells, v in [-6,6]^2 with 32^2 cells (262,144 cells, 67,108,864 DoFs; 4,096 x-DoFs), "
                       "periodic, f0 = (1 + 0.01 cos(0.5 x1) cos(0.5 x2)) exp(-|v|^2/2)/(2 pi), rk45, "
                       "dt = 0.05 dt_crit / k^1.5 with transport velocity (1, 1, 6, 6)",
           "dims": "2x+2v", "degree": 3, "n_dofs": 67108864, "x_dofs": 4096, "rk": "rk45",
           "l2_flush": "inputs larger than L2 (537 MB per FP64 vector vs 129 MB L2)"}
    if extra:
        cfg.update(extra)
    return cfg


def run_vp(args):
    """Vlasov-Poisson step time and CG iterations with the plain (previous-potential), zero and
    learned initial guesses at a fixed accuracy ||r|| <= tol ||rhs||, and the field energy
    against the FP64 oracle after a few steps."""
    import numpy as np
    import torch

    from hyperdeal_gb300 import vlasov_poisson as V

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rank = int(os.environ.get("RANK", "0"))
    two_pi = 4 * math.pi
    hx, hv = two_pi / VP_CELLS_X, 12.0 / VP_CELLS_V
    dt = V.time_step_rule(1.0, VP_CFL, min(hx / 1.0, hv / 6.0), DEGREE, 0.0, 1.0)
    f0 = V.perturbed_maxwellian(VP_DIM_X, eps=0.01, k=0.5, perturbed_dims=(0, 1))

    def make(guess, dtype, tol, rhs_rel, precond=args.vp_precond):
        # "learned": the least-squares fitted network; "learned_adam": the Adam-trained one;
        # "direct": no CG, the SIPG matrix's pseudo-inverse applied (hd_vp_solver)
        p = V.VlasovPoissonParameters(VP_DIM_X, DEGREE, [VP_CELLS_X] * 2, [VP_CELLS_V] * 2, [0.0] * 2,
                                      [two_pi] * 2, [-6.0] * 2, [6.0] * 2, dtype=dtype, cg_tol=tol,
                                      guess="learned" if guess.startswith("learned") else
                                      "zero" if guess == "direct" else guess,
                                      cg_rhs_relative=rhs_rel, cg_precond=precond,
                                      learn_fit="adam" if guess == "learned_adam" else "least_squares",
                                      poisson_solver="direct" if guess == "direct" else "cg")
        return V.VlasovPoissonOperation(p)

    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    runs = {}
    clocks = None
    selected = [r.strip() for r in args.vp_runs.split(",")]
    for dtype in ("f64", "f64x", "f32"):  # f64x: FP64 storage, FP32x2 advection contractions
        for guess in ("previous", "zero", "learned", "learned_adam", "previous_noprecond", "zero_noprecond",
                      "learned_noprecond", "direct"):
            if "%s/%s" % (dtype, guess) not in selected:
                continue
            pre = "none" if guess.endswith("_noprecond") else args.vp_precond
            op = make(guess.replace("_noprecond", ""), dtype[:3], args.vp_tol, True, pre)
            if dtype == "f64x":
                op.set_arithmetic("fp32x2")
            sol = op.initialize_dof_vector()
            op.interpolate(f0, sol)
            Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
            integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
            t = 0.0
            for _ in range(args.warmup):
                op.perform_time_step(integ, sol, t, dt)
                t += dt
            torch.cuda.synchronize()
            st0 = op.cg_stats()
            sampler = None
            if dtype == "f64" and guess == "learned":
                sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
                sampler.start()
                time.sleep(0.3)
            w0 = time.perf_counter()
            e0.record(stream)
            for _ in range(args.steps):
                op.perform_time_step(integ, sol, t, dt)
                t += dt
            e1.record(stream)
            torch.cuda.synchronize()
            wall = (time.perf_counter() - w0) * 1e3 / args.steps
            if sampler is not None:
                clocks = sampler.stop()
            st1 = op.cg_stats()
            solves = st1["solves"] - st0["solves"]
            runs["%s/%s" % (dtype, guess)] = {
                "ms_per_step": round(e0.elapsed_time(e1) / args.steps, 4), "wall_ms_per_step": round(wall, 4),
                "cg_iterations_per_solve": round((st1["total_iterations"] - st0["total_iterations"]) / solves, 3),
                "learned_picked": st1["learned_picked"] - st0["learned_picked"], "solves": solves,
                "field_energy": op.diagnostics(sol)[:VP_DIM_X]}
            del op, sol, Ki, Ti, integ
            torch.cuda.empty_cache()

    # field energy after a few steps from f0: GPU (FP64 and FP32 storage, learned guess) vs FP64 oracle
    energy = {}
    if args.vp_oracle_steps > 0:
        from oracle import oracle as O
        prob = O.Problem(2, 2, DEGREE, [VP_CELLS_X] * 2 + [VP_CELLS_V] * 2, [0.0, 0.0, -6.0, -6.0],
                         [two_pi, two_pi, 6.0, 6.0], [1.0, 1.0, 6.0, 6.0], collocation=True)
        fo = O.interpolate(prob, O.vp_initial_function(2, 2, eps=0.01, k=0.5, perturbed_dims=(0, 1)))
        st = O.VPState(prob, 1e-12)
        c0 = time.perf_counter()
        for s in range(args.vp_oracle_steps):
            O.lsrk_step_op("rk45", fo, s * dt, dt, st.operator)
        cpu_s = (time.perf_counter() - c0) / args.vp_oracle_steps
        e_ref = np.array(st.diagnostics(fo)[:VP_DIM_X])
        for dtype in ("f64", "f64x", "f32"):
            op = make("learned", dtype[:3], args.vp_tol, True)
            if dtype == "f64x":
                op.set_arithmetic("fp32x2")
            sol = op.initialize_dof_vector()
            op.interpolate(f0, sol)
            Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
            integ = V.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
            for s in range(args.vp_oracle_steps):
                op.perform_time_step(integ, sol, s * dt, dt)
            e = np.array(op.diagnostics(sol)[:VP_DIM_X])
            energy[dtype] = {"field_energy": list(e), "rel_err_vs_oracle": float(np.abs(e - e_ref).max() /
                                                                                  np.abs(e_ref).max())}
            del op, sol, Ki, Ti, integ
            torch.cuda.empty_cache()
        energy["oracle"] = {"field_energy": list(e_ref), "steps": args.vp_oracle_steps}
        cpu = {"value": round(cpu_s * 1e3, 1), "unit": "ms/step", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d rk45 steps of the full workload by the oracle (FP64, OpenMP)" % args.vp_oracle_steps}
    else:
        cpu = None

    if rank == 0:
        main_run = runs.get("f64/learned") or next(iter(runs.values()))
        plain = runs.get("f64/previous")
        n = 67108864
        out = {"metric": "Vlasov-Poisson 2x2v k=3 step time (rk45, FP64 phase space, FP64 CG)", "value":
               main_run["ms_per_step"], "unit": "ms/step", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": main_run["ms_per_step"], "higher_is_better": False, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": vp_config({"cg_tolerance": "||r|| <= %g ||rhs||" % args.vp_tol, "dt": dt}),
               "gdof_per_s": round(n * N_STAGES / (main_run["ms_per_step"] / 1e3) / 1e9, 3),
               "plain_guess": plain, "runs": runs, "field_energy_vs_oracle": energy, "cpu_baseline": cpu,
               "clocks": clocks}
        print(json.dumps(out))
    return 0


def batch_workload(seed: int = 0):
    """The seeded 64-instance workload: dimension 4 (2x+2v) or 5 (2x+3v / 3x+2v), degree 2..5,
    cells per dimension drawn independently from 4..12, unit-norm random velocity, FP32 or FP64."""
    import numpy as np
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(64):
        D = int(rng.choice([4, 5]))
        dx = 2 if D == 4 else int(rng.choice([2, 3]))
        k = int(rng.integers(2, 6))
        cells = [int(c) for c in rng.integers(4, 13, size=D)]
        dtype = "f32" if rng.random() < 0.5 else "f64"
        v = rng.standard_normal(D)
        specs.append((dx, D - dx, k, cells, dtype, list(v / np.linalg.norm(v))))
    return specs


def run_batch(args):
    """64 uneven instances: per-instance fused steps vs one persistent launch per class and stage
    (default and autotuned tiles) vs a replayed two-step CUDA graph."""
    import torch

    from hyperdeal_gb300 import advection as A
    from hyperdeal_gb300 import batch as Bt

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    specs = batch_workload(0)
    ops, sols, Ks, Ts, dts = [], [], [], [], []
    for dx, dv, k, cells, dtype, vel in specs:
        p = A.AdvectionParameters(dx, dv, k, cells[:dx], cells[dx:], [0.0] * dx, [1.0] * dx, [0.0] * dv, [1.0] * dv,
                                  vel, dtype=dtype)
        op = A.AdvectionOperation(p)
        u = op.initialize_dof_vector()
        A.VectorTools.interpolate(op, A.Function(2, 1.0, omega=[2 * math.pi] * (dx + dv), speed=[0.0] * (dx + dv)), u)
        ops.append(op)
        sols.append(u)
        Ks.append(op.initialize_dof_vector())
        Ts.append(op.initialize_dof_vector())
        dts.append(0.2 * op.critical_time_step() / k ** 1.5)
    n_total = sum(op.n_dofs for op in ops)
    bytes_step = sum(18 * (8 if op.dtype == torch.float64 else 4) * op.n_dofs for op in ops)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times = [0.0] * len(ops)

    def timed(fn, k):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    integs = [A.LowStorageRungeKuttaIntegrator(K, T, "rk45") for K, T in zip(Ks, Ts)]

    def per_instance():
        for op, u, it, dt in zip(ops, sols, integs, dts):
            it.perform_time_step(u, 0.0, dt, op)

    ms_single = timed(per_instance, args.steps)
    batch = Bt.AdvectionBatch(ops)

    def batched():
        batch.perform_time_step(sols, Ks, Ts, times, dts)

    ms_default = timed(batched, args.steps)
    t0 = time.perf_counter()
    classes = batch.autotune(sols, Ks, reps=2)
    tune_s = time.perf_counter() - t0
    ms_tuned = timed(batched, args.steps)
    batch.capture_graph(sols, Ks, Ts, times, dts)
    sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    sampler.start()
    time.sleep(0.3)
    ms_graph2 = timed(batch.replay_graph, max(1, args.steps // 2))
    clocks = sampler.stop()
    ms_graph = ms_graph2 / 2
    launches_per_step = N_STAGES * sum(1 if c["batched"] else c["members"] for c in classes)
    # the same workload with the FP64 instances in FP32x2 arithmetic (FP64 storage)
    for op in ops:
        if op.dtype == torch.float64:
            op.set_arithmetic("fp32x2")
    batch_x = Bt.AdvectionBatch(ops)
    batch_x.autotune(sols, Ks, reps=2)
    batch_x.capture_graph(sols, Ks, Ts, times, dts)
    ms_graph_x = timed(batch_x.replay_graph, max(1, args.steps // 2)) / 2
    for op in ops:
        if op.dtype == torch.float64:
            op.set_arithmetic("native")
    peak, peak_kind = measured_peak_hbm()

    def line(ms):
        return {"ms_per_step": round(ms, 3), "gdof_per_s": round(n_total * N_STAGES / (ms / 1e3) / 1e9, 2),
                "hbm_gb_per_s": round(bytes_step / (ms / 1e3) / 1e9, 1)}

    out = {"metric": "batched uneven instances: GDoF/s over 64 seeded 4D/5D problems (rk45, fused)",
           "value": line(ms_graph)["gdof_per_s"], "unit": "GDoF/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms_graph, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "config": {"workload": "64 independent advection problems: dim 4 (2x+2v) or 5 (2x+3v, 3x+2v), degree "
                                  "2..5, cells per dimension 4..12, unit random velocity, FP32 or FP64, periodic "
                                  "unit box, numpy default_rng(0)", "n_dofs_total": n_total,
                      "l2_flush": "inputs larger than L2 (%.1f GB resident)" % (bytes_step / 6 / 1e9)},
           "graph_replay": line(ms_graph),
           "graph_replay_f64_fp32x2": dict(line(ms_graph_x), note="FP64 instances with FP32x2 contractions "
                                           "(hd_adv_set_arithmetic), FP64 storage"),
           "batched_autotuned": line(ms_tuned), "batched_default_tiles":
           line(ms_default), "per_instance_launches": line(ms_single), "autotune_seconds": round(tune_s, 2),
           "classes": classes, "gpu_launches_per_step": launches_per_step,
           "roofline": {"bound": "hbm (FP32 classes) / FP64 pipe (FP64 classes)",
                        "achieved": line(ms_graph)["hbm_gb_per_s"], "peak": peak, "unit": "GB/s",
                        "frac": round(line(ms_graph)["hbm_gb_per_s"] / peak, 4),
                        "peak_source": peak_kind}, "clocks": clocks}
    print(json.dumps(out))
    return 0


def run_adv2d(args):
    """2D (1x+1v) k=3, 32 x 32 cells (16,384 DoFs), velocity (1.0, 0.5), f0 = sin(2 pi x) sin(2 pi v):
    100 fused rk45 steps at CFL 0.2, launched one step at a time and as replays of a recorded
    two-step CUDA graph; the error against the exact translated solution after the steps."""
    import torch

    from hyperdeal_gb300 import advection as A
    from hyperdeal_gb300 import batch as Bt

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    vel = [1.0, 0.5]
    p = A.AdvectionParameters(1, 1, 3, [32], [32], [0.0], [1.0], [0.0], [1.0], vel, dtype="f64")
    op = A.AdvectionOperation(p)
    f0 = A.Function(2, 1.0, omega=[2 * math.pi] * 2, speed=[0.0, 0.0])
    dt = 0.2 * op.critical_time_step() / DEGREE ** 1.5
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nsteps = 100

    def fresh():
        u = op.initialize_dof_vector()
        A.VectorTools.interpolate(op, f0, u, 0.0)
        return u, op.initialize_dof_vector(), op.initialize_dof_vector()

    u, K, T = fresh()
    integ = A.LowStorageRungeKuttaIntegrator(K, T, "rk45")
    for _ in range(args.warmup):
        integ.perform_time_step(u, 0.0, dt, op)
    u, K, T = fresh()
    integ = A.LowStorageRungeKuttaIntegrator(K, T, "rk45")
    torch.cuda.synchronize()
    e0.record(stream)
    for s_ in range(nsteps):
        integ.perform_time_step(u, s_ * dt, dt, op)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_plain = e0.elapsed_time(e1) / nsteps
    exact = A.Function(2, 1.0, omega=[2 * math.pi] * 2, speed=vel)
    _, err_plain = A.VectorTools.norm_and_error(op, exact, u, nsteps * dt)

    ug, Kg, Tg = fresh()
    batch = Bt.AdvectionBatch([op])
    batch.capture_graph([ug], [Kg], [Tg], [0.0], [dt])
    for _ in range(max(1, args.warmup // 2)):  # warm-up replays on a copy, then restart from f0
        batch.replay_graph()
    torch.cuda.synchronize()
    A.VectorTools.interpolate(op, f0, ug, 0.0)
    batch.capture_graph([ug], [Kg], [Tg], [0.0], [dt])
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(nsteps // 2):
        batch.replay_graph()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_graph = e0.elapsed_time(e1) / nsteps
    _, err_graph = A.VectorTools.norm_and_error(op, exact, ug, nsteps * dt)
    n = op.n_dofs
    cpu = None
    if not args.no_cpu:
        # the oracle (CPU restatement, FP64) on the same problem and steps, all host threads
        import numpy as np

        from oracle import oracle as O
        O.build()
        threads = os.cpu_count()
        prob = O.Problem(1, 1, DEGREE, [32, 32], [0.0, 0.0], [1.0, 1.0], vel, n_threads=threads)
        fo = O.make_func(2, 1.0, omega=[2 * math.pi] * 2, speed=[0.0, 0.0])
        uo = O.interpolate(prob, fo)
        Ko, To = np.zeros_like(uo), np.zeros_like(uo)
        c0 = time.perf_counter()
        for s_ in range(nsteps):
            O.lsrk_step(prob, "rk45", uo, s_ * dt, dt, Ko, To)
        cpu_s = (time.perf_counter() - c0) / nsteps
        diff = float(np.abs(uo - ug.cpu().numpy()).max() / np.abs(uo).max())
        cpu = {"value": round(n * N_STAGES / cpu_s / 1e9, 4), "unit": "GDoF/s", "cores": threads, "kind": "port",
               "ms_per_step": round(cpu_s * 1e3, 4), "max_rel_diff_gpu_vs_oracle": diff,
               "sample": "the same 100 rk45 steps by the oracle (CPU restatement, FP64, OpenMP)"}
    out = {"metric": "advection GDoF/s (2D k=3, 32 x 32, FP64) over 100 rk45 steps", "value":
           round(n * N_STAGES / (ms_graph / 1e3) / 1e9, 3), "unit": "GDoF/s", "n_gpus": 1, "steps": nsteps,
           "warmup": args.warmup, "ms_per_step": round(ms_graph, 5), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "2D (1x+1v) upwind DG advection, k=3 Gauss-Lobatto collocation, 32 x 32 cells "
                                  "(16,384 DoFs), periodic unit square, velocity (1.0, 0.5), f0 = sin(2 pi x) "
                                  "sin(2 pi v), 100 rk45 steps at CFL 0.2", "l2_flush": "none (launch-bound size)"},
           "graph_replay": {"ms_per_step": round(ms_graph, 5), "error_vs_exact": err_graph},
           "per_step_launches": {"ms_per_step": round(ms_plain, 5), "error_vs_exact": err_plain,
                                 "gdof_per_s": round(n * N_STAGES / (ms_plain / 1e3) / 1e9, 3)},
           "cpu_baseline": cpu, "gpu_launches": N_STAGES * nsteps + 1}
    print(json.dumps(out))
    return 0


def run_adv4d(args):
    """4D (2x+2v) k=3, 16^2 x 16^2 cells (16,777,216 DoFs), velocity (1.0, 0.7, 0.5, 0.3),
    f0 = prod sin(2 pi coord): fused rk45 steps in FP32 storage (the TMA-pipelined kernel, whose
    unit is one x0-row of 16 cells; the generic kernel beside it) and FP64 storage (generic kernel,
    FP64 and FP32x2 contractions), the FP32 - FP64 difference after the same steps, and the
    oracle's FP64 step time."""
    import numpy as np
    import torch

    from hyperdeal_gb300 import advection as A

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    vel = [1.0, 0.7, 0.5, 0.3]
    k4 = args.adv4d_degree  # 3: the BASELINE configuration; other degrees for the compute-bound check
    f0 = A.Function(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4)
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    res, sols = {}, {}
    clocks = None
    for dtype in ("f32", "f32_generic", "f64", "f64_fp32x2"):
        p = A.AdvectionParameters(2, 2, k4, [16, 16], [16, 16], [0.0] * 2, [1.0] * 2, [0.0] * 2, [1.0] * 2, vel,
                                  dtype=dtype[:3])
        op = A.AdvectionOperation(p)
        if dtype == "f64_fp32x2":
            op.set_arithmetic("fp32x2")
        if dtype == "f32_generic":
            op.set_kernel("generic")
        sol = op.initialize_dof_vector()
        A.VectorTools.interpolate(op, f0, sol, 0.0)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        # the generic kernel's tile, picked outside the timed region (the pipelined kernel has none)
        tuned = None if args.adv4d_default_tile or op.kernel == "pipelined" else op.autotune(sol, Ki, reps=2)
        integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")
        dt = CFL * op.critical_time_step() / k4 ** 1.5
        t = 0.0
        for _ in range(args.warmup):
            integ.perform_time_step(sol, t, dt, op)
            t += dt
        sampler = None
        if dtype == "f32":
            sampler = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
            sampler.start()
            time.sleep(0.3)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            integ.perform_time_step(sol, t, dt, op)
            t += dt
        e1.record(stream)
        torch.cuda.synchronize()
        if sampler is not None:
            clocks = sampler.stop()
        ms = e0.elapsed_time(e1) / args.steps
        S = 4 if dtype == "f32" else 8
        res[dtype] = {"ms_per_step": round(ms, 4), "gdof_per_s": round(op.n_dofs * N_STAGES / (ms / 1e3) / 1e9, 2),
                      "hbm_gb_per_s": round(18 * S * op.n_dofs / (ms / 1e3) / 1e9, 1),
                      "kernel": op.kernel, "tile": op.tile_limits(), "autotuned": tuned}
        sols[dtype] = sol.double()
        n = op.n_dofs
    l2 = float(torch.linalg.vector_norm(sols["f32"] - sols["f64"]) / torch.linalg.vector_norm(sols["f64"]))
    res["f64_fp32x2"]["l2_rel_err_vs_f64"] = float(torch.linalg.vector_norm(sols["f64_fp32x2"] - sols["f64"])
                                                   / torch.linalg.vector_norm(sols["f64"]))
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        prob = O.Problem(2, 2, k4, [16] * 4, [0.0] * 4, [1.0] * 4, vel)
        u = O.interpolate(prob, O.make_func(2, 1.0, omega=[2 * math.pi] * 4, speed=[0.0] * 4))
        c0 = time.perf_counter()
        O.lsrk_step(prob, "rk45", u, 0.0, 1e-4)
        cpu_s = time.perf_counter() - c0
        cpu = {"value": round(n * N_STAGES / cpu_s / 1e9, 4), "unit": "GDoF/s", "cores": os.cpu_count(),
               "kind": "port", "sample": "one rk45 step of the full 16^2 x 16^2 mesh by the oracle (FP64, OpenMP)"}
    peak, peak_kind = measured_peak_hbm()
    out = {"metric": "advection GDoF/s (4D k=%d, 16^2 x 16^2) FP32 and FP64 fused rk45" % k4,
           "value": res["f32"]["gdof_per_s"],
           "unit": "GDoF/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": res["f32"]["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": "4D (2x+2v) upwind DG advection, k=%d Gauss-Lobatto collocation, 16^2 x 16^2 cells "
                                  "(65,536 cells, %d DoFs), periodic unit box, velocity (1.0, 0.7, 0.5, 0.3), "
                                  "f0 = prod sin(2 pi coord), fused rk45, CFL 0.2" % (k4, n),
                      "l2_flush": "none: %d MB per FP32 vector (3 vectors > 129 MB L2)" % (4 * n // 10 ** 6)},
           "f32": res["f32"], "f32_generic": res["f32_generic"], "f64": res["f64"], "f64_fp32x2": res["f64_fp32x2"],
           "l2_rel_err_f32_vs_f64": l2,
           "roofline": {"bound": "hbm", "achieved": res["f32"]["hbm_gb_per_s"], "peak": peak, "unit": "GB/s",
                        "frac": round(res["f32"]["hbm_gb_per_s"] / peak, 4), "peak_source": peak_kind},
           "cpu_baseline": cpu, "clocks": clocks, "gpu_launches": N_STAGES * args.steps,
           "kernel": ("hd::ecl6_kernel<stage, 4> (persistent, TMA-pipelined, units of 16 cells)"
                      if res["f32"]["kernel"] == "pipelined" else "hd::ecl_kernel<4,4,float,stage> (generic)")}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--steps-f64", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--l2-steps", type=int, default=20,
                    help="rk45 steps after which the FP32 and FP64 forms are compared (default 20)")
    ap.add_argument("--apply-reps", type=int, default=20, help="timed applies of the per-apply line (0: none)")
    ap.add_argument("--backend", default="nccl", choices=["nccl", "gloo"],
                    help="torch.distributed backend of the ghost-face exchange for --gpus N > 1 (gloo stages the "
                         "faces through host memory)")
    ap.add_argument("--cells-x", type=int, default=CELLS,
                    help="x-cells per direction (8 = the benchmark workload; smaller only for profiling)")
    ap.add_argument("--workload", default="advection6d",
                    choices=["advection6d", "adv2d", "adv4d", "vp2x2v", "batch64"])
    ap.add_argument("--adv4d-degree", type=int, default=3, help="degree of the adv4d workload (default 3)")
    ap.add_argument("--adv4d-default-tile", action="store_true",
                    help="adv4d: keep the default tile instead of picking it with hd_adv_autotune")
    ap.add_argument("--vp-tol", type=float, default=1e-10, help="CG: ||r|| <= tol ||rhs|| (vp2x2v)")
    ap.add_argument("--vp-oracle-steps", type=int, default=2, help="steps compared with the FP64 oracle (vp2x2v)")
    ap.add_argument("--vp-runs", default="f64/previous,f64/zero,f64/learned,f64/learned_adam,f64/previous_noprecond,"
                                         "f64/zero_noprecond,f64/learned_noprecond,f64x/previous,f64x/zero,"
                                         "f64x/learned,f32/previous,f32/zero,f32/learned,f32/previous_noprecond,"
                                         "f32/zero_noprecond,f32/learned_noprecond,f64/direct,f64x/direct,f32/direct",
                    help="dtype/guess combinations timed (vp2x2v; _noprecond: CG without the preconditioner; "
                         "direct: the pseudo-inverse instead of CG)")
    ap.add_argument("--vp-precond", default="block_jacobi", choices=["block_jacobi", "none"],
                    help="preconditioner of the Poisson CG (vp2x2v)")
    args = ap.parse_args()
    if args.workload == "vp2x2v":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the Vlasov-Poisson line is reported by the "
                              "default arm (oracle host time in field_energy_vs_oracle)"}))
            return 0
        return run_vp(args)
    if args.workload == "adv2d":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the 2D line is reported by the default arm"}))
            return 0
        return run_adv2d(args)
    if args.workload == "adv4d":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the 4D line is reported by the default arm"}))
            return 0
        return run_adv4d(args)
    if args.workload == "batch64":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "the batched line is reported by the default arm"}))
            return 0
        return run_batch(args)
    args.steps_cpu = 3
    args.warmup_cpu = 1
    if args.impl == "reference":
        return run_reference(args)

    import numpy as np
    import torch

    from hyperdeal_gb300 import advection as A

    from hyperdeal_gb300.replicas import Replicas, time_steps, whole_job_rate

    rep = Replicas(args.backend)
    world, rank, local = rep.world, rep.rank, rep.local_rank
    torch.cuda.set_device(local % torch.cuda.device_count())
    dist = rep.dist

    def make_params(dtype, layers_v2=CELLS):
        # N > 1: the v2 direction is extended to N x 8 layers (h unchanged), one v-slab of 8 layers per rank
        return A.AdvectionParameters(DIM_X, DIM_V, DEGREE, [args.cells_x] * 3, [CELLS, CELLS, layers_v2],
                                     [0.0] * 3, [1.0] * 3, [0.0] * 3, [1.0, 1.0, layers_v2 / CELLS], VELOCITY,
                                     dtype=dtype)

    def make_op(dtype):
        return A.AdvectionOperation(make_params(dtype))

    rng = np.random.default_rng(0)
    phi = list(rng.uniform(0, 2 * math.pi, 6))
    f0 = A.Function(2, 1.0, omega=[2 * math.pi] * 6, speed=[0.0] * 6, phase=phi)

    stream = torch.cuda.current_stream()
    if world > 1:
        # weak scaling over v-slabs: rank r owns layers [8r, 8r + 8) of v2; the upwind v2 faces of its
        # first layer come from rank r - 1 before every stage (NCCL point-to-point, overlapped with the
        # interior cells)
        from hyperdeal_gb300 import partition as Pt
        op = Pt.PartitionedAdvectionOperation(make_params("f32", CELLS * world), world, rank)
        exchange = Pt.DistributedExchange(op)
        sol = op.initialize_dof_vector()
        op.interpolate(f0, sol, 0.0)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")

        def advance(t_):
            op.perform_time_step(integ, sol, t_, dt, exchange)
    else:
        op = make_op("f32")
        sol = op.initialize_dof_vector()
        A.VectorTools.interpolate(op, f0, sol, 0.0)
        Ki, Ti = op.initialize_dof_vector(), op.initialize_dof_vector()
        integ = A.LowStorageRungeKuttaIntegrator(Ki, Ti, "rk45")

        def advance(t_):
            integ.perform_time_step(sol, t_, dt, op)
    n = op.n_dofs
    dt = CFL * op.critical_time_step() / DEGREE ** 1.5
    t = 0.0
    for _ in range(args.warmup):
        advance(t)
        t += dt
    torch.cuda.synchronize()
    rep.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    tt = {"t": t}

    def one_step():
        advance(tt["t"])
        tt["t"] += dt

    def cuda_clock():
        def start():
            e0.record(stream)

        def stop():
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1)
        return start, stop

    # barrier + synchronisation on both sides, max over ranks (replicas: no collective on the data path)
    ms_step = time_steps(rep, one_step, args.steps, 0, torch.cuda.synchronize, cuda_clock)
    t = tt["t"]
    clocks = sampler.stop()
    value = whole_job_rate(n * N_STAGES, world, ms_step) / 1e9

    # roofline of the dominant kernel (the fused stage kernel, 5 launches per step)
    peak, peak_kind = measured_peak_hbm()
    bytes_per_launch = PASSES_PER_STEP / N_STAGES * 4 * n
    achieved = bytes_per_launch / (ms_step / N_STAGES / 1e3) / 1e9
    traffic = profiled_traffic()
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else "fallback",
                "bytes_per_launch": bytes_per_launch,
                "kernel": ("hd::ecl6_kernel<stage> (persistent, TMA-pipelined)" if op.kernel == "pipelined"
                           else "hd::ecl_kernel<6,4,float,stage> (generic)")}

    # per-apply figures (the reference's operator benchmark, performance/operators_advection_01.likwid.cc:
    # 341-348: DoFs * applies / time): src read, dst written, 2 S N algorithmic bytes per apply
    def time_applies(o, src, reps):
        dst = o.initialize_dof_vector()
        for _ in range(2):
            o.apply(dst, src, 0.0)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            o.apply(dst, src, 0.0)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        S = 4 if o.dtype == torch.float32 else 8
        gbs = 2 * S * o.n_dofs / (ms / 1e3) / 1e9
        del dst
        return {"ms_per_apply": round(ms, 4), "gdof_per_s": round(o.n_dofs / (ms / 1e3) / 1e9, 3),
                "hbm_gb_per_s": round(gbs, 1), "frac": round(gbs / measured_peak_hbm()[0], 4), "applies": reps}

    apply_lines = {}
    if world == 1 and args.apply_reps > 0:
        apply_lines["f32"] = dict(time_applies(op, sol, args.apply_reps),
                                  kernel="hd::ecl6_kernel<kApply>" if op.kernel == "pipelined" else "generic")
        torch.cuda.empty_cache()

    # FP64 form of the same steps, and the L2 difference of the two solutions
    f64 = {}
    l2 = None
    if args.steps_f64 > 0 and world == 1:
        op64 = make_op("f64")
        s64 = op64.initialize_dof_vector()
        A.VectorTools.interpolate(op64, f0, s64, 0.0)
        K64, T64 = op64.initialize_dof_vector(), op64.initialize_dof_vector()
        i64 = A.LowStorageRungeKuttaIntegrator(K64, T64, "rk45")
        t64 = 0.0
        for _ in range(args.warmup):
            i64.perform_time_step(s64, t64, dt, op64)
            t64 += dt
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps_f64):
            i64.perform_time_step(s64, t64, dt, op64)
            t64 += dt
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1) / args.steps_f64
        v64 = n * N_STAGES / (ms64 / 1e3) / 1e9
        f64 = {"value": round(v64, 3), "ms_per_step": round(ms64, 3), "steps": args.steps_f64,
               "arithmetic": "native FP64"}
        # the FP64-storage form with double-word FP32 contractions (hd_adv_set_arithmetic FP32X2)
        op64.set_arithmetic("fp32x2")
        for _ in range(args.warmup):
            i64.perform_time_step(s64, t64, dt, op64)
            t64 += dt
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps_f64):
            i64.perform_time_step(s64, t64, dt, op64)
            t64 += dt
        e1.record(stream)
        torch.cuda.synchronize()
        msx = e0.elapsed_time(e1) / args.steps_f64
        f64x = {"value": round(n * N_STAGES / (msx / 1e3) / 1e9, 3), "ms_per_step": round(msx, 3),
                "steps": args.steps_f64, "arithmetic": "FP32x2 (double-word FP32) contractions, FP64 storage"}
        if args.apply_reps > 0:
            reps64 = max(2, args.apply_reps // 10)
            apply_lines["f64_fp32x2"] = time_applies(op64, s64, reps64)
            op64.set_arithmetic("native")
            apply_lines["f64"] = time_applies(op64, s64, reps64)
            op64.set_arithmetic("fp32x2")
        # the same number of steps from the same initial data in the three forms
        s32 = op.initialize_dof_vector()
        A.VectorTools.interpolate(op, f0, s32, 0.0)
        s64b = op64.initialize_dof_vector()
        A.VectorTools.interpolate(op64, f0, s64b, 0.0)
        s64x = s64b.clone()
        nsteps = args.l2_steps
        tt = 0.0
        for _ in range(nsteps):
            integ.perform_time_step(s32, tt, dt, op)
            op64.set_arithmetic("native")
            i64.perform_time_step(s64b, tt, dt, op64)
            op64.set_arithmetic("fp32x2")
            i64.perform_time_step(s64x, tt, dt, op64)
            tt += dt
        d = (s32.double() - s64b)
        l2 = float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(s64b))
        f64["l2_compared_after_steps"] = nsteps
        f64x["l2_rel_err_vs_f64"] = float(torch.linalg.vector_norm(s64x - s64b) / torch.linalg.vector_norm(s64b))
        f64x["max_rel_err_vs_f64"] = float((s64x - s64b).abs().max() / s64b.abs().max())
        f64["fp32x2"] = f64x
        del op64, s64, K64, T64, i64, s64b, s64x, d, s32
        torch.cuda.empty_cache()

    # end to end through the public API with host buffers: every step copies a state from pinned
    # host memory, runs one fused step through the C ABI (hd_lsrk_step) and copies the result back.
    # Sequential: one stream.  Pipelined: independent states (an ensemble), three buffer triples,
    # H2D / compute / D2H on three streams so that the copies of neighbouring steps overlap the
    # step in between (both copy directions run concurrently over the host link).
    e2e = None
    if not args.no_e2e and world > 1:
        # N ranks: each rank's part through the partitioned public API, its state copied in from pinned
        # host memory and back every step (H2D, step with the ghost exchanges, D2H on one stream)
        host_in = torch.empty(n, dtype=torch.float32, pin_memory=True)
        host_in.copy_(op.owned(sol))
        host_out = torch.empty(n, dtype=torch.float32, pin_memory=True)
        k_e2e = max(4, min(args.steps, 8))

        def e2e_step():
            op.owned(sol).copy_(host_in, non_blocking=True)
            advance(t)
            host_out.copy_(op.owned(sol), non_blocking=True)

        ms_seq = time_steps(rep, e2e_step, k_e2e, 2, torch.cuda.synchronize, cuda_clock)
        e2e = {"value": round(world * n * N_STAGES / (ms_seq / 1e3) / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n, "ms_per_step": round(ms_seq, 3),
               "steps": k_e2e, "path": "PartitionedAdvectionOperation.perform_time_step (C ABI stages, NCCL "
                                       "ghost exchange) on each rank's part copied in from and out to pinned "
                                       "host memory every step; per-rank bytes"}
        del host_in, host_out
    if not args.no_e2e and world == 1:
        import ctypes

        from hyperdeal_gb300 import _lib as hdl
        L = hdl.load()
        host_in = torch.empty(n, dtype=torch.float32, pin_memory=True)
        host_in.copy_(sol)
        host_out = torch.empty(n, dtype=torch.float32, pin_memory=True)
        k_e2e = max(4, min(args.steps, 8))
        for _ in range(2):
            sol.copy_(host_in, non_blocking=True)
            integ.perform_time_step(sol, t, dt, op)
            host_out.copy_(sol, non_blocking=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(k_e2e):
            sol.copy_(host_in, non_blocking=True)
            integ.perform_time_step(sol, t, dt, op)
            host_out.copy_(sol, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize()
        ms_seq = e0.elapsed_time(e1) / k_e2e

        NT = 3
        triples = [(sol, Ki, Ti)] + [tuple(op.initialize_dof_vector() for _ in range(3)) for _ in range(NT - 1)]
        s_in, s_c, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        ev_h2d = [torch.cuda.Event() for _ in range(NT)]
        ev_step = [torch.cuda.Event() for _ in range(NT)]
        ev_d2h = [torch.cuda.Event() for _ in range(NT)]
        used = [False] * NT

        def pipelined_step(k):
            j = k % NT
            tri = triples[j]
            if used[j]:
                s_in.wait_event(ev_d2h[j])
            used[j] = True
            with torch.cuda.stream(s_in):
                tri[0].copy_(host_in, non_blocking=True)
                ev_h2d[j].record(s_in)
            s_c.wait_event(ev_h2d[j])
            X = [ctypes.c_void_p(v.data_ptr()) for v in tri]
            hdl.check(L.hd_lsrk_step(op.handle, integ._h, ctypes.byref(X[0]), ctypes.byref(X[1]),
                                     ctypes.byref(X[2]), ctypes.c_double(t), ctypes.c_double(dt),
                                     ctypes.c_void_p(s_c.cuda_stream)))
            ev_step[j].record(s_c)
            res = next(v for v in tri if v.data_ptr() == X[0].value)
            s_out.wait_event(ev_step[j])
            with torch.cuda.stream(s_out):
                host_out.copy_(res, non_blocking=True)
                ev_d2h[j].record(s_out)

        for k in range(NT):
            pipelined_step(k)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(stream)
        for sx in (s_in, s_c, s_out):
            sx.wait_event(p0)
        for k in range(k_e2e):
            pipelined_step(k)
        stream.wait_stream(s_out)
        p1.record(stream)
        torch.cuda.synchronize()
        ms_pipe = p0.elapsed_time(p1) / k_e2e
        e2e = {"value": round(world * n * N_STAGES / (ms_pipe / 1e3) / 1e9, 3), "unit": UNIT,
               "h2d_bytes_per_step": 4 * n, "d2h_bytes_per_step": 4 * n, "ms_per_step": round(ms_pipe, 3),
               "steps": k_e2e,
               "path": "hd_lsrk_step (C ABI) on states copied in from pinned host memory and back every step; "
                       "independent states, copies of neighbouring steps overlapped with the step (3 streams, "
                       "3 buffer triples)",
               "sequential": {"value": round(world * n * N_STAGES / (ms_seq / 1e3) / 1e9, 3),
                              "ms_per_step": round(ms_seq, 3), "path": "H2D, step, D2H on one stream"}}
        del host_in, host_out, triples
        torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_sample()

    if rank == 0:
        out = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": workload_config({"parallelism": ("v-slabs: %d ranks x 8 layers of v2, one NCCL ghost-face "
                                                          "exchange per stage" % world) if world > 1
                                          else "single GPU",
                                          **({} if args.cells_x == CELLS else
                                             {"profiling_case_cells": "%d^3 x 8^3" % args.cells_x,
                                              "n_dofs": n})}),
               "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
               # per stage: the stage kernel; with N ranks also the face pack and the boundary-layer launch
               "gpu_launches": N_STAGES * args.steps * (3 if world > 1 else 1),
               "f64_form": f64, "f32_over_f64": round(value / f64["value"], 3) if f64 else None,
               "l2_rel_err_f32_vs_f64": l2, "apply": apply_lines or None}
        print(json.dumps(out))
    rep.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
