#!/usr/bin/env python
"""Benchmark of the hydro time-step hot path on GB300.

Workload: 3D rising drops at 192^3 (unit cube, ambient rho 10 / drops rho 1,
mu 1e-2, g = -1 along z, 1-8 seeded drops), FP64, a pinned number of SIMPLE
iterations per step (both arms do the same work per step), pressure solve to
relative residual 1e-8, TVD advection of both phases, property update.
Synthetic seeded inputs of that shape (no external data).

Metric: Mcell-updates/s = cells x time steps / wall seconds, whole job.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form mixed_mg|fp64|fp64_mg]
                  [--no-plain] [--no-cpu-baseline]
  python bench.py --impl reference ...   # the reference algorithm on the CPU

The headline form is "mixed_mg": FP32 assembly and momentum sweeps (FP64
kept where the arithmetic cancels) and FP64 iterative refinement around an
FP32 conjugate-gradient pressure solve preconditioned by geometric multigrid.
Timed beside it in the same run unless --no-plain is given: the plain FP64
form ("plain_fp64": every kernel FP64, Jacobi-preconditioned CG) and the FP64
form with the multigrid-preconditioned refinement ("fp64_multigrid": FP64
kernels and system, FP32 inner corrections).

Multi-GPU: replicas only (the reference's MPI mode runs redundant replicas;
the path has no exchange step here) -- each rank advances its own seeded
case, time is the max over ranks, value the cells x steps of all ranks.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic (compulsory) bytes per cell of one launch of each kernel group,
# FP64 path, 3D: each distinct input read once, each output written once;
# face arrays count ~1 entry per cell per direction.
ALG_BYTES_PER_CELL_FP64 = {
    "cg_spmv": 8 * (1 + 3 + 1 + 1),        # read p, kf[3], diag; write Ap
    "cg_update": 8 * (5 + 3),              # read x, r, p, Ap, 1/diag; write x, r, z
    "cg_dir": 8 * (2 + 1),                 # read z, p; write p
    "mom_sweep": 8 * (7 + 3 + 3 + 3),      # read coef[7], res[3], du[3]; write du[3]
    "mom_assemble": 8 * (26 + 11),         # read u,utc,utp,G[9],F[3],rho,mu,fo[3]; write coef[7],res[3],Dc
    "force": 8 * (3 + 9 + 1 + 1 + 3 + 3 + 6),  # read u,G,p,mu,force,stforce; write fo,fres
    "vel_grad": 8 * (3 + 9),
    "rhie_chow": 8 * (6 + 1 + 6 + 1 + 6),  # read u,du,p,force,fres,Dc; write Fs[3], kf[3]
    "correct": 8 * (6 + 2 + 1 + 1 + 6 + 3 + 1 + 3),  # read u,du,p,pc,Dc,Fs,kf; write u,p,F
    "adv_faces": 8 * (2 + 3 + 6),          # read q[2], F[3]; write qflux[2x3]
    "adv_update": 8 * (2 + 6 + 2),
}
# FP32 inner solve of the mixed path (vectors 4 B)
ALG_BYTES_PER_CELL_FP32 = {
    "cg_spmv": 4 * (6 + 2),                # read z, p_old, kf[3], diag; write p_new, Ap
    "cg_update": 4 * (4 + 2),              # read x, r, p, Ap; write x, r
    "mom_sweep": 4 * (10 + 3 + 3),         # read coef[7]+res[3], du[3]; write du[3]
    "mg_vcycle": None,                     # below
}
# One V-cycle, bytes per cell of the finest level.  Finest level (colour-
# blocked, FP16 couplings): a half-sweep reads the couplings (3 faces x 2 B
# per cell) and, on half of the cells each, its own colour's b and 1/diag,
# the other colour's x, and writes its own x: 6 + 4 x 2 = 14 B; the first
# (black) one also carries the red one from zero (reads the red b and
# 1/diag instead of x, writes the red x: +4 B), the first post-smoothing
# one reads the coarse correction (+0.5 B); 3 + 4 half-sweeps; restriction:
# red b and x, black x, couplings, coarse b and x written = 13 B.  Coarser
# levels (FP32 couplings 12 B per cell): 7 half-sweeps of 20 B, restriction
# 21 B, prolongation 0.5 B per cell of the level, summed over the levels
# (1/8 + 1/64 + ...) of the finest level's cells.
_FINE = (14 + 4) + 14 + 14 + (14 + 0.5) + 3 * 14 + 13
_COARSE = 7 * 20 + 21 + 0.5
ALG_BYTES_PER_CELL_FP32["mg_vcycle"] = int(round(_FINE + _COARSE * (1 / 7)))


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason sampling during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(n, seed, precision, outer, solver="cg"):
    from hydro_gb300 import capi, cases
    d, u0, q0, drops = cases.rising_drops(n=n, seed=seed, dt_max=2e-3)
    d.convergence_tolerance = 0.0
    d.num_iterations_limit = outer
    d.velocity_solver = capi.LINEAR_GAUSS_SEIDEL  # red-black on the GPU
    d.velocity_tolerance = 1e-8
    d.velocity_iters_limit = 200
    d.pressure_tolerance = 1e-8
    d.pressure_iters_limit = 20000
    d.precision = capi.MIXED if precision == "mixed" else capi.FP64
    d.pressure_solver = capi.LINEAR_MGCG if solver == "mgcg" else capi.LINEAR_CG
    return d, u0, q0, drops


def init_dist():
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, world):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ----------------------------------------------------------- CPU baseline --
def init_case(solver, d, u0, q0):
    """Initial state of the workload on any solver (GPU context or CPU
    oracle): velocity at rest, partial densities, initial fluxes and
    properties, then the pressure in hydrostatic balance with the density
    the solver computed (both time layers)."""
    from hydro_gb300 import capi, cases
    solver.set_field(capi.F_VELOCITY, u0)
    solver.set_field(capi.F_PARTIAL_DENSITY, q0)
    solver.init_state()
    p0 = cases.hydrostatic_pressure(d, solver.get_field(capi.F_DENSITY))
    for layer in (capi.TIME_CURR, capi.TIME_PREV):
        solver.set_field(capi.F_PRESSURE, p0, layer)
    return solver


REFERENCE_SOLVERS = ("velocity: one LU sweep (linear.hpp:527-567); pressure: Gauss-Seidel/SOR "
                     "omega 1.9 to a max update of 1e-3, at most 1000 sweeps "
                     "(linear.hpp:671-716; examples/general.hydroconf:112-116)")


def cpu_steps(n, seed, outer, budget_s, max_steps, threads=None):
    """The reference algorithm on the host cores: the CPU oracle port (plain-C
    restatement of FluidSimple + AdvectionSolverMultiExplicit + the property
    update) with the reference's default linear solvers, from the workload's
    initial state.  Complete time steps are timed one by one -- every SOR
    sweep actually run, nothing extrapolated -- until max_steps steps or
    budget_s seconds; at least one step."""
    from hydro_gb300 import capi
    from oracle.oracle import Oracle
    threads = threads or os.cpu_count() or 1
    d, u0, q0, _ = workload(n, seed, "fp64", outer)
    d.velocity_solver = capi.LINEAR_LU
    d.pressure_solver = capi.LINEAR_GAUSS_SEIDEL
    d.pressure_omega = 1.9
    d.pressure_tolerance = 1e-3
    d.pressure_iters_limit = 1000
    o = init_case(Oracle(d, threads=threads), d, u0, q0)
    times, sweeps = [], []
    t_start = time.perf_counter()
    while len(times) < max(1, max_steps):
        t0 = time.perf_counter()
        st = o.step()
        times.append(time.perf_counter() - t0)
        sweeps.append(st["pressure_iterations"])
        if time.perf_counter() - t_start > budget_s:
            break
    total = sum(times)
    ncells = n ** 3
    return {
        "value": ncells * len(times) / total / 1e6,
        "unit": "Mcell-updates/s",
        "cores": threads,
        "kind": "port",
        "steps_timed": len(times),
        "seconds_per_step": total / len(times),
        "step_seconds": [round(t, 2) for t in times],
        "sor_sweeps_per_step": sweeps,
        "sample": ("oracle (C restatement of the reference) at %d^3, %d SIMPLE iterations per "
                   "step, %s; %d complete time steps from the workload's initial state timed "
                   "in full (%s s), SOR sweeps per step %s" % (
                       n, outer, REFERENCE_SOLVERS, len(times),
                       ", ".join("%.1f" % t for t in times), sweeps)),
    }


# ---------------------------------------------------------------- our arm --
def measure(args, form, rank, world, local, stream, e2e=True):
    """Times args.steps steps of one form ("mixed_mg": mixed precision with
    the multigrid CG, "fp64": plain FP64 with Jacobi CG, "fp64_mg": FP64
    with the multigrid-preconditioned refinement) after args.warmup untimed
    steps; returns a dict of results."""
    import numpy as np
    import torch

    from hydro_gb300 import capi
    from hydro_gb300 import solver as S

    precision, solver = {"mixed_mg": ("mixed", "mgcg"), "fp64": ("fp64", "cg"),
                         "fp64_mg": ("fp64", "mgcg"),
                         "learned_mixed_mg": ("mixed", "mgcg")}[form]
    d, u0, q0, drops = workload(args.n, args.seed + rank, precision, args.outer, solver)
    h = init_case(S.Hydro(d, stream=stream.cuda_stream), d, u0, q0)
    net = None
    if form.startswith("learned"):
        from hydro_gb300.net import Net, attach
        from hydro_gb300.train_guess import RHO_SCALE
        if not os.path.exists(args.weights_file):
            raise RuntimeError("learned form: no trained weights at %s (train them with "
                               "python -m hydro_gb300.train_guess)" % args.weights_file)
        net = Net((args.n,) * 3, batch=1)
        net.load(args.weights_file)
        attach(h, net, args.guess_iterations, RHO_SCALE)
    N = d.ncells
    for _ in range(args.warmup):
        h.step()
    h.reset_profile()
    h.set_profiling(True)
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = S.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    stats = [h.step() for _ in range(args.steps)]
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    launches = S.launch_count() - l0
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    prof = h.profile()
    h.set_profiling(False)
    guess = None
    if net is not None:
        from hydro_gb300.net import guess_stats
        used, dropped, skipped = guess_stats(h)
        pms, plaunch = net.last_predict()
        guess = {"used": used, "dropped": dropped, "skipped_steps": skipped,
                 "predict_ms": round(pms, 4),
                 "predict_launches": plaunch, "iterations_guessed": args.guess_iterations}
    ms_max = max_over_ranks(ms, world)
    out = {"form": form, "precision": precision, "solver": solver, "N": N, "drops": len(drops),
           "guess": guess,
           "ms": ms_max, "value": world * N * args.steps / (ms_max / 1e3) / 1e6,
           "launches": launches, "clocks": clk, "stats": stats, "prof": prof, "desc": d}
    if e2e:
        # the same steps as one CUDA-graph launch each (hydro_gpu_step_graph,
        # loops steered on the device); no per-group events inside the graph
        h.step_graph()  # capture
        barrier(world)
        torch.cuda.synchronize()
        g0 = S.launch_count()
        e0.record(stream)
        gstats = [h.step_graph() for _ in range(args.steps)]
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(world)
        gms = max_over_ranks(e0.elapsed_time(e1), world)
        out["graph"] = {"ms": gms, "value": world * N * args.steps / (gms / 1e3) / 1e6,
                        "stats": gstats, "launches": S.launch_count() - g0}
        # through the public C-ABI with host buffers (the graph-captured step):
        # every step uploads the state from pinned host memory and reads the
        # result back
        nph = d.num_phases
        pin_u = torch.empty(N * d.dim, dtype=torch.float64, pin_memory=True).numpy()
        pin_q = torch.empty(N * nph, dtype=torch.float64, pin_memory=True).numpy()
        pin_p = torch.empty(N, dtype=torch.float64, pin_memory=True).numpy()
        pin_u[:] = h.get_field(capi.F_VELOCITY)
        pin_q[:] = h.get_field(capi.F_PARTIAL_DENSITY)
        lib = capi.load()
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            lib.hydro_gpu_set_field(h.ctx, capi.F_VELOCITY, capi.TIME_CURR, dp(pin_u), pin_u.size)
            lib.hydro_gpu_set_field(h.ctx, capi.F_PARTIAL_DENSITY, capi.TIME_CURR, dp(pin_q),
                                    pin_q.size)
            h.step_graph()
            lib.hydro_gpu_get_field(h.ctx, capi.F_VELOCITY, capi.TIME_CURR, dp(pin_u), pin_u.size)
            lib.hydro_gpu_get_field(h.ctx, capi.F_PRESSURE, capi.TIME_CURR, dp(pin_p), pin_p.size)
            lib.hydro_gpu_get_field(h.ctx, capi.F_PARTIAL_DENSITY, capi.TIME_CURR, dp(pin_q),
                                    pin_q.size)
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0, world)
        out["e2e"] = {"value": round(world * N * args.steps / e2e_s / 1e6, 4),
                      "unit": "Mcell-updates/s", "api": "hydro_gpu_step_graph",
                      "h2d_bytes_per_step": (d.dim + nph) * N * 8,
                      "d2h_bytes_per_step": (d.dim + 1 + nph) * N * 8}
    h.close()
    if net is not None:
        net.close()
    return out


# DRAM traffic (ncu dram__bytes_read.sum + dram__bytes_write.sum) per cell of
# one launch of a group, measured on smaller cases of the same workload
# (rising drops, cold cache as ncu replays it) and applied per cell:
#   mg_vcycle: one V-cycle at 160^3, summed over per-kernel captures (one
#              kernel and at most three launches each): 521.0 MB -> 127.2 B/cell
#   cg_spmv:   k_cg_spmv<3, double> at 150^3: 134.9 + 16.0 MB -> 44.7 B/cell
TRAFFIC_PER_CELL = {"mg_vcycle": 521.0e6 / 160 ** 3, "cg_spmv": 150.9e6 / 150 ** 3}


def roofline(res):
    """Roofline figure of the dominant kernel group of one measured form."""
    peak, peak_kind = measured_peaks()
    prof, stats, N = res["prof"], res["stats"], res["N"]
    if not prof:
        return None
    name, (nl, tms) = max(prof.items(), key=lambda kv: kv[1][1])
    table = dict(ALG_BYTES_PER_CELL_FP64)
    if res["precision"] == "mixed":
        table.update(ALG_BYTES_PER_CELL_FP32)
    per_cell = table.get(name)
    if not per_cell:
        return {"bound": "hbm", "kernel": name, "achieved": None, "peak": peak, "unit": "GB/s",
                "frac": None, "traffic": None}
    eff = nl
    if name in ("cg_spmv", "cg_update", "cg_dir"):
        eff = sum(s["pressure_iterations"] for s in stats)
    elif name == "mom_sweep":
        eff = sum(s["velocity_sweeps"] for s in stats)
    bytes_launch = per_cell * N
    achieved = bytes_launch * eff / (tms / 1e3) / 1e9
    tpc = TRAFFIC_PER_CELL.get(name)
    return {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak,
            "unit": "GB/s", "frac": round(achieved / peak, 4),
            "traffic": round(tpc * N) if tpc else None,
            "peak_source": peak_kind, "bytes_per_launch": bytes_launch, "launches": nl,
            "effective_launches": eff, "avg_launch_us": round(tms * 1e3 / max(eff, 1), 2)}


def gpu_local_cpus(local):
    """CPUs attached to the GPU's PCI root (sysfs local_cpulist), or None."""
    try:
        import torch
        prop = torch.cuda.get_device_properties(local)
        dom = getattr(prop, "pci_domain_id", 0)
        bus, dev = getattr(prop, "pci_bus_id"), getattr(prop, "pci_device_id")
        path = "/sys/bus/pci/devices/%04x:%02x:%02x.0/local_cpulist" % (dom, bus, dev)
        with open(path) as f:
            text = f.read().strip()
        cpus = set()
        for part in text.split(","):
            if "-" in part:
                a, b = part.split("-")
                cpus.update(range(int(a), int(b) + 1))
            elif part:
                cpus.add(int(part))
        return cpus or None
    except Exception:
        return None


def run_ours(args, rank, world, local):
    import torch

    from hydro_gb300 import capi

    torch.cuda.set_device(local)
    # host threads and the pinned host buffers of the end-to-end leg on the
    # GPU's own NUMA node (first touch), when sysfs says which CPUs those are
    cpus = gpu_local_cpus(local)
    avail = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") else None
    if cpus and avail and cpus & avail and cpus & avail != avail:
        try:
            os.sched_setaffinity(0, cpus & avail)
        except OSError:
            pass
    try:
        capi.load()
    except RuntimeError:
        from hydro_gb300 import build
        build.build_library()
        capi.load()
    stream = torch.cuda.Stream()
    head = measure(args, args.form, rank, world, local, stream)
    plain = None
    fp64mg = None
    mixed = None
    if args.form.startswith("learned") and not args.no_plain:
        # the same form without the network: what the learned guess gains
        mixed = measure(args, "mixed_mg", rank, world, local, stream, e2e=False)
    if args.form != "fp64" and not args.no_plain:
        plain = measure(args, "fp64", rank, world, local, stream, e2e=False)
        if args.form != "fp64_mg":
            fp64mg = measure(args, "fp64_mg", rank, world, local, stream, e2e=False)
    if avail:
        try:
            os.sched_setaffinity(0, avail)  # the CPU baseline uses every host core
        except OSError:
            pass
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_steps(args.n, args.seed, args.outer, args.cpu_budget, 1)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"error": str(e)}
    if rank != 0:
        return
    stats = head["stats"]
    N = head["N"]
    out = {
        "metric": "Mcell-updates/s",
        "value": round(head["value"], 4),
        "unit": "Mcell-updates/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(head["ms"] / args.steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64+f32" if head["precision"] == "mixed" else "f64",
        "data": "synthetic: seeded rising drops (%d drops), no external data" % head["drops"],
        "config": {
            "workload": "rising_drops_%d^3" % args.n,
            "step": "host-driven (hydro_gpu_step), per-group CUDA events on",
            "cells": N,
            "form": head["form"],
            "precision": head["precision"],
            "pressure_solver": head["solver"],
            "simple_iterations_per_step": args.outer,
            "pressure_residual": 1e-8,
            "seed": args.seed,
            "initial_state": "rest, hydrostatic pressure",
            "linear_solvers": "velocity: red-black Gauss-Seidel to a max update of 1e-8 "
                              "(<= 200 sweeps); pressure: CG to relative residual 1e-8",
            "parallelism": "replicas" if world > 1 else "single",
            "l2": "inputs larger than L2: working set %.1f GB > 129 MB" % (N * 8 * 80 / 1e9),
        },
        "e2e": head.get("e2e"),
        "gpu_launches": head["launches"],
        "roofline": roofline(head),
        "clocks": head["clocks"],
        "cpu_baseline": cpu,
        "step_stats": {
            "outer_iterations": [s["outer_iterations"] for s in stats],
            "pressure_iterations": [s["pressure_iterations"] for s in stats],
            "velocity_sweeps": [s["velocity_sweeps"] for s in stats],
            "pressure_residual_max": max(s["pressure_residual"] for s in stats),
            "dt": stats[-1]["dt"],
        },
        "profile_ms": {k: round(v[1], 3) for k, v in sorted(head["prof"].items())},
        "graph_step": {
            "value": round(head["graph"]["value"], 4),
            "ms_per_step": round(head["graph"]["ms"] / args.steps, 3),
            "api": "hydro_gpu_step_graph",
            "note": "same steps, one CUDA-graph launch per step; value above is the "
                    "host-driven step with per-group CUDA events (roofline source)",
            "pressure_iterations": [s["pressure_iterations"] for s in head["graph"]["stats"]],
            "gpu_launches": head["graph"]["launches"],
        },
    }
    if head.get("guess"):
        out["learned_guess"] = dict(head["guess"])
        out["learned_guess"]["weights"] = os.path.relpath(args.weights_file, ROOT)
    if mixed:
        out["mixed_multigrid"] = {
            "value": round(mixed["value"], 4),
            "ms_per_step": round(mixed["ms"] / args.steps, 3),
            "pressure_iterations": [s["pressure_iterations"] for s in mixed["stats"]],
            "speedup_of_headline": round(head["value"] / mixed["value"], 3),
            "note": "the headline form without the learned guess: what the network gains",
            "clocks": mixed["clocks"],
            "profile_ms": {k: round(v[1], 3) for k, v in sorted(mixed["prof"].items())},
        }
    if plain:
        out["plain_fp64"] = {
            "value": round(plain["value"], 4),
            "ms_per_step": round(plain["ms"] / args.steps, 3),
            "speedup_of_headline": round(head["value"] / plain["value"], 2),
            "pressure_iterations": [s["pressure_iterations"] for s in plain["stats"]],
            "roofline": roofline(plain),
            "clocks": plain["clocks"],
            "profile_ms": {k: round(v[1], 3) for k, v in sorted(plain["prof"].items())},
        }
    if fp64mg:
        out["fp64_multigrid"] = {
            "value": round(fp64mg["value"], 4),
            "ms_per_step": round(fp64mg["ms"] / args.steps, 3),
            "pressure_iterations": [s["pressure_iterations"] for s in fp64mg["stats"]],
            "speedup_of_headline": round(head["value"] / fp64mg["value"], 2),
            "note": "FP64 kernels and FP64 system; pressure by FP64 iterative refinement "
                    "around the FP32 multigrid-preconditioned CG (the strongest FP64 form: "
                    "speedup_of_headline here is the headline over the best FP64 path)",
            "clocks": fp64mg["clocks"],
            "profile_ms": {k: round(v[1], 3) for k, v in sorted(fp64mg["prof"].items())},
        }
    print(json.dumps(out))


def run_reference(args, rank, world):
    """The reference's algorithm on the host cores: the CPU oracle port (the
    reference's own build needs its source tree, absent on the GPU host), all
    host threads, complete time steps of the same workload from the same
    initial state, timed until --steps steps or --cpu-budget seconds."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    r = cpu_steps(args.n, args.seed, args.outer, args.cpu_budget, args.steps, threads=threads)
    wall = time.perf_counter() - t0
    value = r["value"]
    out = {
        "impl": "reference",
        "metric": "Mcell-updates/s",
        "value": round(value, 6),
        "unit": "Mcell-updates/s",
        "n_gpus": world,
        "steps": r["steps_timed"],
        "steps_requested": args.steps,
        "warmup": 0,
        "ms_per_step": round(r["seconds_per_step"] * 1e3, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic: seeded rising drops, no external data",
        "config": {"workload": "rising_drops_%d^3" % args.n, "cells": args.n ** 3,
                   "precision": "fp64", "simple_iterations_per_step": args.outer,
                   "seed": args.seed, "initial_state": "rest, hydrostatic pressure",
                   "linear_solvers": REFERENCE_SOLVERS},
        "cpu_baseline": {"value": round(value, 6), "unit": "Mcell-updates/s", "cores": threads,
                         "kind": "port", "sample": r["sample"]},
        "e2e": {"value": round(value, 6), "unit": "Mcell-updates/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "timing": {"step_seconds": r["step_seconds"],
                   "sor_sweeps_per_step": r["sor_sweeps_per_step"],
                   "wall_s": round(wall, 1),
                   "note": "complete steps timed in full, no warm-up step (the CPU path has "
                           "no caches or compilation to warm up), stopped after --steps "
                           "steps or --cpu-budget seconds"},
    }
    print(json.dumps(out))


def run_batch(args):
    """The batch workload: 512 independent 2D lid-driven cavities of 64^2 to
    256^2 cells (Re log-uniform in [100, 5000], dt 1e-3, SIMPLE converged
    per case to max |du| 1e-8 within 20 iterations), mixed precision with
    the multigrid CG, all cases advanced by one CUDA-graph launch per batch
    step (hydro_gpu_batch_step).  The launch shape of each case's linear
    solves (grid-wide, or one CTA of 256 / 512 / 1024 threads per solve) is
    chosen per grid size by the autotuner (hydro_gb300/autotune.py) before
    the run, unless --cta-threads fixes it.  The process runs with
    CUDA_DEVICE_MAX_CONNECTIONS=32 (set before CUDA starts), so that the
    GPU takes up to 32 of the graph's independent branches at once instead
    of 8.  Prints one JSON line: Mcell-updates/s = cells of all cases x
    batch steps / seconds."""
    import torch

    from hydro_gb300 import autotune, capi, cases
    from hydro_gb300.solver import Batch, launch_count
    specs = cases.cavity_batch(ncases=args.cases, seed=0)
    descs = []
    for d, _, _, _ in specs:
        d = d.copy()
        d.precision = capi.MIXED
        d.pressure_solver = capi.LINEAR_MGCG
        descs.append(d)
    if args.cta_threads is None:
        t0 = time.perf_counter()
        table = autotune.tune([(d, u0, q0) for d, (_, u0, q0, _) in zip(descs, specs)])
        tuning = {"by": "hydro_gb300/autotune.py", "seconds": round(time.perf_counter() - t0, 1),
                  "choices": table}
        autotune.apply(descs, table)
    else:
        for d in descs:
            d.cta_threads = args.cta_threads
            d.cta_cluster = args.cta_cluster
        tuning = {"by": "--cta-threads", "cta_threads": args.cta_threads,
                  "cta_cluster": args.cta_cluster}
    b = Batch(descs)
    for c, (d, u0, q0, _) in zip(b.cases, specs):
        c.set_field(capi.F_VELOCITY, u0)
        c.set_field(capi.F_PARTIAL_DENSITY, q0)
    b.init_state()
    cells = sum(d.ncells for d in descs)
    for _ in range(args.warmup):
        b.step()
    torch.cuda.synchronize()
    l0 = launch_count()
    clocks = ClockSampler(0)
    clocks.start()
    t0 = time.perf_counter()
    stats = [b.step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    clk = clocks.stop()
    iters = [s["outer_iterations"] for st in stats for s in st]
    out = {"metric": "Mcell-updates/s", "value": round(cells * args.steps / sec / 1e6, 4),
           "unit": "Mcell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(sec * 1e3 / args.steps, 2), "higher_is_better": True,
           "dtype": "f64+f32", "data": "synthetic: seeded cavity sizes and Reynolds numbers",
           "config": {"workload": "cavity_batch_%d" % args.cases, "cells": cells,
                      "form": "mixed_mg, one graph launch per batch step",
                      "cuda_device_max_connections":
                          os.environ.get("CUDA_DEVICE_MAX_CONNECTIONS"),
                      "tuning": tuning},
           "gpu_launches": launch_count() - l0, "clocks": clk,
           "simple_iterations_mean": round(sum(iters) / len(iters), 2),
           "status_ok": all(s["status"] == 0 for st in stats for s in st)}
    print(json.dumps(out))
    b.close()


def run_profile_case(args):
    """A short, bounded run of the hot path for profiler captures: the
    rising-drops case at --n^3, one time step of --outer SIMPLE iterations
    with at most --cg-limit pressure-CG iterations per solve, then exit.  At
    n = 150 the arrays of one CG iteration exceed the 129 MB L2 while the
    context stays near 2 GB and the run issues a few hundred kernel launches:
    small enough for ncu captures to end by themselves."""
    from hydro_gb300 import capi
    from hydro_gb300.solver import Hydro, launch_count
    d, u0, q0, _ = workload(args.n, args.seed, args.precision, args.outer,
                            "mgcg" if args.solver == "mgcg" else "cg")
    d.velocity_iters_limit = 50
    if args.velocity == "jacobi":
        d.velocity_solver = capi.LINEAR_JACOBI
    d.pressure_tolerance = 1e-30
    d.pressure_iters_limit = args.cg_limit
    if args.hydrostatic:
        h = init_case(Hydro(d), d, u0, q0)
    else:  # at rest with zero pressure
        h = Hydro(d)
        h.set_field(capi.F_VELOCITY, u0)
        h.set_field(capi.F_PARTIAL_DENSITY, q0)
        h.init_state()
    if args.weights:
        from hydro_gb300.net import Net, attach
        from hydro_gb300.train_guess import RHO_SCALE
        net = Net((args.n,) * 3, batch=1)
        net.load(args.weights)
        attach(h, net, 1, RHO_SCALE)
    st = h.step()
    print("profile case n=%d %s %s: %s launches=%d"
          % (args.n, args.precision, args.solver, st, launch_count()))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--weights-file", default=os.path.join(ROOT, "hydro_gb300", "weights",
                                                           "rising_drops_192.npy"),
                    help="parameters of the learned pressure guess (learned_mixed_mg)")
    ap.add_argument("--guess-iterations", type=int, default=1,
                    help="SIMPLE iterations per step whose pressure solve starts from the "
                         "network's guess (learned_mixed_mg)")
    ap.add_argument("--form", default="learned_mixed_mg",
                    choices=["learned_mixed_mg", "mixed_mg", "fp64", "fp64_mg"],
                    help="headline form: the learned guess + mixed precision + multigrid CG "
                         "(the metric's form), without the guess, or FP64")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain FP64 measurement reported beside the headline")
    ap.add_argument("--n", "--grid", dest="n", type=int, default=192,
                    help="cells per side (--grid under torchrun, whose parser claims --n)")
    ap.add_argument("--outer", type=int, default=5, help="SIMPLE iterations per step")
    ap.add_argument("--seed", type=int, default=40,
                    help="drop seed (40: the first held-out seed of the learned guess)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=150.0,
                    help="seconds of complete CPU steps (reference arm; the cpu_baseline leg "
                         "times one step)")
    ap.add_argument("--profile-case", action="store_true",
                    help="one bounded step for profiler captures (see run_profile_case)")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="--profile-case: arithmetic of the SIMPLE iteration")
    ap.add_argument("--solver", default="cg", choices=["cg", "mgcg"],
                    help="--profile-case: pressure solver")
    ap.add_argument("--cg-limit", type=int, default=40,
                    help="--profile-case: pressure iterations per solve")
    ap.add_argument("--velocity", default="gs", choices=["jacobi", "gs"],
                    help="--profile-case: momentum sweeps")
    ap.add_argument("--hydrostatic", action="store_true",
                    help="--profile-case: start from the hydrostatic pressure (default: zero)")
    ap.add_argument("--weights", default=None,
                    help="--profile-case: attach the learned guess with these parameters")
    ap.add_argument("--workload", default="drops", choices=["drops", "batch"],
                    help="batch: the 512-cavity batch (its own JSON line)")
    ap.add_argument("--cases", type=int, default=512, help="--workload batch: cases")
    ap.add_argument("--cta-threads", type=int, default=None,
                    help="--workload batch: launch shape of every case's solves (0: grid-wide; "
                         "default: chosen per grid size by the autotuner)")
    ap.add_argument("--cta-cluster", type=int, default=0,
                    help="--workload batch with --cta-threads: CTAs per solve's cluster")
    args = ap.parse_args()
    if args.workload == "batch":
        # before anything starts CUDA in this process
        os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
        run_batch(args)
        return
    if args.profile_case:
        run_profile_case(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = init_dist()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
