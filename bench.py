#!/usr/bin/env python
"""Benchmark of the picFoam particle hot path on GB300.

Metric: particle-steps/s of push + track + deposit (picgpu_move: the fused
move kernel per species, the charge update and the compaction of removed
particles) on the 3-D two-species workload: 0.05 m cube, 64^3 hex cells,
electrons and Ar+ at 50/cell each (26.2M particles), n = 1e15 m^-3,
T_e = 2 eV, T_i = 0.03 eV, B = 0.01 T along z, grounded absorbing walls,
Boris pusher, FP32 push/track with FP64 charge accumulation.  The particle
store (26.2M x 28 B = 734 MB) is larger than L2, so consecutive steps do not
hit in L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica ("replicas
only": the path has no exchange on one GPU per rank); value sums the ranks'
particle-steps over the slowest rank's time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s (push+track+deposit)"
UNIT = "particle-steps/s"
BYTES_FP32 = 56   # int32 tet + 3 x f32 barycentric + 3 x f32 velocity, read + write
BYTES_FP64 = 104  # int32 tet + 3 x f64 barycentric + 3 x f64 velocity, read + write


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cells", type=int, default=64)
    p.add_argument("--ppc", type=int, default=50)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--poisson-steps", type=int, default=3)
    p.add_argument("--sort-interval", type=int, default=10,
                   help="re-sort the particle store into cell order every N steps (0: never)")
    return p.parse_args()


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("gloo")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as tdist
        tdist.barrier()


def allreduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([x], dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as tdist
    t = torch.tensor([x], dtype=torch.float64)
    tdist.all_reduce(t, op=tdist.ReduceOp.SUM)
    return float(t.item())


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(args):
    return {"workload": f"3-D two-species electrostatic PIC, {args.cells}^3 hex cells in a 0.05 m cube, "
                        f"e- + Ar+ at {args.ppc}/cell each, B_z = 0.01 T, Boris, absorbing walls",
            "cells": args.cells ** 3, "particles": 2 * args.ppc * args.cells ** 3,
            "precision": "FP32 push/track, FP64 deposit" if args.precision == "mixed" else "FP64",
            "l2": "particle store larger than L2 (no flush needed)"}


def cpu_baseline(args, steps=2):
    """The CPU oracle (FP64 restatement) on all host cores, on a bounded
    sample of the same workload: same mesh, fewer particles per cell."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from picfoam_gb300 import abi, cases
    cores = os.cpu_count() or 1
    ppc = max(1, min(args.ppc, 4))
    case = cases.two_species_3d(n_cells=args.cells, per_cell=ppc, precision=abi.PREC_FP64)
    sim = cases.build(case, backend=pyoracle.OracleBackend(cores))
    sim.initialise_fields()
    n = sim.count(0) + sim.count(1)
    be = sim.backend
    t0 = be.move_seconds(sim._h)
    for _ in range(steps):
        sim.move()
    dt = be.move_seconds(sim._h) - t0
    sim.close()
    return {"value": n * steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{args.cells}^3 cells, {ppc}/cell per species ({n} particles), {steps} steps, "
                      f"FP64 CPU restatement"}


def run_reference(args, rank, ws):
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from picfoam_gb300 import abi, cases
    cores = os.cpu_count() or 1
    ppc = max(1, min(args.ppc, 2))
    case = cases.two_species_3d(n_cells=args.cells, per_cell=ppc, precision=abi.PREC_FP64)
    sim = cases.build(case, backend=pyoracle.OracleBackend(cores))
    sim.initialise_fields()
    for _ in range(args.warmup):
        sim.move()
    n = sim.count(0) + sim.count(1)
    be = sim.backend
    t0 = be.move_seconds(sim._h)
    w0 = time.perf_counter()
    tot = 0
    for _ in range(args.steps):
        tot += sim.count(0) + sim.count(1)
        sim.move()
    dt = be.move_seconds(sim._h) - t0
    wall = time.perf_counter() - w0
    value = tot / dt
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Maxwellian plasma)", "config": workload(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.cells}^3 cells, {ppc}/cell per species ({n} particles) per step; "
                                       "CPU restatement of picFoam's move + deposit (the reference needs "
                                       "OpenFOAM-9 and cannot be built here)"},
            "e2e": {"value": tot / wall, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    sim.close()
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank, ws):
    import numpy as np
    from picfoam_gb300 import abi, cases
    from picfoam_gb300.simulation import Simulation
    local = int(os.environ.get("LOCAL_RANK", "0"))
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    case = cases.two_species_3d(n_cells=args.cells, per_cell=args.ppc, precision=prec, seed=1234 + rank)
    case.cfg.sort_interval = args.sort_interval
    sim = cases.build(case)
    sim.initialise_fields()
    sim.set_profiling(True)
    for _ in range(max(args.warmup, 3)):
        sim.move()
    sim.phase_times(reset=True)
    l0 = sim.kernel_launches()
    n_steps_particles = 0
    counts = [sim.count(0), sim.count(1)]
    barrier(ws)
    sim.synchronize()
    clocks = Clocks(local)
    clocks.start()
    sim.timer_start()
    for _ in range(args.steps):
        n_steps_particles += sim.count(0) + sim.count(1)
        sim.move()
    ms = sim.timer_stop()
    clk = clocks.stop()
    launches = sim.kernel_launches() - l0
    ph = sim.phase_times()
    move_ms, move_launches = ph["move"]
    bytes_pp = BYTES_FP32 if prec == abi.PREC_MIXED else BYTES_FP64
    achieved = n_steps_particles * bytes_pp / (move_ms * 1e-3) / 1e9 if move_ms > 0 else 0.0
    ms_max = allreduce_max(ms, ws)
    total_ps = allreduce_sum(n_steps_particles, ws)
    value = total_ps / (ms_max * 1e-3)
    # Poisson ms/step and iterations on full steps
    pois = {}
    if args.poisson_steps > 0:
        sim.phase_times(reset=True)
        it = []
        for _ in range(args.poisson_steps):
            st = sim.step(1)
            it.append(st.pcg_iterations)
        ph2 = sim.phase_times()
        pois = {"ms_per_step": ph2["poisson"][0] / args.poisson_steps,
                "efield_ms_per_step": ph2["efield"][0] / args.poisson_steps,
                "pcg_iterations_per_step": float(np.mean(it)), "tolerance": case.cfg.pcg_tol,
                "preconditioner": "Jacobi", "cells": args.cells ** 3}
    sim.close()
    # e2e through the public API with host buffers: upload the population,
    # K move passes (each returns its counters to the host), download it.
    e2e = None
    if not args.no_e2e:
        parts = case.particles
        t0 = time.perf_counter()
        sim2 = Simulation(case.mesh, case.cfg)
        t_create = time.perf_counter() - t0
        h2d = 0
        t0 = time.perf_counter()
        for s, (tet, bary, U) in parts.items():
            sim2.set_particles(s, tet, bary, U)
            h2d += tet.nbytes + bary.nbytes + U.nbytes
        ps = 0
        for _ in range(args.steps):
            ps += sim2.count(0) + sim2.count(1)
            sim2.move()
        d2h = 0
        for s in parts:
            tet, bary, U = sim2.get_particles(s)
            d2h += tet.nbytes + bary.nbytes + U.nbytes
        wall = time.perf_counter() - t0
        sim2.close()
        e2e_val = allreduce_sum(ps, ws) / allreduce_max(wall, ws)
        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps,
               "d2h_bytes_per_step": d2h // args.steps + 64,
               "note": "upload of the particle population from host arrays, K picgpu_move calls "
                       "(counters read back each step), download of the population; "
                       f"context creation ({t_create:.2f} s) excluded"}
    peak, peak_kind = peaks()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 push/track + f64 deposit" if prec == abi.PREC_MIXED else "f64",
            "data": "synthetic (seeded Maxwellian plasma, uniform positions)", "config": workload(args),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": None,
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "kernel": "move_kernel_fp32" if prec == abi.PREC_MIXED else "move_kernel_fp64",
                         "bytes_per_particle_step": bytes_pp,
                         "kernel_ms_per_launch": move_ms / max(move_launches, 1),
                         "launches": move_launches},
            "gpu_launches": int(allreduce_sum(launches, ws)), "clocks": clk, "poisson": pois,
            "particles": counts}
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(args)
        except Exception as ex:  # reported, not fatal
            line["cpu_baseline"] = {"value": None, "error": str(ex)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    rank, ws = dist()
    if args.impl == "reference":
        return run_reference(args, rank, ws)
    return run_ours(args, rank, ws)


if __name__ == "__main__":
    sys.exit(main())
