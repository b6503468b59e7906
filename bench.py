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
# DRAM bytes (read + write) per particle-step of move_cell_kernel_fp32 measured
# by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on this workload at
# full size (64^3 cells, 50 per cell and species: one electron and one ion
# launch, 1559 MB for 26.1M particles); profiles/move_cell_kernel_fp32_two_species.md.
TRAFFIC_FP32_PER_PARTICLE = 59.7


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
    p.add_argument("--no-learned", action="store_true", help="skip the Poisson learned-vs-plain comparison")
    p.add_argument("--ws-cells", type=int, default=128)
    p.add_argument("--ws-ppc", type=int, default=4)
    p.add_argument("--ws-train", type=int, default=100)
    p.add_argument("--ws-iters", type=int, default=4)
    p.add_argument("--ws-refine", type=int, default=1)
    p.add_argument("--ws-measure", type=int, default=10)
    p.add_argument("--no-ensemble", action="store_true", help="skip the batched-ensemble measurement")
    p.add_argument("--ens-cases", type=int, default=64)
    p.add_argument("--ens-steps", type=int, default=100)
    p.add_argument("--ens-graph", type=int, default=10)
    p.add_argument("--ens-seq-steps", type=int, default=20)
    p.add_argument("--only", default=None, choices=["electrode", "unet", "ensemble", "init", "coulomb", "learned",
                                                   "swarm"],
                   help="profiling drivers: run one workload briefly and print a short summary "
                        "(electrode: electrode_box steps; unet: one forward + train steps; "
                        "ensemble: two graph replays)")
    p.add_argument("--only-steps", type=int, default=2)
    p.add_argument("--only-precond", default="jacobi", choices=["jacobi", "multigrid"],
                   help="Poisson preconditioner of the electrode driver")
    p.add_argument("--no-multigrid", action="store_true", help="skip the multigrid-preconditioned Poisson arm")
    p.add_argument("--no-init", action="store_true", help="skip the device initial-condition measurement")
    p.add_argument("--no-forms", action="store_true",
                   help="skip the FP64 form and the BorisNR / Vay / Higuera-Cary runs of the workload")
    p.add_argument("--no-collisions", action="store_true", help="skip the MCC swarm and Coulomb timings")
    p.add_argument("--pusher", default="boris", choices=["boris", "boris_nr", "vay", "hc"],
                   help="pusher of the headline workload")
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


PUSHER_NAMES = {"boris": "Boris", "boris_nr": "BorisNR", "vay": "Vay", "hc": "HigueraCary"}


def workload(args, precision=None):
    prec = precision or ("FP32 push/track, FP64 deposit" if args.precision == "mixed" else "FP64")
    return {"workload": f"3-D two-species electrostatic PIC, {args.cells}^3 hex cells in a 0.05 m cube, "
                        f"e- + Ar+ at {args.ppc}/cell each, B_z = 0.01 T, {PUSHER_NAMES[args.pusher]}, "
                        f"absorbing walls",
            "cells": args.cells ** 3, "particles": 2 * args.ppc * args.cells ** 3,
            "precision": prec,
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
    # the same sample on one thread (a single picFoam MPI rank's throughput)
    sim1 = cases.build(case, backend=pyoracle.OracleBackend(1))
    sim1.initialise_fields()
    t1 = sim1.backend.move_seconds(sim1._h)
    sim1.move()
    dt1 = sim1.backend.move_seconds(sim1._h) - t1
    sim1.close()
    return {"value": n * steps / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "single_thread_value": n / dt1,
            "sample": f"{args.cells}^3 cells, {ppc}/cell per species ({n} particles), {steps} steps on "
                      f"{cores} threads (1 step on 1 thread), FP64 CPU restatement"}


def run_reference(args, rank, ws):
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from picfoam_gb300 import abi, cases
    cores = os.cpu_count() or 1
    ppc = args.ppc
    case = cases.two_species_3d(n_cells=args.cells, per_cell=ppc, precision=abi.PREC_FP64,
                                pusher=PUSHERS[args.pusher])
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
            "data": "synthetic (seeded Maxwellian plasma)",
            "config": workload(args, precision="FP64 (picFoam's own arithmetic; the CPU restatement has no "
                                                "FP32 form)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"the whole workload: {args.cells}^3 cells, {ppc}/cell per species "
                                       f"({n} particles), {args.steps} timed steps on {cores} threads; "
                                       "CPU restatement of picFoam's move + deposit (the reference needs "
                                       "OpenFOAM-9 and cannot be built here)"},
            "e2e": {"value": tot / wall, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    sim.close()
    print(json.dumps(line), flush=True)
    return 0


PUSHERS = {"boris": 1, "boris_nr": 2, "vay": 3, "hc": 4}


def time_moves(sim, steps=10, warm=3):
    """Device time of `steps` picgpu_move passes (CUDA events around each
    move phase) after `warm` untimed ones: (particle-steps/s of the move
    kernels, ms per kernel launch, particle-steps timed)."""
    sim.set_profiling(True)
    for _ in range(warm):
        sim.move()
    sim.phase_times(reset=True)
    n = 0
    for _ in range(steps):
        n += sim.count(0) + sim.count(1)
        sim.move()
    ms, launches = sim.phase_times()["move"]
    return n / (ms * 1e-3), ms / max(launches, 1), n


def forms(args, case, peak):
    """The BASELINE config-2 runs beside the headline: the plain FP64 path
    (move_kernel_fp64, 104 B per particle-step) and the FP32 form with the
    BorisNR, Vay and Higuera-Cary pushers, each on the same particles."""
    import numpy as np
    from picfoam_gb300 import abi, cases
    from picfoam_gb300.simulation import Simulation
    out = {}
    for name, pid in (("boris_nr", abi.PUSHER_BORIS_NR), ("vay", abi.PUSHER_VAY), ("hc", abi.PUSHER_HIGUERA_CARY)):
        cfg = abi.Config.from_buffer_copy(case.cfg)
        cfg.pusher = pid
        sim = Simulation(case.mesh, cfg)
        for s, (tet, bary, U) in case.particles.items():
            sim.set_particles(s, tet, bary, U)
        sim.initialise_fields()
        v, ms_launch, n = time_moves(sim)
        sim.close()
        out[f"fp32_{name}"] = {"particle_steps_per_s": v, "kernel_ms_per_launch": ms_launch,
                               "hbm_frac": BYTES_FP32 * v / 1e9 / peak}
    fcase = cases.two_species_3d(n_cells=args.cells, per_cell=args.ppc, precision=abi.PREC_FP64)
    for name, pid in (("boris", abi.PUSHER_BORIS), ("vay", abi.PUSHER_VAY), ("hc", abi.PUSHER_HIGUERA_CARY)):
        cfg = abi.Config.from_buffer_copy(fcase.cfg)
        cfg.pusher = pid
        sim = Simulation(fcase.mesh, cfg)
        for s, (tet, bary, U) in fcase.particles.items():
            sim.set_particles(s, tet, bary, U)
        sim.initialise_fields()
        v, ms_launch, n = time_moves(sim, steps=5)
        sim.close()
        out[f"fp64_{name}"] = {"particle_steps_per_s": v, "kernel_ms_per_launch": ms_launch,
                               "hbm_frac": BYTES_FP64 * v / 1e9 / peak, "kernel": "move_kernel_fp64",
                               "bytes_per_particle_step": BYTES_FP64}
    out["note"] = ("same mesh, population and seed as the headline; FP64: the exact form (bit-exact against the "
                   "oracle), FP32: the mixed form; particle-steps/s of the move kernels from CUDA events")
    return out


def collisions(args):
    """BASELINE config 3 at size: the electron swarm (10M electrons on
    32x32x256 cells, E = 1e4 V/m, argon-like gas at 1e21, MCC with
    ionisation, FP32 push) and the Coulomb thermalisation (16^3 cells, 400
    electrons per cell, NanbuYonemura + Nanbu, coulombLog 15): ms per
    collision phase and particle-steps/s of whole steps."""
    from picfoam_gb300 import abi, cases
    out = {}
    case = cases.electron_swarm()
    sim = cases.build(case)
    sim.set_profiling(True)
    for _ in range(3):
        sim.step(1)
    sim.phase_times(reset=True)
    n0 = sim.count(0)
    steps = 10
    sim.synchronize()
    sim.timer_start()
    ps = 0
    for _ in range(steps):
        ps += sim.count(0) + sim.count(1)
        st = sim.step(1)
    ms = sim.timer_stop()
    ph = sim.phase_times()
    out["swarm"] = {"electrons_at_start": n0, "electrons_at_end": sim.count(0), "steps": steps,
                    "mcc_ms_per_step": ph["mcc"][0] / steps, "move_ms_per_step": ph["move"][0] / steps,
                    "step_ms": ms / steps, "particle_steps_per_s": ps / (ms * 1e-3),
                    "mcc_candidates_last_step": int(st.mcc_candidates),
                    "config": "32x32x256 cells, 0.02x0.02x0.16 m, E_z = 1e4 V/m, n_gas = 1e21 m^-3, 256-point "
                              "elastic/excitation/ionisation tables, NanbuElectronNeutral, FP32 push"}
    sim.close()
    case = cases.coulomb_thermalisation(n_cells=16, per_cell=400, precision=abi.PREC_MIXED)
    sim = cases.build(case)
    sim.set_profiling(True)
    sim.step(2)
    sim.phase_times(reset=True)
    steps = 5
    sim.synchronize()
    sim.timer_start()
    sim.step(steps)
    ms = sim.timer_stop()
    ph = sim.phase_times()
    out["coulomb"] = {"electrons": sim.count(0), "steps": steps, "coulomb_ms_per_step": ph["coulomb"][0] / steps,
                      "step_ms": ms / steps, "particle_steps_per_s": sim.count(0) * steps / (ms * 1e-3),
                      "config": "16^3 cells, 400 e-/cell, n = 1e18 m^-3, T_x = 2 eV, T_yz = 1 eV, NanbuYonemura "
                                "pairing, Nanbu collide, coulombLog 15, FP32 push"}
    sim.close()
    return out


def learned_vs_plain(args):
    """Poisson ms/step and PCG iterations on the electrode geometry (128^3
    cells, two floating boxes, a 100 V box, PCG to 1e-8): previous-potential
    start against the learned warm start after its training solves."""
    import numpy as np
    from picfoam_gb300 import cases
    out = {}
    from picfoam_gb300 import abi
    modes = ("plain", "learned") if args.no_multigrid else ("plain", "learned", "multigrid")
    for mode in modes:
        case = cases.electrode_box(n_cells=args.ws_cells, per_cell=args.ws_ppc)
        if mode == "multigrid":
            case.cfg.pcg_precond = abi.PRECOND_MULTIGRID
        if mode == "learned":
            case.cfg.learned.enabled = 1
            case.cfg.learned.train_steps = args.ws_train
            case.cfg.learned.train_iters = args.ws_iters
            case.cfg.learned.refine = args.ws_refine
            case.cfg.learned.lr = 2e-3
        sim = cases.build(case)
        sim.set_profiling(True)
        t0 = time.perf_counter()
        pre = args.ws_train + 2 if mode == "learned" else 3
        last = None
        for _ in range(pre):
            last = sim.step(1)
        t_train = time.perf_counter() - t0
        sim.phase_times(reset=True)
        its, r0, rp, alpha = [], [], [], []
        for _ in range(args.ws_measure):
            st = sim.step(1)
            its.append(st.pcg_iterations)
            r0.append(st.pcg_residual_initial)
            rp.append(st.learned_residual)
            alpha.append(st.learned_alpha)
        ph = sim.phase_times()
        d = {"poisson_ms_per_step": ph["poisson"][0] / args.ws_measure,
             "pcg_iterations_per_step": float(np.mean(its)),
             "start_residual": float(np.mean(r0))}
        if mode == "learned":
            d.update({"previous_potential_residual": float(np.mean(rp)), "line_search_alpha": float(np.mean(alpha)),
                      "training_solves": args.ws_train, "adam_steps_per_solve": args.ws_iters,
                      "refine_passes": args.ws_refine, "final_training_loss": last.learned_loss,
                      "training_wall_s": t_train, "active": bool(st.learned_active)})
            # the fallback check closes its first window after 20 net-started solves
            sim.phase_times(reset=True)
            for _ in range(max(0, 20 - args.ws_measure) + 10):
                st = sim.step(1)
            ph = sim.phase_times()
            d["fallback_after_20_solves"] = bool(st.learned_fallback)
            d["poisson_ms_per_step_after_check"] = ph["poisson"][0] / (max(0, 20 - args.ws_measure) + 10)
        out[mode] = d
        sim.close()
    out["iteration_ratio_plain_over_learned"] = (out["plain"]["pcg_iterations_per_step"] /
                                                 max(out["learned"]["pcg_iterations_per_step"], 1e-9))
    out["ms_ratio_plain_over_learned"] = (out["plain"]["poisson_ms_per_step"] /
                                          max(out["learned"]["poisson_ms_per_step"], 1e-9))
    if "multigrid" in out:
        out["iteration_ratio_plain_over_multigrid"] = (out["plain"]["pcg_iterations_per_step"] /
                                                       max(out["multigrid"]["pcg_iterations_per_step"], 1e-9))
        out["ms_ratio_plain_over_multigrid"] = (out["plain"]["poisson_ms_per_step"] /
                                                max(out["multigrid"]["poisson_ms_per_step"], 1e-9))
    out["config"] = (f"{args.ws_cells}^3 cells, 0.1 m cube, two floating 8^3-cell boxes and a 100 V box, "
                     f"e- + Ar+ at {args.ws_ppc}/cell, FP64 Jacobi PCG (Chronopoulos-Gear) to 1e-8 relative residual; "
                     f"multigrid: flexible FP64 PCG with an FP32 aggregation V-cycle (2 + 2 Jacobi sweeps), same "
                     f"tolerance; "
                     f"{args.ws_measure} measured steps")
    return out


def init_conditions(args, reps=3):
    """picgpu_initialise on the benchmark workload (64^3 cells, 0.05 m, e- and
    Ar+ at n = 1e15 with the benchmark's weight: 50 per cell and species,
    Equipartition at 2 eV / 0.03 eV): device placement time (CUDA events) and
    particles/s, against the oracle's restatement (one thread, a bounded
    sample of 16^3 cells) and the host path it replaces (numpy sampling of
    the same population + upload through picgpu_set_particles)."""
    import numpy as np
    from picfoam_gb300 import abi, cases
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    L, n = 0.05, 1e15
    w = n * L ** 3 / (args.cells ** 3 * args.ppc)
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    species = [(cases.M_E, -cases.E_CHARGE, w, True), (cases.M_AR, cases.E_CHARGE, w, True)]
    init = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(n, n), temperature=(2.0, 0.03),
                             electron_volt=True)
    case = cases.empty_case(n_cells=(args.cells,) * 3, length=(L,) * 3, species=species, precision=prec)
    sim = cases.build(case)
    times, added = [], 0
    for _ in range(reps + 1):                       # the first call also sizes the store
        st = sim.initialise(init)
        times.append(st.place_ms)
        added = st.added[0] + st.added[1]
    ms = float(np.median(times[1:]))
    t0 = time.perf_counter()
    init.solve_fields = 0
    sim.initialise(init)
    wall = time.perf_counter() - t0
    sim.close()
    # host path: numpy sampling of the same population and the upload
    t0 = time.perf_counter()
    hc = cases.two_species_3d(n_cells=args.cells, per_cell=args.ppc, precision=prec)
    t1 = time.perf_counter()
    sim2 = cases.build(hc)
    t2 = time.perf_counter()
    sim2.close()
    # oracle, one thread, 16^3-cell sample at the same density and weight
    sc = 16
    ocase = cases.empty_case(n_cells=(sc,) * 3, length=(L * sc / args.cells,) * 3, species=species,
                             precision=abi.PREC_FP64)
    osim = cases.build(ocase, backend=pyoracle.OracleBackend(1))
    t3 = time.perf_counter()
    ost = osim.initialise(init)
    t4 = time.perf_counter()
    osim.close()
    on = ost.added[0] + ost.added[1]
    return {"model": "Equipartition", "particles": int(added), "place_ms": ms,
            "particles_per_s": added / (ms * 1e-3), "initialise_call_wall_s": wall,
            "host_numpy_sampling_s": t1 - t0, "host_upload_s": t2 - t1,
            "oracle_single_thread_particles_per_s": on / (t4 - t3), "oracle_sample_particles": int(on),
            "config": f"{args.cells}^3 cells, 0.05 m, e- + Ar+ at 1e15 m^-3, weight {w:.4g} "
                      f"({args.ppc}/cell per species), {args.precision} store"}


def ensemble(args):
    """Batched swarm ensemble (64 cases of 16x16x128 cells, 10-1000 Td,
    1e5-4e6 electrons each from seed 7): one context, CUDA-graph steps with
    tuned launch shapes, against the same cases run one after another."""
    import numpy as np
    from picfoam_gb300 import cases
    case = cases.swarm_ensemble(n_cases=args.ens_cases)
    sim = cases.build_ensemble(case)
    S = args.ens_graph
    # tuning replays (live steps) then warm-up
    sim.step_graph(32 * S, S)
    bps, blk, tune = sim.graph_tuning()
    n0 = sim.count(0) + sim.count(1)
    sim.synchronize()
    sim.timer_start()
    st = sim.step_graph(args.ens_steps, S)
    ms = sim.timer_stop()
    n1 = sim.count(0) + sim.count(1)
    batched = 0.5 * (n0 + n1) * args.ens_steps / (ms * 1e-3)
    out, iz = sim.case_stats(0, args.ens_cases)
    dt = case.meta["dt"]
    steps_total = sim_steps = 32 * S + args.ens_steps
    drift = out[:, 3] / np.maximum(out[:, 0], 1)
    sim.close()
    # the same cases one after another, each in its own context (regular steps)
    seq_ps, seq_s = 0, 0.0
    counts = case.meta["counts"]
    tet, bary, U = case.particles[0]
    cpc = case.meta["cells_per_case"]
    case_of = (tet // 12) // cpc
    from picfoam_gb300.simulation import Simulation
    for k in range(args.ens_cases):
        sel = case_of == k
        cfg = case.cfg
        cfg.E_applied[2] = case.meta["E"][k, 2]
        s1 = Simulation(case.mesh, cfg, keepalive=case.keepalive)
        s1.set_particles(0, tet[sel] - 12 * cpc * k, bary[sel], U[sel])
        s1.set_particles(1, np.zeros(0, np.int32), np.zeros((0, 3)), np.zeros((0, 3)))
        s1.step(2)
        s1.synchronize()
        s1.timer_start()
        for _ in range(args.ens_seq_steps):
            seq_ps += s1.count(0) + s1.count(1)
            s1.step(1)
        seq_s += s1.timer_stop() * 1e-3
        s1.close()
    sequential = seq_ps / seq_s
    return {"config": f"{args.ens_cases} cases of 16x16x128 cells (0.01x0.01x0.08 m), E/N 10-1000 Td at 1e21 m^-3, "
                      f"1e5-4e6 e- per case (seed 7, {int(counts.sum())} total), NanbuElectronNeutral MCC with "
                      f"ionisation, FP32 push, MaxwellSolver none",
            "batched_particle_steps_per_s": batched, "sequential_particle_steps_per_s": sequential,
            "speedup": batched / sequential, "steps_per_graph": S, "timed_steps": args.ens_steps,
            "ms_per_step": ms / args.ens_steps,
            "tuning": {"move_blocks_per_sm": bps, "mcc_block": blk,
                       "candidate_ns_per_particle_step": [float(x) for x in tune if x > 0]},
            "per_case_drift_velocity_mps": [float(x) for x in drift],
            "per_case_ionisation_rate_per_s": [float(iz[k]) / max(out[k, 0], 1) / (steps_total * dt)
                                               for k in range(args.ens_cases)],
            "per_case_EN_Td": [float(x) for x in case.meta["EN_Td"]],
            "ionisations": int(st.mcc_ionization)}


def run_ours(args, rank, ws):
    import numpy as np
    from picfoam_gb300 import abi, cases
    from picfoam_gb300.simulation import Simulation
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        # one GPU per rank: the library uses the current device of its own
        # (static) CUDA runtime, so the rank's GPU is the only one it sees
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devs = [d for d in vis.split(",") if d] if vis else None
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local % len(devs)] if devs else str(local)
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    case = cases.two_species_3d(n_cells=args.cells, per_cell=args.ppc, precision=prec, seed=1234 + rank,
                                pusher=PUSHERS[args.pusher])
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
        it, pairs = [], []
        for _ in range(args.poisson_steps):
            phi_prev = sim.field(abi.FIELD_PHI) if not args.no_multigrid else None
            st = sim.step(1)
            it.append(st.pcg_iterations)
            if phi_prev is not None:
                pairs.append((sim.field(abi.FIELD_RHO), phi_prev))
        ph2 = sim.phase_times()
        pois = {"ms_per_step": ph2["poisson"][0] / args.poisson_steps,
                "efield_ms_per_step": ph2["efield"][0] / args.poisson_steps,
                "pcg_iterations_per_step": float(np.mean(it)), "tolerance": case.cfg.pcg_tol,
                "preconditioner": "Jacobi", "cells": args.cells ** 3}
        if pairs:
            # the same solves (each step's charge density, the previous
            # potential as the start) with the multigrid preconditioner
            cfg_mg = abi.Config.from_buffer_copy(case.cfg)
            cfg_mg.pcg_precond = abi.PRECOND_MULTIGRID
            mg = Simulation(case.mesh, cfg_mg)
            mg.set_profiling(True)
            mg.solve_poisson(*pairs[0])             # warm-up (graph capture)
            mg.phase_times(reset=True)
            mit = [mg.solve_poisson(rho, phi0)[1].pcg_iterations for rho, phi0 in pairs]
            mph = mg.phase_times()
            mg.close()
            pois["multigrid"] = {"ms_per_step": mph["poisson"][0] / len(pairs),
                                 "pcg_iterations_per_step": float(np.mean(mit)),
                                 "note": "FP64 flexible PCG with the FP32 aggregation V-cycle, same tolerance "
                                         "and start guesses"}
        # whole picgpu_step (push + track + deposit, charge update, Poisson,
        # E and its interpolation, store maintenance) with either preconditioner
        full = {}
        for precond in ("jacobi", "multigrid"):
            if precond == "jacobi":
                fs = sim
            else:
                if args.no_multigrid:
                    continue
                cfg_mg = abi.Config.from_buffer_copy(case.cfg)
                cfg_mg.pcg_precond = abi.PRECOND_MULTIGRID
                fs = Simulation(case.mesh, cfg_mg)
                for sp, (tet, bary, U) in case.particles.items():
                    fs.set_particles(sp, tet, bary, U)
                fs.initialise_fields()
                fs.step(2)
            nps = fs.count(0) + fs.count(1)
            fs.synchronize()
            fs.timer_start()
            fs.step(args.poisson_steps)
            fms = fs.timer_stop()
            full[precond] = {"particle_steps_per_s": nps * args.poisson_steps / (fms * 1e-3),
                             "ms_per_step": fms / args.poisson_steps}
            if fs is not sim:
                fs.close()
        pois["full_step"] = full
    sim.close()
    # e2e through the public API with host buffers in page-locked memory
    # (picgpu_host_alloc): upload the population, K move passes (each returns
    # its counters to the host), download it into host buffers.
    e2e = None
    if not args.no_e2e:
        from picfoam_gb300.simulation import pinned_empty
        host_in, host_out = {}, {}
        for s, (tet, bary, U) in case.particles.items():
            n = len(tet)
            bufs = (pinned_empty(n, np.int32), pinned_empty((n, 3), np.float64), pinned_empty((n, 3), np.float64))
            for dst, src in zip(bufs, (tet, bary, U)):
                dst[...] = src
            host_in[s] = bufs
            host_out[s] = (pinned_empty(n, np.int32), pinned_empty((n, 3), np.float64),
                           pinned_empty((n, 3), np.float64))
            for a in host_out[s]:
                a.fill(0)
        # storage sized with the context (capacity_hint), as set_particles would
        cfg2 = abi.Config.from_buffer_copy(case.cfg)
        for s, (tet, _, _) in case.particles.items():
            cfg2.species[s].capacity_hint = len(tet) + len(tet) // 4
        t0 = time.perf_counter()
        sim2 = Simulation(case.mesh, cfg2)
        t_create = time.perf_counter() - t0
        # untimed warm-up of the same path and buffers (the first DMA over a
        # freshly page-locked buffer is several times slower)
        for s, bufs in host_in.items():
            sim2.set_particles(s, *bufs)
        sim2.move()
        for s in host_in:
            sim2.get_particles(s, out=host_out[s])
        h2d = 0
        t0 = time.perf_counter()
        for s, (tet, bary, U) in host_in.items():
            sim2.set_particles(s, tet, bary, U)
            h2d += tet.nbytes + bary.nbytes + U.nbytes
        t1 = time.perf_counter()
        ps = 0
        for _ in range(args.steps):
            ps += sim2.count(0) + sim2.count(1)
            sim2.move()
        t2 = time.perf_counter()
        d2h = 0
        for s in host_in:
            tet, bary, U = sim2.get_particles(s, out=host_out[s])
            d2h += tet.nbytes + bary.nbytes + U.nbytes
        wall = time.perf_counter() - t0
        split = {"upload_s": t1 - t0, "moves_s": t2 - t1, "download_s": t0 + wall - t2}
        sim2.close()
        del host_in, host_out
        e2e_val = allreduce_sum(ps, ws) / allreduce_max(wall, ws)
        e2e = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d // args.steps, **split,
               "d2h_bytes_per_step": d2h // args.steps + 64,
               "note": "upload of the particle population from page-locked host arrays "
                       "(picgpu_host_alloc), K picgpu_move calls (counters read back each step), download of "
                       "the population into page-locked host arrays; "
                       "device storage sized at context creation (capacity_hint), one untimed warm-up pass "
                       "of the same path; "
                       f"context creation ({t_create:.2f} s) excluded"}
    peak, peak_kind = peaks()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 push/track + f64 deposit" if prec == abi.PREC_MIXED else "f64",
            "data": "synthetic (seeded Maxwellian plasma, uniform positions)", "config": workload(args),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (TRAFFIC_FP32_PER_PARTICLE * n_steps_particles / max(move_launches, 1)
                                     if prec == abi.PREC_MIXED else None),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one electron and "
                                           "one ion launch of this workload, per particle "
                                           "(profiles/move_cell_kernel_fp32_two_species.md)",
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "kernel": "move_cell_kernel_fp32" if prec == abi.PREC_MIXED else "move_kernel_fp64",
                         "bytes_per_particle_step": bytes_pp,
                         "kernel_ms_per_launch": move_ms / max(move_launches, 1),
                         "launches": move_launches},
            "gpu_launches": int(allreduce_sum(launches, ws)), "clocks": clk, "poisson": pois,
            "particles": counts}
    if e2e:
        line["e2e"] = e2e
    if rank == 0 and ws == 1 and not args.no_learned:
        try:
            line["poisson_learned_vs_plain"] = learned_vs_plain(args)
        except Exception as ex:  # reported, not fatal
            line["poisson_learned_vs_plain"] = {"error": str(ex)}
    if rank == 0 and ws == 1 and not args.no_init:
        try:
            line["initial_conditions"] = init_conditions(args)
        except Exception as ex:  # reported, not fatal
            line["initial_conditions"] = {"error": str(ex)}
    if rank == 0 and ws == 1 and not args.no_ensemble:
        try:
            line["ensemble"] = ensemble(args)
        except Exception as ex:  # reported, not fatal
            line["ensemble"] = {"error": str(ex)}
    if rank == 0 and ws == 1 and not args.no_forms:
        try:
            line["forms"] = forms(args, case, peak)
        except Exception as ex:  # reported, not fatal
            line["forms"] = {"error": str(ex)}
    if rank == 0 and ws == 1 and not args.no_collisions:
        try:
            line["collisions"] = collisions(args)
        except Exception as ex:  # reported, not fatal
            line["collisions"] = {"error": str(ex)}
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_baseline(args)
        except Exception as ex:  # reported, not fatal
            line["cpu_baseline"] = {"value": None, "error": str(ex)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_only(args):
    """Short runs of one workload for ncu captures (no timing claims)."""
    import ctypes as C
    import numpy as np
    from picfoam_gb300 import cases, native
    if args.only == "electrode":
        case = cases.electrode_box(n_cells=args.ws_cells, per_cell=args.ws_ppc)
        if args.only_precond == "multigrid":
            from picfoam_gb300 import abi
            case.cfg.pcg_precond = abi.PRECOND_MULTIGRID
        sim = cases.build(case)
        for _ in range(args.only_steps):
            st = sim.step(1)
        print(json.dumps({"only": "electrode", "cells": args.ws_cells ** 3, "pcg_iterations": st.pcg_iterations}))
    elif args.only == "unet":
        lib = native.load()
        n = args.ws_cells
        V = n ** 3
        h = C.c_void_p()
        assert lib.picgpu_unet_create(n, n, n, 3, C.byref(h)) == 0
        rng = np.random.default_rng(0)
        x = np.zeros((V, 2), np.float32)
        x[:, 0] = rng.standard_normal(V)
        x[:, 1] = 1.0
        t = rng.standard_normal(V).astype(np.float32)
        m = np.ones(V, np.float32)
        out = np.zeros(V, np.float32)
        p = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
        assert lib.picgpu_unet_forward(h, p(x), p(out)) == 0
        loss = C.c_double()
        assert lib.picgpu_unet_train(h, p(x), p(t), p(m), args.only_steps, 1e-3, C.byref(loss)) == 0
        lib.picgpu_unet_destroy(h)
        print(json.dumps({"only": "unet", "grid": n, "loss": loss.value}))
    elif args.only == "learned":
        # the learned warm start against the previous-potential start on the
        # electrode geometry with the --ws-* settings (BASELINE config 4 as
        # stated: --ws-ppc 30 --ws-train 500 --ws-measure 2000)
        print(json.dumps({"only": "learned", "poisson_learned_vs_plain": learned_vs_plain(args)}))
    elif args.only == "swarm":
        # the electron swarm of the collision benchmark (32x32x256 cells,
        # 10M electrons, background MCC with the FP32 store)
        case = cases.electron_swarm()
        sim = cases.build(case)
        for _ in range(args.only_steps):
            st = sim.step(1)
        print(json.dumps({"only": "swarm", "electrons": sim.count(0), "mcc_candidates": st.mcc_candidates}))
    elif args.only == "coulomb":
        # the Coulomb thermalisation of the swarm workload (16^3 cells, 400
        # electrons per cell, NanbuYonemura + Nanbu), FP32 store
        from picfoam_gb300 import abi
        case = cases.coulomb_thermalisation(n_cells=16, per_cell=400, precision=abi.PREC_MIXED)
        sim = cases.build(case)
        for _ in range(args.only_steps):
            st = sim.step(1)
        print(json.dumps({"only": "coulomb", "electrons": sim.count(0), "pairs": st.coulomb_pairs}))
    elif args.only == "init":
        from picfoam_gb300 import abi
        L, n = 0.05, 1e15
        w = n * L ** 3 / (args.cells ** 3 * args.ppc)
        case = cases.empty_case(n_cells=(args.cells,) * 3, length=(L,) * 3, precision=abi.PREC_MIXED,
                                species=[(cases.M_E, -cases.E_CHARGE, w, True), (cases.M_AR, cases.E_CHARGE, w, True)])
        sim = cases.build(case)
        init = cases.init_config(abi.INIT_EQUIPARTITION, number_density=(n, n), temperature=(2.0, 0.03),
                                 electron_volt=True)
        for _ in range(args.only_steps):
            st = sim.initialise(init)
        print(json.dumps({"only": "init", "particles": st.added[0] + st.added[1], "place_ms": st.place_ms}))
    else:
        case = cases.swarm_ensemble(n_cases=args.ens_cases)
        sim = cases.build_ensemble(case)
        sim.step_graph(10, 10)
        sim.step_graph(10, 10)
        print(json.dumps({"only": "ensemble", "cases": args.ens_cases, "particles": sim.count(0)}))
    return 0


def main():
    args = parse()
    if args.only:
        return run_only(args)
    rank, ws = dist()
    if args.impl == "reference":
        return run_reference(args, rank, ws)
    return run_ours(args, rank, ws)


if __name__ == "__main__":
    sys.exit(main())
