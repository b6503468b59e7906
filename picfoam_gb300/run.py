"""Run a picFoam case directory on the GPU (the picFoam application's time
loop, solver/picFoam/picFoam.C, over the picgpu C ABI).

    python -m picfoam_gb300.run CASE [--steps N] [--write-mesh] [--mixed]
                                     [--restart] [--allow-unsupported] [--oracle]

Reads the case (`ofcase.load_case`), runs picInitialise when the case has a
picInitialiseDict, steps to controlDict's endTime (or N steps) and writes a
time directory (phiE, E, rhoCharge, lagrangian/pic) every writeInterval and
at the end.  --write-mesh also writes constant/polyMesh.  --restart continues
from the latest time directory (startFrom latestTime; see ofcase.restart for
what is restored).  --oracle runs the CPU oracle instead of the GPU (test use
only).
"""
import argparse
import sys
import time

from . import abi, ofcase


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("case")
    ap.add_argument("--steps", type=int, default=None, help="steps to run (default: to endTime)")
    ap.add_argument("--write-mesh", action="store_true")
    ap.add_argument("--mixed", action="store_true", help="FP32 push/track, FP64 charge and Poisson")
    ap.add_argument("--allow-unsupported", action="store_true")
    ap.add_argument("--restart", action="store_true", help="continue from the latest time directory")
    ap.add_argument("--oracle", action="store_true", help=argparse.SUPPRESS)
    args = ap.parse_args(argv)

    case = ofcase.load_case(args.case, allow_unsupported=args.allow_unsupported,
                            precision=abi.PREC_MIXED if args.mixed else abi.PREC_FP64)
    for u in case.unsupported:
        print(f"[picfoam_gb300] not mapped: {u}", file=sys.stderr)
    backend = None
    if args.oracle:
        import os
        sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
        import pyoracle
        backend = pyoracle.OracleBackend(1)
    if args.write_mesh:
        ofcase.write_poly_mesh(case)
    sim = case.build(backend=backend, initialise=not args.restart)
    done = 0
    if args.restart:
        t_start = ofcase.restart(sim, case)
        done = int(round(t_start / case.delta_t))
        print(f"[picfoam_gb300] restarted at Time = {ofcase.time_name(t_start)}", flush=True)
    total = int(round(case.end_time / case.delta_t))
    steps = done + args.steps if args.steps is not None else total
    every = max(1, int(round(case.write_interval / case.delta_t))) if case.write_interval > 0 else steps
    t0 = time.time()
    while done < steps:
        k = min(every - done % every, steps - done)
        st = sim.step(k)
        done += k
        t = done * case.delta_t
        counts = " ".join(f"{n}={st.n_particles[s]}" for s, n in enumerate(case.species))
        print(f"Time = {ofcase.time_name(t)}  {counts}  PCG iterations {st.pcg_iterations}", flush=True)
        if done % every == 0 or done == steps:
            ofcase.write_fields(sim, case, t, step_index=done)
    print(f"[picfoam_gb300] {done} steps in {time.time() - t0:.2f} s")
    return 0


if __name__ == "__main__":
    sys.exit(main())
