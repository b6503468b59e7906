"""The FP32 form's errors against the FP64 oracle, measured (TEST
INFRASTRUCTURE; needs a GPU; the tests in test_gpu_forms.py and
test_gpu_parity.py bound the same quantities).

    python tests/fp32_form_errors.py > fp32_form_errors.json

Prints one JSON document:
  energy_drift      1-D plasma oscillation (128 cells, 200/cell, dt = 0.05/wpe,
                    2000 steps): total-energy drift (last - first) / first of
                    the FP32 form, the FP64 form and the oracle
  gyro              magneticRotation set-up (one electron at 0.1 c in 1 T,
                    200 steps per orbit, 10 orbits) per pusher: gyro-phase
                    difference [rad], relative radius and speed differences
  drift_velocity    E x B drift (E_x = 2e5 V/m, B_z = 1 T, 100 steps per
                    orbit, orbits 2-4): relative difference of the drift
"""
import json
import math
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import pyoracle  # noqa: E402
from picfoam_gb300 import abi, cases  # noqa: E402
from picfoam_gb300.simulation import GpuBackend, Mesh  # noqa: E402


def energy_drift(gpu):
    out = {}
    for name, prec, be in [("oracle", abi.PREC_FP64, pyoracle.OracleBackend(4)),
                           ("fp64", abi.PREC_FP64, gpu), ("fp32", abi.PREC_MIXED, gpu)]:
        case = cases.plasma_oscillation_1d(Mesh, n_cells=128, per_cell=200, precision=prec)
        sim = cases.build(case, backend=be)
        sim.initialise_fields()
        d = sim.diagnostics()
        e0 = d.kinetic_energy[0] + d.field_energy
        sim.step(2000)
        d = sim.diagnostics()
        out[name] = (d.kinetic_energy[0] + d.field_energy - e0) / e0
        sim.close()
    out["fp32_minus_oracle"] = out["fp32"] - out["oracle"]
    return out


def gyration(case, backend, orbits, spo):
    sim = cases.build(case, backend=backend)
    m = Mesh(case.mesh)
    sim.step(orbits * spo)
    tet, bary, U = sim.get_particles(0)
    return m.position(tet, bary)[0], U[0]


def gyro(gpu):
    out = {}
    names = {abi.PUSHER_BORIS: "Boris", abi.PUSHER_BORIS_NR: "BorisNR", abi.PUSHER_VAY: "Vay",
             abi.PUSHER_HIGUERA_CARY: "HigueraCary"}
    for pusher, name in names.items():
        spo, orbits = 200, 10
        case = cases.magnetic_rotation(Mesh, pusher=pusher, precision=abi.PREC_MIXED, steps_per_orbit=spo)
        xg, ug = gyration(case, gpu, orbits, spo)
        case.cfg.precision = abi.PREC_FP64
        xo, uo = gyration(case, pyoracle.OracleBackend(1), orbits, spo)
        out[name] = {
            "phase_rad": abs(math.remainder(math.atan2(ug[1], ug[0]) - math.atan2(uo[1], uo[0]), 2 * math.pi)),
            "radius_rel": abs(np.linalg.norm(xg[:2]) - np.linalg.norm(xo[:2])) / np.linalg.norm(xo[:2]),
            "speed_rel": abs(np.linalg.norm(ug) - np.linalg.norm(uo)) / np.linalg.norm(uo),
        }
    return out


def drift_velocity(gpu):
    B, E, spo, orbits = 1.0, (2e5, 0.0, 0.0), 100, 4
    v = {}
    for name, prec, be in (("fp32", abi.PREC_MIXED, gpu), ("oracle", abi.PREC_FP64, pyoracle.OracleBackend(1))):
        case = cases.magnetic_rotation(Mesh, pusher=abi.PUSHER_BORIS, precision=prec, beta=0.01, B=B, E=E,
                                       steps_per_orbit=spo)
        sim = cases.build(case, backend=be)
        m = Mesh(case.mesh)
        sim.step(spo)
        tet, bary, _ = sim.get_particles(0)
        x1 = m.position(tet, bary)[0]
        sim.step(spo * (orbits - 1))
        tet, bary, _ = sim.get_particles(0)
        x2 = m.position(tet, bary)[0]
        v[name] = (x2 - x1) / ((orbits - 1) * spo * case.meta["dt"])
    vd = E[0] / B
    return {"expected_m_per_s": vd, "oracle": list(v["oracle"]), "fp32": list(v["fp32"]),
            "fp32_minus_oracle_rel": float(np.abs(v["fp32"] - v["oracle"]).max() / vd)}


if __name__ == "__main__":
    g = GpuBackend()
    print(json.dumps({"energy_drift": energy_drift(g), "gyro": gyro(g), "drift_velocity": drift_velocity(g)},
                     indent=1), flush=True)
