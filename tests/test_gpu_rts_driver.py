"""The compiled C++ host (picgpu_rts_driver over picgpu_rts.hpp) against
the Python host, on the GPU: the same case with the sub-models chosen by
their picFoam TypeNames in the driver and by the config fields in Python
gives the same parcels, bit for bit (FP32 store with fixed-point deposits,
so both runs are deterministic), and the same step statistics.  An unknown
TypeName is refused before any GPU work."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from picfoam_gb300 import abi, cases

pytestmark = pytest.mark.gpu

SELECT = [("ParticlePusher", "Vay", "pusher", abi.PUSHER_VAY),
          ("FieldWeigthing", "CellAverage", "field_weighting", abi.WEIGHTING_CELL_AVERAGE),
          ("ChargeDistribution", "VolumeWeighting", "charge_distribution", abi.WEIGHTING_VOLUME)]


def write_case(path, case):
    with open(path, "wb") as f:
        f.write(bytes(case.mesh))
        f.write(bytes(case.cfg))
        for s in range(case.cfg.n_species):
            tet, bary, U = case.particles[s]
            f.write(np.int64(len(tet)).tobytes())
            f.write(np.ascontiguousarray(tet, dtype=np.int32).tobytes())
            f.write(np.ascontiguousarray(bary, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(U, dtype=np.float64).tobytes())


def read_result(path, n_species):
    raw = open(path, "rb").read()
    k = ctypes.sizeof(abi.StepStats)
    st = abi.StepStats.from_buffer_copy(raw[:k])
    parts = []
    for _ in range(n_species):
        n = int(np.frombuffer(raw, np.int64, 1, k)[0])
        k += 8
        tet = np.frombuffer(raw, np.int32, n, k)
        k += 4 * n
        bary = np.frombuffer(raw, np.float64, 3 * n, k).reshape(n, 3)
        k += 24 * n
        U = np.frombuffer(raw, np.float64, 3 * n, k).reshape(n, 3)
        k += 24 * n
        parts.append((tet, bary, U))
    return st, parts


def driver():
    from picfoam_gb300 import build
    build.build()
    assert os.path.exists(build.DRIVER)
    return build.DRIVER


def test_rts_driver_matches_python_host(gpu, tmp_path):
    exe = driver()
    case = cases.two_species_3d(n_cells=8, per_cell=20, precision=abi.PREC_MIXED,
                                deposit=abi.DEPOSIT_FIXED_POINT)
    steps = 3
    write_case(tmp_path / "case.bin", case)
    args = [exe, str(tmp_path / "case.bin"), str(tmp_path / "out.bin"), str(steps)]
    args += [f"{fam}={name}" for fam, name, _, _ in SELECT]
    r = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for fam, name, _, _ in SELECT:
        assert f"{fam} {name}" in r.stdout
    st_d, parts_d = read_result(tmp_path / "out.bin", case.cfg.n_species)

    for _, _, field, value in SELECT:
        setattr(case.cfg, field, value)
    sim = cases.build(case, backend=gpu)
    sim.initialise_fields()
    for _ in range(steps):
        st_p = sim.step(1)
    assert st_d.pcg_iterations == st_p.pcg_iterations
    for s in range(case.cfg.n_species):
        assert st_d.n_particles[s] == st_p.n_particles[s]
        for a, b in zip(parts_d[s], sim.get_particles(s)):
            np.testing.assert_array_equal(a, b)
    sim.close()


def test_rts_driver_refuses_unknown_typename(gpu, tmp_path):
    exe = driver()
    case = cases.two_species_3d(n_cells=4, per_cell=2)
    write_case(tmp_path / "case.bin", case)
    r = subprocess.run([exe, str(tmp_path / "case.bin"), str(tmp_path / "out.bin"), "1",
                        "ParticlePusher=Leapfrog"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "Leapfrog" in r.stderr and "HigueraCary" in r.stderr
    assert not (tmp_path / "out.bin").exists()
