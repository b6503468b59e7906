"""The C++ run-time selection header include/picgpu_rts.hpp (no GPU): every
picFoam TypeName of the GPU path's model families is registered and writes
its choice into picgpu_config, and an unknown TypeName is refused with the
list of valid ones (as OpenFOAM's run-time selection does)."""
import shutil
import subprocess

import pytest

from picfoam_gb300 import abi
from picfoam_gb300.build import INCLUDE

PROBE = r"""
#include <cstdio>
#include "picgpu_rts.hpp"
using namespace picgpu::rts;
int main() {
    picgpu_config c{};
    const char* fams[] = {"ParticlePusher", "FieldWeigthing", "ChargeDistribution", "MaxwellSolver",
                          "CoulombCollisionModel", "PairingAlgorithm", "WeightCorrectionModel",
                          "IonizationModel", "ParticleMerging", "BinaryCollisionModel"};
    for (const char* f : fams) {
        std::printf("%s:", f);
        for (const auto& t : types(f)) std::printf(" %s", t.c_str());
        std::printf("\n");
    }
    select(c, "ParticlePusher", "HigueraCary");
    select(c, "FieldWeigthing", "CellAverage");
    select(c, "ChargeDistribution", "VolumeWeighting");
    select(c, "MaxwellSolver", "ElectroStatic");
    select(c, "CoulombCollisionModel", "Perez");
    select(c, "PairingAlgorithm", "TakizukaAbe");
    select(c, "WeightCorrectionModel", "SentokuKempNR");
    select(c, "IonizationModel", "Perez");
    select(c, "ParticleMerging", "PairMerging");
    std::printf("cfg %d %d %d %d %d %d %d %d %d %d\n", c.pusher, c.field_weighting, c.charge_distribution,
                c.maxwell_solver, c.coulomb.enabled, c.coulomb.collide, c.coulomb.pairing,
                c.coulomb.weight_correction, c.perez.enabled, c.merging.enabled);
    try {
        select(c, "ParticlePusher", "Leapfrog");
    } catch (const std::invalid_argument& e) {
        std::printf("refused: %s\n", e.what());
    }
    return 0;
}
"""


def test_rts_tables(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "probe.cpp"
    src.write_text(PROBE)
    exe = tmp_path / "probe"
    subprocess.run([cxx, "-std=c++17", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    fams = dict(line.split(":", 1) for line in out if ":" in line and not line.startswith("refused"))
    assert fams["ParticlePusher"].split() == sorted(["none", "Boris", "BorisNR", "Vay", "HigueraCary"])
    assert fams["FieldWeigthing"].split() == ["CellAverage", "VolumeWeighting"]
    assert fams["CoulombCollisionModel"].split() == ["Nanbu", "Perez", "none"]
    assert fams["WeightCorrectionModel"].split() == ["Nanbu", "SentokuKemp", "SentokuKempNR", "none"]
    cfg = [int(x) for x in next(line for line in out if line.startswith("cfg ")).split()[1:]]
    assert cfg == [abi.PUSHER_HIGUERA_CARY, abi.WEIGHTING_CELL_AVERAGE, abi.WEIGHTING_VOLUME,
                   abi.MAXWELL_ELECTROSTATIC, 1, abi.COLLIDE_PEREZ, abi.PAIRING_TAKIZUKA_ABE, 2, 1, 1]
    refused = next(line for line in out if line.startswith("refused"))
    assert "Leapfrog" in refused and "HigueraCary" in refused


def test_rts_driver_builds_and_prints_usage():
    from picfoam_gb300 import build
    build.build()
    r = subprocess.run([build.DRIVER], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2
    assert "Family=TypeName" in r.stderr
