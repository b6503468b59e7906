"""picFoam case directories (no GPU): the FoamFile reader, a case written
here mapped onto the configuration (a block whose local axes are permuted
and reversed, boundary models, initial conditions), the cell-order map
against blockMesh's numbering, the polyMesh writer's conventions, time
directories written from an oracle run and read back, and the reference's
own tutorial cases (when the reference tree is present)."""
import math
import os

import numpy as np
import pytest

from picfoam_gb300 import abi, cases, foam, ofcase
from picfoam_gb300.simulation import Mesh

HEADER = 'FoamFile\n{\n    version 2.0;\n    format ascii;\n    class dictionary;\n    object %s;\n}\n'


def test_parser_forms():
    d = foam.parse(HEADER % "x" + r'''
/* block
   comment */
a 1;            // trailing
b 2.5e-3;
c "a b;c";
dims [0 2 -1 0 0 0 0];
list (e "Ar+" 3 (1 2 3));
counted 3(4 5 6);
field nonuniform List<scalar> 2(1.5 2.5);
models ( "x|y" { type T; TCoeffs { k (0 0 1); } } z { type none; } );
#include "other"
nested { inner { deep true; } }
unclosed { v 1;
''')
    assert d["a"] == 1 and d["b"] == 2.5e-3 and d["c"] == "a b;c"
    assert list(d["dims"]) == [0, 2, -1, 0, 0, 0, 0]
    assert d["list"] == ["e", "Ar+", [1, 2, 3]]         # "3 (1 2 3)" is a counted list
    assert d["counted"] == [4, 5, 6]
    assert foam.numeric_list(d["field"]).tolist() == [1.5, 2.5]
    (n1, m1), (n2, m2) = d["models"]
    assert n1 == "x|y" and m1["type"] == "T" and m1.sub("TCoeffs")["k"] == [0, 0, 1] and n2 == "z"
    assert d.sub("nested").sub("inner").flag("deep")
    assert d["#include"] == "other"
    assert d.sub("unclosed")["v"] == 1


def write(path, rel, text):
    f = os.path.join(path, rel)
    os.makedirs(os.path.dirname(f), exist_ok=True)
    with open(f, "w") as fh:
        fh.write(HEADER % os.path.basename(rel) + text)


def make_case(path, pusher="Boris", injection=True, merging=False):
    """A 6 x 4 x 5 block whose local axes are x1 = -y, x2 = -z, x3 = +x
    (injection=False leaves the SimpleInjection of the source patch out;
    merging=True merges both species' parcels in cells of more than 900)."""
    merge = ("""PairMerging;
PairMergingCoeffs { species (e Ar+); nDeviation (5e3 5e3); reductionFactor 0.9; cellParcelsMax 900; maxChecks 300;
                    nCheckNeighbors 6; angleDifference 20; velocityRatio 0.6; mergeMaximumPerCell 40; }"""
             if merging else "none;")
    source = ("""source { type SimpleInjection; SimpleInjectionCoeffs { frequencies (1e15 2e14); injectionEndTime 1;
                     eV (2 0.1); injectionTypeIds (e Ar+); velocityModel halfMaxwellianFlux;
                     interactions { e { type deletion; } Ar+ { type deletion; } } } }"""
              if injection else "")
    write(path, "system/blockMeshDict", """
convertToMeters 0.001;
vertices ((0 4 5) (0 0 5) (0 0 0) (0 4 0) (6 4 5) (6 0 5) (6 0 0) (6 4 0));
blocks ( hex (0 1 2 3 4 5 6 7) (4 5 6) simpleGrading (1 1 1) );
edges ();
boundary
(
    source { type patch; faces ((3 0 1 2)); }
    collector { type patch; faces ((4 5 6 7)); }
    walls { type wall; faces ((3 0 4 7) (6 5 1 2)); }
    sides { type patch; faces ((0 1 5 4) (7 6 2 3)); }
);
mergePatchPairs ();
""")
    write(path, "0/phiE", """
dimensions [1 2 -3 0 0 -1 0];
internalField uniform 0;
boundaryField
{
    source { type fixedValue; value uniform 10; }
    collector { type circuitBoundary; value uniform 0; }
    walls { type zeroGradient; }
    sides { type fixedValue; value uniform 0; }
}
""")
    write(path, "0/B", "dimensions [1 0 -2 0 0 -1 0];\ninternalField uniform (0 0 0.02);\n")
    write(path, "constant/picProperties", f"""
SolverSettings {{ typeIdList (e Ar+); ChargeDistribution VolumeWeighting; FieldWeigthing CellAverage;
                 spaceCharge 1e-12; }}
moleculeProperties
{{
    e {{ mass 9.109e-31; charge -1.602176e-19; solveMovement true; nEquivalentParticles 1e3; }}
    Ar+ {{ mass 6.6335e-26; charge 1.602176e-19; solveMovement true; nEquivalentParticles 1e3; }}
    SpeciesRelations {{ electronTypeId e; }}
}}
BoundaryModels
{{
    WallReflectionModel SpecularReflection;
    PatchEventModels {{ modelList (); }}
    PatchBoundaryModels
    {{
        modelList
        (
            {source}
            collector {{ type FloatingPotential; }}
        );
    }}
}}
MaxwellSolver ElectroStatic;
ParticlePusher {pusher};
CollisionModels {{ BackgroundGasModel none; ElectronNeutralCollisionModel none; BinaryCollisionModel none;
                  CoulombCollisionModel none; IonNeutralCollisionModel none; }}
ParticleMerging {merge}
""")
    write(path, "system/controlDict", "deltaT 1e-12;\nendTime 4e-12;\nwriteInterval 2e-12;\n")
    write(path, "system/fvSolution", "solvers { phiE { solver PCG; preconditioner DIC; tolerance 1e-9; relTol 0; } }\n")
    write(path, "system/picInitialiseDict", """
numberDensities { e 1e15; Ar+ 1e15; }
InitializationModel Maxwellian;
MaxwellianCoeffs { e { driftVelocity (1e4 0 0); thermalVelocity (4e5 4e5 4e5); }
                   Ar+ { driftVelocity (0 0 0); thermalVelocity (300 300 300); } }
solveMaxwellEquations true;
initalizeLeapFrog true;
clearParticles true;
""")


def test_case_mapping(tmp_path):
    make_case(str(tmp_path))
    c = ofcase.load_case(str(tmp_path))
    assert list(c.mesh.n) == [6, 4, 5]
    assert list(c.mesh.origin) == pytest.approx([0, 0, 0]) and list(c.mesh.length) == pytest.approx([6e-3, 4e-3, 5e-3])
    assert c.side_names == ["source", "collector", "walls", "walls", "sides", "sides"]
    kinds = [c.mesh.side[s].kind for s in range(6)]
    assert kinds == [abi.PATCH_ABSORB, abi.PATCH_FLOATING, abi.PATCH_WALL, abi.PATCH_WALL,
                     abi.PATCH_ABSORB, abi.PATCH_ABSORB]
    assert c.mesh.side[0].phi_bc == abi.PHI_FIXED_VALUE and c.mesh.side[0].phi == 10.0
    assert c.mesh.side[2].phi_bc == abi.PHI_ZERO_GRADIENT and c.mesh.side[4].phi_bc == abi.PHI_FIXED_VALUE
    cfg = c.cfg
    assert cfg.charge_distribution == abi.WEIGHTING_VOLUME and cfg.field_weighting == abi.WEIGHTING_CELL_AVERAGE
    assert cfg.space_charge == 1e-12 and list(cfg.B) == [0, 0, 0.02] and cfg.dt == 1e-12
    assert cfg.pcg_tol == 1e-9 and cfg.pcg_precond == abi.PRECOND_JACOBI and cfg.electron_species == 0
    assert cfg.species[0].weight == 1e3 and cfg.species[1].mass == 6.6335e-26
    (q,) = c.injections
    assert q.patch == 0 and q.velocity_model == abi.EMIT_HALF_MAXWELLIAN_FLUX and list(q.frequency[:2]) == [1e15, 2e14]
    assert c.init.model == abi.INIT_MAXWELLIAN and c.init.leapfrog == 1 and c.init.solve_fields == 1
    assert list(c.init.drift_velocity[0]) == [1e4, 0, 0] and c.init.thermal_velocity[1][2] == 300
    assert c.write_interval == 2e-12 and c.end_time == 4e-12


def test_cell_order_matches_blockmesh_numbering(tmp_path):
    make_case(str(tmp_path))
    c = ofcase.load_case(str(tmp_path))
    # blockMesh cell (i1, i2, i3), x1 fastest, centre v0 + (i + 1/2) along the local axes
    v0 = np.array([0, 4, 5]) * 1e-3
    e = [np.array([0, -1, 0]) * 1e-3, np.array([0, 0, -1]) * 1e-3, np.array([1, 0, 0]) * 1e-3]
    nl = (4, 5, 6)
    centres = np.array([v0 + (i + .5) * e[0] + (j + .5) * e[1] + (k + .5) * e[2]
                        for k in range(nl[2]) for j in range(nl[1]) for i in range(nl[0])])
    cc, _ = Mesh(c.mesh).cells()
    np.testing.assert_allclose(cc[c.cell_order], centres, atol=1e-15)


def test_poly_mesh_conventions(tmp_path):
    make_case(str(tmp_path))
    c = ofcase.load_case(str(tmp_path))
    d = ofcase.write_poly_mesh(c)
    pts = _list_file(os.path.join(d, "points"))
    faces = _list_file(os.path.join(d, "faces")).astype(int)
    owner = _list_file(os.path.join(d, "owner")).astype(int)
    neigh = _list_file(os.path.join(d, "neighbour")).astype(int)
    nc, ni = 6 * 4 * 5, len(neigh)
    assert len(pts) == 7 * 5 * 6 and ni == 5 * 4 * 5 + 6 * 3 * 5 + 6 * 4 * 4
    assert len(faces) == ni + 2 * (4 * 5 + 6 * 5 + 6 * 4)
    assert np.all(owner[:ni] < neigh)
    assert np.all(np.diff(owner[:ni] * nc + neigh) > 0)           # upper-triangular order
    assert np.bincount(np.concatenate([owner, neigh]), minlength=nc).tolist() == [6] * nc
    cc = np.zeros((nc, 3))
    for f, o in enumerate(owner):
        cc[o] += pts[faces[f]].mean(axis=0) / 6
    for f, nb in enumerate(neigh):
        cc[nb] += pts[faces[f]].mean(axis=0) / 6
    for f in range(len(faces)):
        p = pts[faces[f]]
        nrm = np.cross(p[1] - p[0], p[2] - p[1])
        ref = (cc[neigh[f]] if f < ni else p.mean(axis=0)) - cc[owner[f]]
        assert nrm @ ref > 0
    b = foam.read(os.path.join(d, "boundary"))
    assert b is not None


def _list_file(path):
    """The list that follows the header of a polyMesh / lagrangian file."""
    (lst,) = [v for k, v in foam.read(path).items() if k != "FoamFile"]
    return np.asarray(lst, dtype=np.float64)


def test_cyclic_halves_match(tmp_path):
    case = cases.empty_case(n_cells=(3, 4, 2), sides=[cases.patch(abi.PATCH_CYCLIC)] * 6)
    c = ofcase.OFCase(path=str(tmp_path), mesh=case.mesh, cfg=case.cfg, species=["e", "Ar+"],
                      side_names=["l", "r", "lo", "up", "b", "f"],
                      patches={k: [i] for i, k in enumerate(["l", "r", "lo", "up", "b", "f"])},
                      patch_types={k: "cyclic" for k in ["l", "r", "lo", "up", "b", "f"]}, phi_bc={},
                      cell_order=np.arange(24))
    d = ofcase.write_poly_mesh(c)
    pts = _list_file(os.path.join(d, "points"))
    faces = _list_file(os.path.join(d, "faces")).astype(int)
    ni = len(_list_file(os.path.join(d, "neighbour")))
    start = ni
    centres = {}
    for name, cnt in zip(["l", "r", "lo", "up", "b", "f"], [8, 8, 6, 6, 12, 12]):
        centres[name] = pts[faces[start:start + cnt]].mean(axis=1)
        start += cnt
    for a, (lo, hi) in enumerate((("l", "r"), ("lo", "up"), ("b", "f"))):
        other = [x for x in range(3) if x != a]
        np.testing.assert_allclose(centres[lo][:, other], centres[hi][:, other])
    assert "neighbourPatch  r;" in open(os.path.join(d, "boundary")).read()


def test_time_directory_round_trip(tmp_path, oracle_backend):
    make_case(str(tmp_path))
    c = ofcase.load_case(str(tmp_path))
    sim = c.build(backend=oracle_backend.OracleBackend(1))
    sim.step(2)
    d = ofcase.write_fields(sim, c, 2e-12)
    assert os.path.basename(d) == "2e-12"
    np.testing.assert_array_equal(ofcase.read_field(os.path.join(d, "phiE")), sim.field(abi.FIELD_PHI)[c.cell_order])
    np.testing.assert_array_equal(ofcase.read_field(os.path.join(d, "E")),
                                  sim.field(abi.FIELD_E_CELL).reshape(-1, 3)[c.cell_order])
    tid = _list_file(os.path.join(d, "lagrangian", "pic", "typeId"))
    assert (tid == 0).sum() == sim.count(0) and (tid == 1).sum() == sim.count(1)
    phi = foam.read(os.path.join(d, "phiE"))["boundaryField"]
    assert phi["source"]["value"] == ("uniform", 10.0) and phi["walls"]["type"] == "zeroGradient"


# picFoam's tutorials directory (PICFOAM_TUTORIALS=<picFoam source>/tutorials)
REF = os.environ.get("PICFOAM_TUTORIALS", "")


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PICFOAM_TUTORIALS is not set to picFoam's tutorials")
@pytest.mark.parametrize("name,strict", [("plasmaOscillation", True), ("rlcCircuit", True), ("thermalization", True),
                                         ("thermalization_binaryCollision", True), ("floatingBoundary", False),
                                         ("ionization", True), ("magneticRotation", True),
                                         ("electricAcceleration", False)])
def test_reference_tutorials_load(name, strict):
    c = ofcase.load_case(os.path.join(REF, name), allow_unsupported=not strict)
    assert (not c.unsupported) == strict
    if name == "rlcCircuit":
        assert c.cfg.circuit.model == abi.CIRCUIT_RLC and list(c.mesh.n) == [200, 1, 1]
        assert c.cfg.circuit.C == 1e-6 and c.cfg.circuit.L == 0.04 and c.cfg.circuit.V == 100
        assert c.mesh.side[0].phi_bc == abi.PHI_RLC and c.init.model == abi.INIT_MAXWELLIAN
    if name == "plasmaOscillation":
        assert all(c.mesh.side[s].kind == abi.PATCH_CYCLIC for s in range(6))
        assert c.init.model == abi.INIT_UNIFORM_DISPLACEMENT
    if name == "thermalization":
        assert c.cfg.coulomb.enabled and c.cfg.coulomb.collide == abi.COLLIDE_PEREZ and c.cfg.coulomb.coulomb_log == 15
    if name == "thermalization_binaryCollision":
        assert c.cfg.binary.enabled and c.cfg.binary.weight_correction == abi.WEIGHT_CORRECTION_NANBU
    if name == "ionization":
        mc = c.cfg.mcc
        assert mc.enabled and mc.neutral_parcels and c.species[mc.neutral_species] == "Ar"
        assert c.species[mc.ion_species] == "Ar+" and mc.iz_threshold == 15.76 and mc.scatter == 1
        assert mc.xs_ionization[0] == 3.43943e-20 and mc.xs_elastic[0] == 0.0 and mc.find_max_energy == 500
    if name == "floatingBoundary":
        assert c.mesh.side[1].kind == abi.PATCH_FLOATING and len(c.injections) == 1


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PICFOAM_TUTORIALS is not set to picFoam's tutorials")
def test_reference_gmsh_case_is_refused():
    with pytest.raises(ofcase.UnsupportedCase):
        ofcase.load_case(os.path.join(REF, "ionDriftVelocity"), allow_unsupported=True)


@pytest.mark.skipif(not REF or not os.path.isdir(REF), reason="PICFOAM_TUTORIALS is not set to picFoam's tutorials")
def test_reference_magnetic_rotation_gyrates(oracle_backend):
    # ParticleList: one electron at 0.1 c in B_z = 1 T; HigueraCary keeps the
    # gyration radius and the speed
    c = ofcase.load_case(os.path.join(REF, "magneticRotation"))
    assert c.particle_list and c.cfg.pusher == abi.PUSHER_HIGUERA_CARY
    sim = c.build(backend=oracle_backend.OracleBackend(1))
    m = Mesh(c.mesh)
    r0 = abs(c.particle_list[0][1][1])
    for _ in range(3):
        sim.step(50)
        t, b, U = sim.get_particles(0)
        x = m.position(t, b)
        assert np.linalg.norm(x[0, :2]) == pytest.approx(r0, rel=1e-7)
        assert np.linalg.norm(U[0]) == pytest.approx(29979246.0, rel=1e-12)


def test_merging_maps_and_restarts_bit_for_bit(oracle_backend, tmp_path):
    """PairMergingCoeffs map onto picgpu_merging, and a run with merging
    written at step 2 and continued from that time directory reproduces the
    uninterrupted run: nParticle and chargeModifier are written per parcel
    and read back (PICParcelIO.C:98-160)."""
    from picfoam_gb300 import run
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    make_case(a, injection=False, merging=True)
    make_case(b, injection=False, merging=True)
    mg = ofcase.load_case(a).cfg.merging
    assert mg.enabled == 1 and mg.n_species == 2 and list(mg.species[:2]) == [0, 1]
    assert (mg.cell_parcels_max, mg.n_check_neighbors, mg.merge_maximum_per_cell) == (900, 6, 40)
    assert mg.reduction_factor == 0.9 and mg.angle_difference == 20 and list(mg.n_deviation[:2]) == [5e3, 5e3]
    assert run.main([a, "--oracle", "--steps", "4"]) == 0
    assert run.main([b, "--oracle", "--steps", "2"]) == 0
    assert run.main([b, "--oracle", "--restart", "--steps", "2"]) == 0
    la, lb = (os.path.join(p, "4e-12", "lagrangian", "pic") for p in (a, b))
    for name in ("picgpuTet", "picgpuBarycentric", "U", "typeId", "nParticle", "chargeModifier"):
        np.testing.assert_array_equal(ofcase.read_list(os.path.join(la, name)),
                                      ofcase.read_list(os.path.join(lb, name)))
    assert ofcase.read_list(os.path.join(la, "nParticle")).max() > 1e3      # merged parcels


def test_restart_continues_bit_for_bit(oracle_backend, tmp_path):
    """startFrom latestTime (PICParcelIO.C:83-120): a run written at step 2
    and continued from that time directory reproduces the uninterrupted run
    -- particles, potential and the floating patch's charge -- bit for bit
    in FP64."""
    from picfoam_gb300 import run
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    make_case(a, injection=False)
    make_case(b, injection=False)
    assert run.main([a, "--oracle", "--steps", "4"]) == 0
    assert run.main([b, "--oracle", "--steps", "2"]) == 0
    assert run.main([b, "--oracle", "--restart", "--steps", "2"]) == 0
    la, lb = (os.path.join(p, "4e-12", "lagrangian", "pic") for p in (a, b))
    for name in ("picgpuTet", "picgpuBarycentric", "U", "typeId"):
        np.testing.assert_array_equal(ofcase.read_list(os.path.join(la, name)),
                                      ofcase.read_list(os.path.join(lb, name)))
    np.testing.assert_array_equal(ofcase.read_field(os.path.join(a, "4e-12", "phiE")),
                                  ofcase.read_field(os.path.join(b, "4e-12", "phiE")))
    sa = foam.read(os.path.join(a, "4e-12", "uniform", "picgpuState"))
    sb = foam.read(os.path.join(b, "4e-12", "uniform", "picgpuState"))
    assert sa["stepIndex"] == sb["stepIndex"] == 4
    np.testing.assert_array_equal(foam.numeric_list(sa["patchSigma"]), foam.numeric_list(sb["patchSigma"]))
    assert np.abs(foam.numeric_list(sa["patchSigma"])).max() > 0      # the collector has charged
