"""picFoam case directories: read a case into a context, write its results.

`load_case(path)` maps an OpenFOAM / picFoam case onto the picgpu C ABI:
- `system/blockMeshDict`: one axis-aligned hex block (simpleGrading 1),
  patches of type patch / wall / cyclic / empty; the block's local axes may
  be any permutation and orientation of x, y, z;
- `0/phiE`: fixedValue, zeroGradient, circuitBoundary, RLCBoundary, cyclic,
  empty; `0/B` and `0/E` uniform values (the magnetic field, and the applied
  field of MaxwellSolver none);
- `constant/picProperties`: SolverSettings (typeIdList, ChargeDistribution,
  FieldWeigthing, spaceCharge), moleculeProperties (with SpeciesRelations'
  electronTypeId), MaxwellSolver, ParticlePusher, BoundaryModels
  (WallReflectionModel SpecularReflection; FloatingPotential,
  SimpleInjection, FreeStream with `0/boundaryT` / `0/boundaryU`,
  circuitRLC, IdealVoltageSource, IdealCurrentSource with their Thermionic
  and FowlerNordheim EmissionModels), CollisionModels
  (ElectronNeutralCollisionModel with neutral parcels and FixedValue cross
  sections, CoulombCollisionModel with its pairing and collide models,
  BinaryCollisionModel IsotropicScattering);
- `system/controlDict` (deltaT, endTime, writeInterval), `system/fvSolution`
  (phiE: tolerance; GAMG selects the multigrid preconditioner),
  `system/picInitialiseDict` (Equipartition, Maxwellian, Isotropization,
  QuasineutralPlasma, UniformDisplacement, ParticleList, none).
Anything else raises `UnsupportedCase` naming it, unless
`allow_unsupported=True` (then it is listed in `OFCase.unsupported` and left
out).

`write_fields` writes a time directory (phiE, E, rhoCharge and the
lagrangian fields U, typeId, chargeModifier, nParticle of cloud "pic",
PICParcelIO.C:107-166) in the case's own cell order; `write_poly_mesh`
writes constant/polyMesh for the block.
"""
import math
import os
from dataclasses import dataclass, field

import numpy as np

from . import abi, cases, foam

E_CHARGE, K_B = cases.E_CHARGE, cases.K_B


class UnsupportedCase(ValueError):
    """The case selects a model or a mesh this loader does not map."""


@dataclass
class OFCase:
    path: str
    mesh: abi.MeshDesc
    cfg: abi.Config
    species: list                        # typeIdList names, in species index order
    side_names: list                     # OpenFOAM patch name of each block side (-x, +x, -y, +y, -z, +z)
    patches: dict                        # OpenFOAM patch name -> list of block sides
    patch_types: dict                    # OpenFOAM patch name -> polyMesh type
    phi_bc: dict                         # OpenFOAM patch name -> phiE boundary dictionary
    cell_order: np.ndarray               # OpenFOAM cell index -> context cell index
    init: object = None                  # abi.Init or None
    injections: list = field(default_factory=list)
    freestreams: list = field(default_factory=list)
    emissions: list = field(default_factory=list)
    delta_t: float = 0.0
    end_time: float = 0.0
    write_interval: float = 0.0
    unsupported: list = field(default_factory=list)
    keepalive: list = field(default_factory=list)   # arrays the config points to
    particle_list: list = field(default_factory=list)  # ParticleList parcels: (species, position, velocity)

    def build(self, backend=None, initialise=True):
        """A Simulation of the case: boundary models attached, picInitialise
        run (when the case has a picInitialiseDict), initial fields solved."""
        from .simulation import Simulation
        sim = Simulation(self.mesh, self.cfg, backend=backend)
        if self.injections:
            sim.set_injection(self.injections)
        if self.freestreams:
            sim.set_freestream(self.freestreams)
        if self.emissions:
            sim.set_emission(self.emissions)
        if initialise and self.particle_list:
            from .simulation import Mesh
            m = Mesh(self.mesh)
            for s in range(len(self.species)):
                mine = [(p, u) for sp, p, u in self.particle_list if sp == s]
                if not mine:
                    continue
                tet, bary = m.locate(np.array([p for p, _ in mine], dtype=np.float64))
                sim.set_particles(s, tet, bary, np.array([u for _, u in mine], dtype=np.float64))
        if initialise and self.init is not None:
            sim.initialise(self.init)
        sim.initialise_fields()
        return sim


def _read_optional(path):
    return foam.read(path) if os.path.exists(path) else foam.Dict()


def _uniform_vector(d):
    """The value of a `uniform (x y z)` internalField, or None."""
    v = d.get("internalField") if d else None
    if isinstance(v, tuple) and len(v) == 2 and v[0] == "uniform" and isinstance(v[1], list):
        return [float(x) for x in v[1]]
    return None


def _uniform_scalar(v):
    if isinstance(v, tuple) and len(v) == 2 and v[0] == "uniform":
        return float(v[1])
    if isinstance(v, (int, float)):
        return float(v)
    return None


class _Unsupported:
    def __init__(self, allow):
        self.allow = allow
        self.items = []

    def __call__(self, what):
        if not self.allow:
            raise UnsupportedCase(what)
        self.items.append(what)


def _block(path):
    """The hex block: grid counts per global axis, origin, lengths, the map
    from OpenFOAM cell index to context cell index, and each boundary
    patch's sides."""
    f = os.path.join(path, "system", "blockMeshDict")
    if not os.path.exists(f):
        raise UnsupportedCase("the case has no system/blockMeshDict (meshes from other generators are not read)")
    d = foam.read(f)
    scale = d.number("convertToMeters", d.number("scale", 1.0))
    verts = np.asarray(d["vertices"], dtype=np.float64) * scale
    blocks = d["blocks"]
    if not isinstance(blocks, list) or blocks.count("hex") != 1:
        raise UnsupportedCase("blockMeshDict: exactly one hex block is supported")
    lists = [b for b in blocks if isinstance(b, list)]
    vid, nloc = [int(x) for x in lists[0]], [int(x) for x in lists[1]]
    if "edgeGrading" in blocks:
        raise UnsupportedCase("blockMeshDict: edgeGrading is not supported")
    if "simpleGrading" in blocks and len(lists) > 2:
        if any(isinstance(x, list) or float(x) != 1.0 for x in lists[2]):
            raise UnsupportedCase("blockMeshDict: only simpleGrading (1 1 1) is supported")
    edges = d.get("edges", [])
    if isinstance(edges, list) and edges:
        raise UnsupportedCase("blockMeshDict: curved edges are not supported")
    P = verts[vid]
    local = [P[1] - P[0], P[3] - P[0], P[4] - P[0]]   # blockMesh local axes x1, x2, x3
    axis, sign = [0, 0, 0], [1, 1, 1]
    for k, e in enumerate(local):
        nz = np.flatnonzero(np.abs(e) > 1e-12 * np.abs(e).max())
        if len(nz) != 1:
            raise UnsupportedCase("blockMeshDict: the block is not aligned with the coordinate axes")
        axis[k] = int(nz[0])
        sign[k] = 1 if e[nz[0]] > 0 else -1
    if sorted(axis) != [0, 1, 2]:
        raise UnsupportedCase("blockMeshDict: degenerate block")
    lo, hi = P.min(axis=0), P.max(axis=0)
    n = [0, 0, 0]
    for k in range(3):
        n[axis[k]] = nloc[k]
    # OpenFOAM's cells: x1 fastest, then x2, then x3 (local indices from vertex 0)
    i1, i2, i3 = np.meshgrid(np.arange(nloc[0]), np.arange(nloc[1]), np.arange(nloc[2]), indexing="ij")
    loc = [i1.transpose(2, 1, 0).ravel(), i2.transpose(2, 1, 0).ravel(), i3.transpose(2, 1, 0).ravel()]
    g = [None, None, None]
    for k in range(3):
        g[axis[k]] = loc[k] if sign[k] > 0 else nloc[k] - 1 - loc[k]
    cell_order = (g[0] + n[0] * (g[1] + n[1] * g[2])).astype(np.int64)
    patches, types = {}, {}
    for name, pd in d.get("boundary", []):
        types[name] = pd.word("type", "patch")
        sides = []
        for quad in pd.get("faces", []):
            q = verts[[int(x) for x in quad]]
            side = None
            for a in range(3):
                if np.allclose(q[:, a], lo[a], atol=1e-12 * (hi[a] - lo[a])):
                    side = 2 * a
                elif np.allclose(q[:, a], hi[a], atol=1e-12 * (hi[a] - lo[a])):
                    side = 2 * a + 1
            if side is None:
                raise UnsupportedCase(f"blockMeshDict: a face of patch {name} is not on the block's surface")
            sides.append(side)
        patches[name] = sides
    return n, lo, hi - lo, cell_order, patches, types


_PUSHERS = {"none": abi.PUSHER_NONE, "Boris": abi.PUSHER_BORIS, "BorisNR": abi.PUSHER_BORIS_NR,
            "Vay": abi.PUSHER_VAY, "HigueraCary": abi.PUSHER_HIGUERA_CARY}
_WEIGHTING = {"CellAverage": abi.WEIGHTING_CELL_AVERAGE, "VolumeWeighting": abi.WEIGHTING_VOLUME}
_EMIT = {"birdMaxwellianFlux": abi.EMIT_BIRD_MAXWELLIAN_FLUX, "mostProbableSpeed": abi.EMIT_MOST_PROBABLE_SPEED,
         "maxwellianFlux": abi.EMIT_MAXWELLIAN_FLUX, "halfMaxwellianFlux": abi.EMIT_HALF_MAXWELLIAN_FLUX}
_INIT = {"none": abi.INIT_NONE, "Equipartition": abi.INIT_EQUIPARTITION, "Maxwellian": abi.INIT_MAXWELLIAN,
         "Isotropization": abi.INIT_ISOTROPIZATION, "QuasineutralPlasma": abi.INIT_QUASINEUTRAL_PLASMA,
         "UniformDisplacement": abi.INIT_UNIFORM_DISPLACEMENT}
_WEIGHT_CORRECTION = {"none": abi.WEIGHT_CORRECTION_NONE, "Nanbu": abi.WEIGHT_CORRECTION_NANBU,
                      "SentokuKempNR": abi.WEIGHT_CORRECTION_SENTOKU_KEMP_NR,
                      "SentokuKemp": abi.WEIGHT_CORRECTION_SENTOKU_KEMP}
_PHI_DIM = "[1 2 -3 0 0 -1 0]"
_E_DIM = "[1 1 -3 0 0 -1 0]"
_RHO_DIM = "[0 -3 1 0 0 1 0]"


def _model_patches(name, patches):
    """Patches a PatchBoundaryModels entry names ("a|b" selects several)."""
    names = [n for n in str(name).strip("()").split("|") if n]
    missing = [n for n in names if n not in patches]
    if missing:
        raise UnsupportedCase(f"BoundaryModels: no patch {missing[0]}")
    return names


def _species_values(d, names, default=0.0):
    """A `{ e 1e15; Ar+ 1e15; }` dictionary as a list in species order."""
    return [float(d.number(n, default)) if isinstance(d, foam.Dict) else default for n in names]


def load_case(path, allow_unsupported=False, precision=abi.PREC_FP64, seed=1234, ionization_model=None):
    """Map a picFoam case directory onto the picgpu configuration (see the
    module docstring for what is read).  ionization_model overrides the
    Coulomb model's IonizationModel entry (e.g. "Perez" to switch on the
    coefficients a case carries)."""
    bad = _Unsupported(allow_unsupported)
    n, origin, length, cell_order, patch_sides, patch_types = _block(path)
    zero = os.path.join(path, "0") if os.path.isdir(os.path.join(path, "0")) else os.path.join(path, "0.org")
    phiE = _read_optional(os.path.join(zero, "phiE"))
    bfield = phiE.sub("boundaryField")
    props = foam.read(os.path.join(path, "constant", "picProperties"))
    control = _read_optional(os.path.join(path, "system", "controlDict"))
    fvsol = _read_optional(os.path.join(path, "system", "fvSolution"))

    # species
    settings = props.sub("SolverSettings")
    names = [str(x) for x in settings.get("typeIdList", [])]
    if not 1 <= len(names) <= abi.MAX_SPECIES:
        raise UnsupportedCase("SolverSettings: typeIdList must name 1..4 species")
    mol = props.sub("moleculeProperties")
    species = []
    for s in names:
        p = mol.sub(s)
        species.append((p.number("mass"), p.number("charge", 0.0), p.number("nEquivalentParticles", 1.0),
                        p.flag("solveMovement", True)))
    rel = mol.sub("SpeciesRelations")
    e_name = rel.word("electronTypeId", "none")
    electron = names.index(e_name) if e_name in names else -1

    dt = control.number("deltaT", 0.0)
    if not dt > 0:
        raise UnsupportedCase("controlDict: deltaT missing")
    maxwell = {"ElectroStatic": abi.MAXWELL_ELECTROSTATIC, "none": abi.MAXWELL_NONE}.get(props.word("MaxwellSolver"))
    if maxwell is None:
        raise UnsupportedCase(f"MaxwellSolver {props.word('MaxwellSolver')}")
    pusher = _PUSHERS.get(props.word("ParticlePusher", "Boris"))
    if pusher is None:
        raise UnsupportedCase(f"ParticlePusher {props.word('ParticlePusher')}")
    cfg = cases.base_config(dt, species, pusher=pusher, precision=precision, deposit=abi.DEPOSIT_FIXED_POINT,
                            maxwell=maxwell, seed=seed, electron_species=electron)
    for key, attr in (("ChargeDistribution", "charge_distribution"), ("FieldWeigthing", "field_weighting")):
        w = _WEIGHTING.get(settings.word(key, "VolumeWeighting"))
        if w is None:
            raise UnsupportedCase(f"SolverSettings: {key} {settings.word(key)}")
        setattr(cfg, attr, w)
    cfg.space_charge = settings.number("spaceCharge", 0.0)
    B = _uniform_vector(_read_optional(os.path.join(zero, "B")))
    if B is not None:
        for a in range(3):
            cfg.B[a] = B[a]
    if maxwell == abi.MAXWELL_NONE:
        Ea = _uniform_vector(_read_optional(os.path.join(zero, "E")))
        if Ea is not None:
            for a in range(3):
                cfg.E_applied[a] = Ea[a]
    solver = fvsol.sub("solvers").sub("phiE")
    if solver:
        cfg.pcg_tol = solver.number("tolerance", 1e-6)
        cfg.pcg_norm = 1                          # OpenFOAM's normalised residual
        if solver.word("solver") == "GAMG" or solver.word("preconditioner") == "GAMG":
            cfg.pcg_precond = abi.PRECOND_MULTIGRID

    # boundary models: patch name -> (kind, phi_bc, phi)
    bm = props.sub("BoundaryModels")
    wall_model = bm.word("WallReflectionModel", "SpecularReflection")
    if wall_model not in ("SpecularReflection", "none"):
        bad(f"WallReflectionModel {wall_model}")
    kinds = {}
    for name, t in patch_types.items():
        kinds[name] = {"cyclic": abi.PATCH_CYCLIC, "empty": abi.PATCH_EMPTY,
                       "wall": abi.PATCH_WALL}.get(t, abi.PATCH_ABSORB)
    injections, freestreams, emission_models = [], [], []
    boundaryT = _read_optional(os.path.join(zero, "boundaryT")).sub("boundaryField")
    boundaryU = _read_optional(os.path.join(zero, "boundaryU")).sub("boundaryField")
    circuit_model, circuit = None, None
    for entry in bm.sub("PatchBoundaryModels").get("modelList", []):
        if not isinstance(entry, tuple):
            continue
        pname, md = entry
        mtype = md.word("type")
        targets = _model_patches(pname, patch_sides)
        coeffs = md.sub(f"{mtype}Coeffs")
        if mtype == "none":
            continue
        if mtype == "FloatingPotential":
            for p in targets:
                kinds[p] = abi.PATCH_FLOATING
        elif mtype == "SimpleInjection":
            model = _EMIT.get(coeffs.word("velocityModel", "maxwellianFlux"))
            if model is None:
                raise UnsupportedCase(f"SimpleInjection velocityModel {coeffs.word('velocityModel')}")
            ids = [str(x) for x in coeffs.get("injectionTypeIds", [])]
            freq = [float(x) for x in coeffs.get("frequencies", [])]
            eV = [float(x) for x in coeffs.get("eV", [])]
            inter = coeffs.sub("interactions")
            itypes = {inter.sub(s).word("type", "deletion") for s in ids}
            if len(itypes) > 1:
                bad("SimpleInjection: different interactions per species on one patch")
            itype = itypes.pop() if itypes else "deletion"
            for s in ids:
                if inter.sub(s).flag("useInitalVelocity", False):
                    bad("SimpleInjection: useInitalVelocity re-emission")
            for p in targets:
                kinds[p] = {"deletion": abi.PATCH_ABSORB, "reflection": abi.PATCH_WALL,
                            "floating": abi.PATCH_FLOATING}.get(itype, abi.PATCH_ABSORB)
                for side in patch_sides[p]:
                    injections.append((side, cases.injection(side, [names.index(s) for s in ids], freq, eV,
                                                            model=model,
                                                            end_time=coeffs.number("injectionEndTime", 1e300))))
        elif mtype == "FreeStream":
            nd = coeffs.sub("numberDensities")
            ids = list(nd.keys())
            for p in targets:
                kinds[p] = abi.PATCH_ABSORB
                T = _uniform_scalar(boundaryT.sub(p).get("value"))
                U = boundaryU.sub(p).get("value")
                U = [float(x) for x in U[1]] if isinstance(U, tuple) and U[0] == "uniform" else [0.0, 0.0, 0.0]
                if T is None:
                    raise UnsupportedCase(f"FreeStream: no uniform boundaryT on patch {p}")
                for side in patch_sides[p]:
                    freestreams.append((side, cases.freestream(side, [names.index(s) for s in ids],
                                                               [nd.number(s) for s in ids], T, velocity=U)))
        elif mtype in ("circuitRLC", "IdealVoltageSource", "IdealCurrentSource"):
            if circuit is not None:
                raise UnsupportedCase("BoundaryModels: more than one circuit model")
            for em_type in coeffs.get("EmissionModels", []) or []:
                emission_models.append((str(em_type), coeffs.sub(f"{em_type}Coeffs")))
            circuit_model = mtype
            circuit = {"coeffs": coeffs, "anode": None, "cathode": None}
            for p in targets:
                role = coeffs.sub(p).word("type")
                if role not in ("anode", "cathode"):
                    raise UnsupportedCase(f"{mtype}: patch {p} is neither anode nor cathode")
                circuit[role] = p
                kinds[p] = abi.PATCH_CIRCUIT
        else:
            bad(f"BoundaryModel {mtype}")
    if bm.sub("PatchEventModels").get("modelList"):
        bad("PatchEventModels")

    # sides
    side_names = [None] * 6
    for name, sides in patch_sides.items():
        for s in sides:
            side_names[s] = name
    if any(x is None for x in side_names):
        raise UnsupportedCase("blockMeshDict: every side of the block must belong to a patch")
    side_patches = []
    for s in range(6):
        name = side_names[s]
        bc = bfield.sub(name)
        t = bc.word("type", "zeroGradient")
        kind = kinds[name]
        phi_bc, phi = abi.PHI_ZERO_GRADIENT, 0.0
        if t == "fixedValue":
            phi_bc, phi = abi.PHI_FIXED_VALUE, _uniform_scalar(bc.get("value")) or 0.0
        elif t == "RLCBoundary":
            phi_bc = abi.PHI_RLC
        elif t == "circuitBoundary" and kind == abi.PATCH_CIRCUIT:
            phi_bc = abi.PHI_CIRCUIT_GRADIENT
        elif t in ("circuitBoundary", "zeroGradient", "cyclic", "empty", "calculated"):
            phi_bc = abi.PHI_ZERO_GRADIENT
        else:
            bad(f"phiE boundary condition {t} on patch {name}")
        if kind == abi.PATCH_FLOATING and t != "circuitBoundary":
            raise UnsupportedCase(f"FloatingPotential on {name} needs the circuitBoundary potential")
        side_patches.append(cases.patch(kind, phi, phi_bc))
    mesh = cases.block_mesh(n, length, side_patches, origin=origin)

    # circuit
    if circuit is not None:
        c = cfg.circuit
        co = circuit["coeffs"]
        c.model = {"circuitRLC": abi.CIRCUIT_RLC, "IdealVoltageSource": abi.CIRCUIT_IDEAL_VOLTAGE,
                   "IdealCurrentSource": abi.CIRCUIT_IDEAL_CURRENT}[circuit_model]
        for role, attr in (("cathode", "cathode_patch"), ("anode", "anode_patch")):
            p = circuit[role]
            if p is None:
                if role == "cathode":
                    raise UnsupportedCase(f"{circuit_model}: no cathode")
                setattr(c, attr, -1)
                continue
            if len(patch_sides[p]) != 1:
                raise UnsupportedCase(f"{circuit_model}: the {role} must be one side of the block")
            setattr(c, attr, patch_sides[p][0])
        c.R, c.L, c.C, c.V = (co.number(k, 0.0) for k in ("R", "L", "C", "V"))
        c.omega = co.number("omega", 0.0)
        c.phase = co.number("phase", math.pi / 2)
        c.epsilon = co.number("epsilon", 0.0)
        c.I, c.J, c.ref_area = co.number("I", -1.0), co.number("J", -1.0), co.number("refArea", 0.0)
        kb = bfield.sub(circuit["cathode"])
        for i, k in enumerate(("Q", "Q1", "Q2", "Q3")):
            c.Q[i] = kb.number(k, 0.0)
        if c.model == abi.CIRCUIT_RLC:
            c.sigma = kb.number("sigma", 0.0)
        elif c.model == abi.CIRCUIT_IDEAL_CURRENT:
            eps0 = 1.0 / (4e-7 * math.pi * 299792458.0 ** 2)
            c.sigma = kb.number("circuitGradient", kb.number("gradient", 0.0)) * eps0

    emissions = []
    for em_type, eco in emission_models:
        if em_type not in ("Thermionic", "FowlerNordheim"):
            bad(f"EmissionModel {em_type}")
            continue
        model = abi.EMISSION_THERMIONIC if em_type == "Thermionic" else abi.EMISSION_FOWLER_NORDHEIM
        emissions.append(cases.emission(cfg.circuit.cathode_patch, model, eco.number("fnW"),
                                        temperature=eco.number("T", 0.0), lambda_r=eco.number("lambdaR", 0.0),
                                        weight=eco.number("nParticle", -1.0)))

    init_dict = _read_optional(os.path.join(path, "system", "picInitialiseDict"))
    keep = []
    _collisions(props.sub("CollisionModels"), cfg, names, mol, bad, init_dict, keep, ionization_model)
    merging = props.word("ParticleMerging", "none")
    if merging == "PairMerging":
        _merging(props.sub("PairMergingCoeffs"), cfg, names)
    elif merging != "none":
        bad(f"ParticleMerging {merging}")

    plist = []
    init = _init(init_dict, names, cfg, seed, bad, plist)
    return OFCase(path=path, mesh=mesh, cfg=cfg, species=names, side_names=side_names, patches=patch_sides,
                  patch_types=patch_types, phi_bc={k: bfield.sub(k) for k in patch_sides},
                  cell_order=cell_order, init=init, injections=[q for _, q in injections],
                  freestreams=[q for _, q in freestreams], emissions=emissions, delta_t=dt, end_time=control.number("endTime", 0.0),
                  write_interval=control.number("writeInterval", 0.0), unsupported=bad.items, keepalive=keep,
                  particle_list=plist)


def _electron_neutral(cm, cfg, names, mol, init_dict, bad, keep):
    """ElectronNeutralCollisionModel with neutral parcels (BackgroundGasModel
    none): one neutral species, FixedValue or none cross sections
    (FixedValueCrossSection.C: the value at every energy, the threshold
    applied by the collision model), FindMaximum start values."""
    model = cm.word("ElectronNeutralCollisionModel", "none")
    if model == "none":
        return
    scatter = {"NanbuElectronNeutral": 0, "RelativisticElectronNeutral": 1}.get(model)
    if scatter is None:
        raise UnsupportedCase(f"ElectronNeutralCollisionModel {model}")
    if cm.word("BackgroundGasModel", "none") != "none":
        bad("ElectronNeutralCollisionModel with a background gas (set picgpu_mcc's gas fields)")
        return
    co = cm.sub("ElectronNeutralCollisionCoeffs")
    if co.word("WeightCorrection", "none") not in ("none", "Nanbu"):
        bad(f"ElectronNeutral WeightCorrection {co.word('WeightCorrection')}")
    xs = co.sub("CrossSectionModels")
    neutrals = [k for k, v in xs.items() if isinstance(v, foam.Dict)]
    if len(neutrals) != 1 or neutrals[0] not in names:
        raise UnsupportedCase("ElectronNeutralCollisionModel: exactly one neutral species is supported")
    nname = neutrals[0]
    d = xs.sub(nname)
    values, thresholds = {}, {}
    for kind in ("Elastic", "Excitation", "Ionization"):
        t = d.word(f"{kind}CrossSection", "none")
        if t == "none":
            values[kind], thresholds[kind] = 0.0, 0.0
        elif t == "FixedValue":
            fc = d.sub(f"{kind}FixedValueCoeffs")
            values[kind], thresholds[kind] = fc.number("value", 0.0), fc.number("threshold", 0.0)
        else:
            raise UnsupportedCase(f"{kind}CrossSection {t} (only FixedValue and none are read from a case)")
    ion_name = None
    for _, rel in mol.sub("SpeciesRelations").items():
        if isinstance(rel, foam.Dict) and rel.word("neutralTypeId") == nname:
            ion_name = rel.word("ionTypeId")
    tables = [np.array([0.0, 1e6]), np.full(2, values["Elastic"]), np.full(2, values["Excitation"]),
              np.full(2, values["Ionization"])]
    tables = [np.ascontiguousarray(a, dtype=np.float64) for a in tables]
    keep.extend(tables)
    import ctypes as C
    mc = cfg.mcc
    mc.enabled = 1
    mc.scatter = scatter
    mc.create_electron = 1 if co.flag("createElectron", True) else 0
    mc.create_ion = 1 if (co.flag("createIon", True) and ion_name in names) else 0
    mc.ion_species = names.index(ion_name) if ion_name in names else -1
    mc.n_xs = 2
    ns = names.index(nname)
    mc.gas_mass = cfg.species[ns].mass
    mc.gas_weight = cfg.species[ns].weight
    mc.ex_threshold = thresholds["Excitation"]
    mc.iz_threshold = thresholds["Ionization"]
    search = init_dict.sub("CrossSectionInitialization").sub("electronNeutral_searchParameter")
    mc.find_max_energy = search.number("maximumEnergy", 1000.0)
    mc.find_energy_step = search.number("energyStep", 0.01)
    mc.xs_energy, mc.xs_elastic, mc.xs_excitation, mc.xs_ionization = [
        a.ctypes.data_as(C.POINTER(C.c_double)) for a in tables]
    mc.neutral_parcels = 1
    mc.neutral_species = ns
    mc.keep_neutrals = 0 if co.flag("deleteNeutral", True) else 1
    mc.keep_neutral_velocity = 0 if co.flag("updateNeutralVelocity", True) else 1
    if co.number("ionization_nEquivalentParticles", 0.0) > 0:
        bad("ionization_nEquivalentParticles (one weight per species)")


def _merging(co, cfg, names):
    """PairMergingCoeffs (PairMerging.C:35-68): species in merge order with
    nDeviation per species, reductionFactor, cellParcelsMax, maxChecks,
    nCheckNeighbors, angleDifference [deg], velocityRatio,
    mergeMaximumPerCell."""
    species = [str(x) for x in co.get("species", [])]
    dev = [float(x) for x in co.get("nDeviation", [])]
    if not species or len(dev) != len(species) or any(s not in names for s in species):
        raise UnsupportedCase("PairMerging: species must be defined and nDeviation give one value per species")
    cases.set_merging(cfg, [names.index(s) for s in species],
                      cell_parcels_max=int(co.number("cellParcelsMax")), reduction_factor=co.number("reductionFactor"),
                      max_checks=int(co.number("maxChecks")), n_check_neighbors=int(co.number("nCheckNeighbors")),
                      angle_difference=co.number("angleDifference"), velocity_ratio=co.number("velocityRatio"),
                      n_deviation=dev, merge_maximum_per_cell=int(co.number("mergeMaximumPerCell")))


def _perez(coeffs, cfg, names):
    """PerezIonizationCoeffs (PerezIonizationModel.C:50-116): one entry per
    ion species with atomicNumber, the optional ionizationLimit and the
    bindingEnergy / ionizationEnergy lists [eV]."""
    pz = cfg.perez
    pz.enabled = 1
    k = 0
    for _, d in coeffs.items():
        if not isinstance(d, foam.Dict):
            continue
        ion = str(d.word("ionSpecies"))
        if ion not in names:
            raise UnsupportedCase(f"PerezIonization: ionSpecies {ion} is not defined")
        if k >= abi.PEREZ_MAX_IONS:
            raise UnsupportedCase(f"PerezIonization: more than {abi.PEREZ_MAX_IONS} ion species")
        A = int(d.number("atomicNumber"))
        binding = [float(x) for x in d.get("bindingEnergy", [])]
        energy = [float(x) for x in d.get("ionizationEnergy", [])]
        if not 1 <= A <= abi.PEREZ_MAX_Z or len(binding) != A or len(energy) != A:
            raise UnsupportedCase("PerezIonization: bindingEnergy and ionizationEnergy need atomicNumber entries")
        e = pz.ion[k]
        e.species = names.index(ion)
        e.atomic_number = A
        limit = d.number("ionizationLimit", None)
        e.ionization_limit = -1 if limit is None else int(limit)
        for i in range(A):
            e.binding_energy[i] = binding[i]
            e.ionization_energy[i] = energy[i]
        k += 1
    pz.n_ions = k


def _collisions(cm, cfg, names, mol, bad, init_dict=None, keep=None, ionization_model=None):
    """CollisionModels: electron-neutral collisions with neutral parcels
    (FixedValue cross sections), Coulomb (fixed or computed coulombLog) and
    binary IsotropicScattering map; background-gas MCC and ion-neutral
    collisions are set through picgpu_mcc / picgpu_ion_mcc."""
    _electron_neutral(cm, cfg, names, mol, init_dict if init_dict is not None else foam.Dict(), bad,
                      keep if keep is not None else [])
    if cm.word("IonNeutralCollisionModel", "none") != "none":
        bad(f"IonNeutralCollisionModel {cm.word('IonNeutralCollisionModel')} "
            "(cross sections are set through picgpu_ion_mcc)")
    coul = cm.word("CoulombCollisionModel", "none")
    if coul != "none":
        co = cm.sub("CoulombCollisionCoeffs")
        c = cfg.coulomb
        c.enabled = 1
        c.collide = {"Nanbu": abi.COLLIDE_NANBU, "Perez": abi.COLLIDE_PEREZ}.get(coul, -1)
        if c.collide < 0:
            raise UnsupportedCase(f"CoulombCollisionModel {coul}")
        c.pairing = {"NanbuYonemura": abi.PAIRING_NANBU_YONEMURA,
                     "TakizukaAbe": abi.PAIRING_TAKIZUKA_ABE}.get(co.word("pairingAlgorithm", "NanbuYonemura"), -1)
        if c.pairing < 0:
            raise UnsupportedCase(f"pairingAlgorithm {co.word('pairingAlgorithm')}")
        wc = _WEIGHT_CORRECTION.get(co.word("WeightCorrection", "none"))
        if wc is None:
            raise UnsupportedCase(f"WeightCorrection {co.word('WeightCorrection')}")
        c.weight_correction = wc
        c.allow_intra = 1 if co.flag("allowIntraCollision", True) else 0
        c.calculate_bmin = 1 if co.flag("calculateBmin", False) else 0
        logs = {float(d.number("coulombLog", 0.0)) for _, d in co.sub("Collisions").items()
                if isinstance(d, foam.Dict)}
        if len(logs) > 1:
            bad("CoulombCollisionCoeffs: different coulombLog per pair (one value is used)")
        c.coulomb_log = max(logs) if logs else 0.0
        model = ionization_model or co.word("IonizationModel", "none")
        if model == "Perez":
            _perez(co.sub("PerezIonizationCoeffs"), cfg, names)
        elif model != "none":
            bad(f"IonizationModel {model}")
    binary = cm.word("BinaryCollisionModel", "none")
    if binary != "none":
        if binary != "IsotropicScattering":
            raise UnsupportedCase(f"BinaryCollisionModel {binary}")
        co = cm.sub("IsotropicScatteringCoeffs")
        b = cfg.binary
        b.enabled = 1
        b.cross_section = {"HardSphere": abi.XS_HARD_SPHERE,
                           "VariableHardSphere": abi.XS_VARIABLE_HARD_SPHERE}.get(
            co.word("TotalCrossSectionModel", "HardSphere"), -1)
        if b.cross_section < 0:
            raise UnsupportedCase(f"TotalCrossSectionModel {co.word('TotalCrossSectionModel')}")
        wc = _WEIGHT_CORRECTION.get(co.word("WeightCorrection", "none"))
        if wc is None:
            raise UnsupportedCase(f"WeightCorrection {co.word('WeightCorrection')}")
        b.weight_correction = wc
        # IsotropicScatteringCoeffs handleChargeExchange (a tutorial entry)
        # is read by none of picFoam's collision code, so it is ignored here
        vhs = cm.sub("VariableHardSphereCoeffs")
        b.tref = vhs.number("Tref", 273.0)
        b.background_species = -1
        for i, s in enumerate(names):
            b.diameter[i] = mol.sub(s).number("diameter", 0.0)
            b.omega[i] = mol.sub(s).number("omega", 0.5)
    if cm.word("BackgroundGasModel", "none") != "none" and binary != "none":
        bad("BinaryCollisionModel with a background gas (set picgpu_binary.background_species)")


def _init(d, names, cfg, seed, bad, plist=None):
    """system/picInitialiseDict as an abi.Init (None without the file).  A
    ParticleList (ParticleListInitialization: one parcel per entry, species,
    position, velocity) goes to plist as (species, position, velocity) and
    the Init places nothing, then applies the leapfrog and field settings to
    the listed parcels."""
    if not d:
        return None
    model = d.word("InitializationModel", "none")
    if model == "ParticleList" and plist is not None:
        for _, e in d.sub("ParticleListCoeffs").items():
            if not isinstance(e, foam.Dict):
                continue
            if e.number("temperature", 0.0) != 0.0:
                bad("ParticleList: a parcel with a temperature (thermal spread)")
            sp = str(e.word("species"))
            if sp not in names:
                raise UnsupportedCase(f"ParticleList: no species {sp}")
            plist.append((names.index(sp), [float(x) for x in e["position"]],
                          [float(x) for x in e.get("velocity", [0, 0, 0])]))
        return cases.init_config(abi.INIT_NONE, seed=seed, clear=False,
                                 solve_fields=d.flag("solveMaxwellEquations", False),
                                 leapfrog=d.flag("initalizeLeapFrog", False))
    code = _INIT.get(model)
    if code is None:
        bad(f"InitializationModel {model}")
        return None
    co = d.sub(f"{model}Coeffs")
    ev = d.flag("electronVolt", False)
    kw = {}
    if model == "Equipartition":
        kw["velocity"] = [float(x) for x in co.get("velocity", [0, 0, 0])]
    elif model == "Maxwellian":
        kw["drift_velocity"] = [[float(x) for x in co.sub(s).get("driftVelocity", [0, 0, 0])] for s in names]
        kw["thermal_velocity"] = [[float(x) for x in co.sub(s).get("thermalVelocity", [0, 0, 0])] for s in names]
    elif model == "Isotropization":
        kw["tperp_over_tpara"] = co.number("Tperp_over_Tpara", 1.0)
    elif model == "QuasineutralPlasma":
        kw["cell_count"] = co.number("cellCount", 0.0)
        ion = co.word("ionSpecies")
        kw["ion_species"] = names.index(ion) if ion in names else -1
        kw["use_maxwellian"] = co.flag("useMaxwellian", True)
    elif model == "UniformDisplacement":
        kw["species"] = [names.index(str(s)) for s in co.get("species", [])]
        for k, key in (("min", "min"), ("max", "max"), ("displacement_dir", "displacementDir")):
            if key in co:
                kw[k] = [float(x) for x in co[key]]
        kw["particle_numbers"] = [int(x) for x in co.get("particleNumbers", [1, 1, 1])]
        kw["cycles"] = co.number("cycles", 1.0)
        disp = co.get("displacement", [])
        disp = disp if isinstance(disp, list) else [disp]
        sp = kw["species"]
        kw["displacement"] = [float(disp[sp.index(s)]) if s in sp and sp.index(s) < len(disp) else 0.0
                              for s in range(len(names))]
    return cases.init_config(code, seed=seed, number_density=_species_values(d.get("numberDensities"), names),
                             temperature=_species_values(d.get("temperature"), names),
                             clear=d.flag("clearParticles", True), solve_fields=d.flag("solveMaxwellEquations", False),
                             leapfrog=d.flag("initalizeLeapFrog", False), electron_volt=ev, **kw)


# ----------------------------------------------------------------- output --
def time_name(t):
    """OpenFOAM's `timeFormat general; timePrecision 6` directory name."""
    return "%.6g" % t


def _ctx_ijk(case):
    n = list(case.mesh.n)
    c = np.arange(n[0] * n[1] * n[2], dtype=np.int64)
    return c % n[0], (c // n[0]) % n[1], c // (n[0] * n[1])


def _of_of_ctx(case):
    inv = np.empty_like(case.cell_order)
    inv[case.cell_order] = np.arange(len(case.cell_order))
    return inv


def side_owner_cells(case, side):
    """OpenFOAM cell indices of the cells owning the faces of a block side,
    in blockMesh's face order (rising owner index)."""
    n = list(case.mesh.n)
    ijk = _ctx_ijk(case)
    a, hi = side // 2, side % 2
    on = ijk[a] == (n[a] - 1 if hi else 0)
    return np.sort(_of_of_ctx(case)[np.flatnonzero(on)])


def _patch_owner_cells(case, name):
    return np.concatenate([side_owner_cells(case, s) for s in case.patches[name]])


def _boundary_field(case, values_of, vector, phi=False):
    """boundaryField entries: empty / cyclic as such, fixedValue potentials
    with their value, everything else `calculated` (or the case's own type for
    the potential) with the owner cells' values."""
    out = ["boundaryField\n{\n"]
    for name in case.patches:
        ptype = case.patch_types[name]
        out.append(f"    {name}\n    {{\n")
        if ptype in ("empty", "cyclic"):
            out.append(f"        type            {ptype};\n    }}\n")
            continue
        bc = case.phi_bc.get(name, foam.Dict())
        t = bc.word("type", "calculated") if phi else "calculated"
        if phi and t == "fixedValue":
            v = _uniform_scalar(bc.get("value")) or 0.0
            out.append(f"        type            fixedValue;\n        value           uniform {v!r};\n    }}\n")
            continue
        vals = values_of[_patch_owner_cells(case, name)]
        body = foam.format_vectors(vals) if vector else foam.format_scalars(vals)
        kind = "List<vector>" if vector else "List<scalar>"
        out.append(f"        type            {t};\n        value           nonuniform {kind} {body};\n    }}\n")
    out.append("}\n")
    return "".join(out)


def _write_vol(path, obj, dims, values_of, vector, case, phi=False):
    cls = "volVectorField" if vector else "volScalarField"
    body = foam.format_vectors(values_of) if vector else foam.format_scalars(values_of)
    kind = "List<vector>" if vector else "List<scalar>"
    with open(path, "w") as f:
        f.write(foam.header(cls, obj, location=os.path.basename(os.path.dirname(path))))
        f.write(f"dimensions      {dims};\n\n")
        f.write(f"internalField   nonuniform {kind} {body};\n\n")
        f.write(_boundary_field(case, values_of, vector, phi))


def write_fields(sim, case, t, cloud="pic", step_index=None):
    """Write time directory `t` of the case: phiE, E, rhoCharge (cells in the
    case's order) and lagrangian/<cloud>/{U, typeId, chargeModifier,
    nParticle} (PICParcelIO.C:107-166) plus cartesianPositions (a vector
    field of this writer: positions as points, not OpenFOAM's barycentric
    coordinates).  For a restart with this library (`restart`) it also
    writes the exact particle state -- picgpuTet (the context's tet index,
    cell 12 + local tet) and picgpuBarycentric (coordinates 1..3) -- and
    uniform/picgpuState (the step index and the floating patches' surface
    charge density).  Every number has 17 significant digits, so the state
    reads back bit for bit.  Returns the directory."""
    d = os.path.join(case.path, time_name(t))
    os.makedirs(d, exist_ok=True)
    order = case.cell_order
    phi = sim.field(abi.FIELD_PHI)[order]
    E = sim.field(abi.FIELD_E_CELL).reshape(-1, 3)[order]
    rho = sim.field(abi.FIELD_RHO)[order]
    _write_vol(os.path.join(d, "phiE"), "phiE", _PHI_DIM, phi, False, case, phi=True)
    _write_vol(os.path.join(d, "E"), "E", _E_DIM, E, True, case)
    _write_vol(os.path.join(d, "rhoCharge"), "rhoCharge", _RHO_DIM, rho, False, case)
    from .simulation import Mesh
    m = Mesh(case.mesh)
    U, tid, npart, pos, tets, barys, zq = [], [], [], [], [], [], []
    for s in range(len(case.species)):
        tet, bary, u = sim.get_particles(s)
        w, z = sim.get_parcel_attributes(s)
        if len(tet) == 0:
            continue
        U.append(u)
        tid.append(np.full(len(tet), s, dtype=np.int64))
        npart.append(w)
        zq.append(z.astype(np.int64))
        pos.append(m.position(tet, bary))
        tets.append(tet.astype(np.int64))
        barys.append(bary)
    if U:
        ld = os.path.join(d, "lagrangian", cloud)
        os.makedirs(ld, exist_ok=True)
        U, tid, npart, pos, tets, barys, zq = (np.concatenate(x) for x in (U, tid, npart, pos, tets, barys, zq))
        loc = os.path.join(time_name(t), "lagrangian", cloud)
        for name, cls, body in (("U", "vectorField", foam.format_vectors(U)),
                                ("typeId", "labelField", foam.format_labels(tid)),
                                ("chargeModifier", "labelField", foam.format_labels(zq)),
                                ("nParticle", "scalarField", foam.format_scalars(npart)),
                                ("cartesianPositions", "vectorField", foam.format_vectors(pos)),
                                ("picgpuTet", "labelField", foam.format_labels(tets)),
                                ("picgpuBarycentric", "vectorField", foam.format_vectors(barys))):
            with open(os.path.join(ld, name), "w") as f:
                f.write(foam.header(cls, name, location=loc))
                f.write(body)
    if step_index is None:
        step_index = int(round(t / case.delta_t)) if case.delta_t > 0 else 0
    sigma = sim.field(abi.FIELD_PATCH_SIGMA)
    ud = os.path.join(d, "uniform")
    os.makedirs(ud, exist_ok=True)
    with open(os.path.join(ud, "picgpuState"), "w") as f:
        f.write(foam.header("dictionary", "picgpuState", location=os.path.join(time_name(t), "uniform")))
        f.write(f"stepIndex       {int(step_index)};\n\n")
        f.write("patchSigma      " + foam.format_scalars(sigma).replace("\n", " ") + ";\n")
    return d


def read_list(path):
    """The list after the FoamFile header of a lagrangian or polyMesh file
    (labels, scalars or vectors) as a numpy array."""
    with open(path) as f:
        txt = f.read()
    body = txt[txt.index("}", txt.index("FoamFile")) + 1:]
    inner = body[body.index("(") + 1:body.rindex(")")]
    vectors = "(" in inner
    vals = np.array(inner.replace("(", " ").replace(")", " ").split(), dtype=np.float64)
    return vals.reshape(-1, 3) if vectors else vals


def latest_time(case):
    """The latest time directory of the case (controlDict startFrom latestTime)."""
    times = []
    for name in os.listdir(case.path):
        try:
            t = float(name)
        except ValueError:
            continue
        if os.path.isdir(os.path.join(case.path, name)) and t > 0:
            times.append(t)
    if not times:
        raise FileNotFoundError(f"{case.path}: no time directory to restart from")
    return max(times)


def restart(sim, case, t=None, cloud="pic"):
    """Continue a run from time directory `t` (default: the latest), the
    startFrom latestTime of picFoam (PICParcelIO.C:83-120 reads the parcels
    back): particles from picgpuTet / picgpuBarycentric / U / typeId (the
    state this library writes; without them the cartesianPositions are
    located again, which rounds the coordinates), their nParticle and
    chargeModifier where they differ from the species', the potential phiE,
    the step index and the floating patches' surface charge.  E is computed
    from the written potential (no Poisson solve; the next step deposits the
    charge again), so a FP64 run continues bit for bit.  Not restored: the remainders of injection, emission and
    collision models, MCC (sigma v)_max and circuit states.  Returns t."""
    if t is None:
        t = latest_time(case)
    d = os.path.join(case.path, time_name(t))
    ld = os.path.join(d, "lagrangian", cloud)
    if os.path.isdir(ld):
        tid = read_list(os.path.join(ld, "typeId")).astype(np.int64)
        U = read_list(os.path.join(ld, "U")).reshape(-1, 3)
        if os.path.exists(os.path.join(ld, "picgpuTet")):
            tet = read_list(os.path.join(ld, "picgpuTet")).astype(np.int32)
            bary = read_list(os.path.join(ld, "picgpuBarycentric")).reshape(-1, 3)
        else:
            from .simulation import Mesh
            tet, bary = Mesh(case.mesh).locate(read_list(os.path.join(ld, "cartesianPositions")).reshape(-1, 3))
        w = read_list(os.path.join(ld, "nParticle")) if os.path.exists(os.path.join(ld, "nParticle")) else None
        z = (read_list(os.path.join(ld, "chargeModifier")).astype(np.int32)
             if os.path.exists(os.path.join(ld, "chargeModifier")) else None)
        for s in range(len(case.species)):
            sel = tid == s
            sim.set_particles(s, tet[sel], bary[sel], U[sel])
            # per-parcel weights and charge states where they differ from
            # the species' (PICParcelIO.C:98-113)
            if w is not None and z is not None and np.any(sel) and (
                    np.any(w[sel] != case.cfg.species[s].weight) or np.any(z[sel] != 1)):
                sim.set_parcel_attributes(s, w[sel], z[sel])
    phi_case = read_field(os.path.join(d, "phiE"))
    phi = np.empty_like(phi_case)
    phi[case.cell_order] = phi_case
    state_path = os.path.join(d, "uniform", "picgpuState")
    step_index = int(round(t / case.delta_t)) if case.delta_t > 0 else 0
    if os.path.exists(state_path):
        st = foam.read(state_path)
        step_index = int(st["stepIndex"])
        sim.set_field(abi.FIELD_PATCH_SIGMA, foam.numeric_list(st["patchSigma"]))
    sim.set_step_index(step_index)
    sim.set_field(abi.FIELD_PHI, phi)
    # E from the written potential: the charge density of that step was
    # deposited before the step's last changes to the parcels (PairMerging
    # runs after the field solve), so it is not deposited again here
    sim.compute_field()
    return t


def read_field(path):
    """The internal field of a volScalarField / volVectorField file (values
    in the file's cell order)."""
    d = foam.read(path)
    v = d["internalField"]
    if isinstance(v, tuple) and v[0] == "uniform":
        return np.asarray(v[1], dtype=np.float64)
    return foam.numeric_list(v)


def _quads(a, i, j, k, positive, npt):
    """Point quads of faces normal to axis a at grid planes (i, j, k),
    ordered for a normal along +a (positive) or -a."""
    nx1, ny1 = npt[0], npt[1]

    def pid(ii, jj, kk):
        return ii + nx1 * (jj + ny1 * kk)

    if a == 0:
        q = [pid(i, j, k), pid(i, j + 1, k), pid(i, j + 1, k + 1), pid(i, j, k + 1)]
    elif a == 1:
        q = [pid(i, j, k), pid(i, j, k + 1), pid(i + 1, j, k + 1), pid(i + 1, j, k)]
    else:
        q = [pid(i, j, k), pid(i + 1, j, k), pid(i + 1, j + 1, k), pid(i, j + 1, k)]
    q = np.stack(q, axis=1)
    return np.where(positive[:, None], q, q[:, ::-1])


def write_poly_mesh(case, out_dir=None):
    """constant/polyMesh of the block (points, faces, owner, neighbour,
    boundary) with the case's cell numbering: internal faces in
    upper-triangular order (by owner, then neighbour) pointing from owner to
    neighbour, boundary faces patch by patch (each side's faces by rising
    owner), outward; cyclic halves list their faces in matching order.
    Returns the directory."""
    d = out_dir or os.path.join(case.path, "constant", "polyMesh")
    os.makedirs(d, exist_ok=True)
    n = [int(x) for x in case.mesh.n]
    npt = [x + 1 for x in n]
    h = [case.mesh.length[a] / n[a] for a in range(3)]
    kk, jj, ii = np.meshgrid(np.arange(npt[2]), np.arange(npt[1]), np.arange(npt[0]), indexing="ij")
    pts = np.stack([case.mesh.origin[0] + ii.ravel() * h[0], case.mesh.origin[1] + jj.ravel() * h[1],
                    case.mesh.origin[2] + kk.ravel() * h[2]], axis=1)
    of_idx = _of_of_ctx(case)
    ci, cj, ck = _ctx_ijk(case)
    ncell = len(of_idx)
    # internal faces
    owners, neighbours, quads = [], [], []
    for a in range(3):
        lower = np.flatnonzero([ci, cj, ck][a] < n[a] - 1)
        step = [1, n[0], n[0] * n[1]][a]
        upper = lower + step
        ijk_face = [ci[lower], cj[lower], ck[lower]]
        ijk_face[a] = ijk_face[a] + 1
        o_l, o_u = of_idx[lower], of_idx[upper]
        positive = o_l < o_u                         # owner is the lower-coordinate cell
        owners.append(np.minimum(o_l, o_u))
        neighbours.append(np.maximum(o_l, o_u))
        quads.append(_quads(a, *ijk_face, positive, npt))
    owner = np.concatenate(owners) if owners else np.zeros(0, np.int64)
    neighbour = np.concatenate(neighbours) if neighbours else np.zeros(0, np.int64)
    faces = np.concatenate(quads) if quads else np.zeros((0, 4), np.int64)
    order = np.lexsort((neighbour, owner))
    owner, neighbour, faces = owner[order], neighbour[order], faces[order]
    n_internal = len(owner)
    # boundary faces
    bnames, bstart, bcount = [], [], []
    b_owner, b_faces = [], []
    start = n_internal
    for name in case.patches:
        cnt = 0
        for side in case.patches[name]:
            a, hi = side // 2, side % 2
            cells_of = side_owner_cells(case, side)           # OpenFOAM indices, sorted
            ctx = case.cell_order[cells_of]
            ijk_face = [ci[ctx], cj[ctx], ck[ctx]]
            if hi:
                ijk_face[a] = ijk_face[a] + 1
            b_faces.append(_quads(a, *ijk_face, np.full(len(ctx), bool(hi)), npt))
            b_owner.append(cells_of)
            cnt += len(ctx)
        bnames.append(name)
        bstart.append(start)
        bcount.append(cnt)
        start += cnt
    all_faces = np.concatenate([faces] + b_faces)
    all_owner = np.concatenate([owner] + b_owner)
    note = f"nPoints:{len(pts)}  nCells:{ncell}  nFaces:{len(all_faces)}  nInternalFaces:{n_internal}"
    with open(os.path.join(d, "points"), "w") as f:
        f.write(foam.header("vectorField", "points", location="constant/polyMesh"))
        f.write(foam.format_vectors(pts))
    with open(os.path.join(d, "faces"), "w") as f:
        f.write(foam.header("faceList", "faces", location="constant/polyMesh"))
        f.write(f"{len(all_faces)}\n(\n" + "\n".join("4(%d %d %d %d)" % tuple(q) for q in all_faces) + "\n)\n")
    for name, arr in (("owner", all_owner), ("neighbour", neighbour)):
        with open(os.path.join(d, name), "w") as f:
            f.write(foam.header("labelList", name, location="constant/polyMesh", note=note))
            f.write(foam.format_labels(arr))
    with open(os.path.join(d, "boundary"), "w") as f:
        f.write(foam.header("polyBoundaryMesh", "boundary", location="constant/polyMesh"))
        f.write(f"{len(bnames)}\n(\n")
        for name, s0, cnt in zip(bnames, bstart, bcount):
            t = case.patch_types[name]
            f.write(f"    {name}\n    {{\n        type            {t};\n")
            if t in ("wall", "empty", "cyclic"):
                f.write(f"        inGroups        List<word> 1({t});\n")
            f.write(f"        nFaces          {cnt};\n        startFace       {s0};\n")
            if t == "cyclic":
                side = case.patches[name][0]
                f.write(f"        neighbourPatch  {case.side_names[side ^ 1]};\n")
            f.write("    }\n")
        f.write(")\n")
    return d
