"""picFoam tutorial cases as fixtures (TEST INFRASTRUCTURE).

`dump` turns a case loaded by picfoam_gb300.ofcase.load_case from one of
picFoam's tutorial directories into a JSON document of the C ABI structures
it maps to (mesh description, configuration with its cross-section tables,
initial conditions, boundary models, ParticleList parcels); `load` rebuilds
an OFCase from it.  The GPU tests run the fixtures where picFoam's tree is
absent; make_tutorial_cases.py writes them from the tutorials.
"""
import ctypes as C
import json

import numpy as np

from picfoam_gb300 import abi, ofcase

# pointer fields of picgpu_config and the count field that sizes each
POINTERS = {("mcc", "xs_energy"): "n_xs", ("mcc", "xs_elastic"): "n_xs", ("mcc", "xs_excitation"): "n_xs",
            ("mcc", "xs_ionization"): "n_xs", ("ion_mcc", "xs_energy"): "n_xs",
            ("ion_mcc", "xs_elastic"): "n_xs", ("ion_mcc", "xs_charge_exchange"): "n_xs"}


def to_json(obj):
    if isinstance(obj, C.Structure):
        out = {}
        for name, t in obj._fields_:
            v = getattr(obj, name)
            if isinstance(t, type) and issubclass(t, C._Pointer):
                continue
            out[name] = to_json(v)
        return out
    if isinstance(obj, C.Array):
        return [to_json(x) for x in obj]
    if isinstance(obj, float):
        return repr(obj)              # 17 digits survive the round trip
    return obj


def from_json(target, data):
    for name, t in target._fields_:
        if name not in data:
            continue
        v = data[name]
        cur = getattr(target, name)
        if isinstance(cur, C.Structure):
            from_json(cur, v)
        elif isinstance(cur, C.Array):
            for i, x in enumerate(v):
                if isinstance(cur[i], (C.Structure, C.Array)):
                    from_json_any(cur[i], x)
                else:
                    cur[i] = float(x) if isinstance(x, str) else x
        else:
            setattr(target, name, float(v) if isinstance(v, str) else v)
    return target


def from_json_any(target, v):
    if isinstance(target, C.Structure):
        return from_json(target, v)
    for i, x in enumerate(v):
        if isinstance(target[i], (C.Structure, C.Array)):
            from_json_any(target[i], x)
        else:
            target[i] = float(x) if isinstance(x, str) else x
    return target


def dump(case):
    pointers = {}
    for (sub, name), count in POINTERS.items():
        s = getattr(case.cfg, sub)
        p = getattr(s, name)
        n = getattr(s, count)
        if p and n > 0:
            pointers[f"{sub}.{name}"] = [repr(float(p[i])) for i in range(n)]
    return {
        "species": list(case.species),
        "side_names": list(case.side_names),
        "cell_order": [int(x) for x in case.cell_order],
        "mesh": to_json(case.mesh),
        "cfg": to_json(case.cfg),
        "pointers": pointers,
        "init": to_json(case.init) if case.init is not None else None,
        "injections": [to_json(x) for x in case.injections],
        "freestreams": [to_json(x) for x in case.freestreams],
        "emissions": [to_json(x) for x in case.emissions],
        "particle_list": [[int(s), [repr(float(v)) for v in p], [repr(float(v)) for v in u]]
                          for s, p, u in case.particle_list],
        "delta_t": repr(case.delta_t), "end_time": repr(case.end_time), "write_interval": repr(case.write_interval),
        "unsupported": list(case.unsupported),
    }


def load(path, precision=None):
    with open(path) as f:
        d = json.load(f)
    mesh = from_json(abi.MeshDesc(), d["mesh"])
    cfg = from_json(abi.Config(), d["cfg"])
    if precision is not None:
        cfg.precision = precision
    keep = []
    for key, vals in d["pointers"].items():
        sub, name = key.split(".")
        arr = np.ascontiguousarray([float(x) for x in vals], dtype=np.float64)
        keep.append(arr)
        setattr(getattr(cfg, sub), name, arr.ctypes.data_as(C.POINTER(C.c_double)))
    case = ofcase.OFCase(path=None, mesh=mesh, cfg=cfg, species=d["species"], side_names=d["side_names"],
                         patches={}, patch_types={}, phi_bc={}, cell_order=np.array(d["cell_order"]))
    case.init = from_json(abi.Init(), d["init"]) if d["init"] is not None else None
    case.injections = [from_json(abi.Injection(), x) for x in d["injections"]]
    case.freestreams = [from_json(abi.FreeStream(), x) for x in d["freestreams"]]
    case.emissions = [from_json(abi.Emission(), x) for x in d["emissions"]]
    case.particle_list = [(s, [float(v) for v in p], [float(v) for v in u]) for s, p, u in d["particle_list"]]
    case.delta_t, case.end_time, case.write_interval = (float(d[k]) for k in ("delta_t", "end_time", "write_interval"))
    case.unsupported = d["unsupported"]
    case.keepalive = keep
    return case
