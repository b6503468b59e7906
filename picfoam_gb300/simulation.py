"""Host-side mirror of the picFoam cloud interface over the picgpu C ABI.

Simulation plays the role of PICCloud for the caller: it owns one device
case (mesh, sub-models, particles, fields) and exposes the calls the picFoam
time loop makes (evolve -> step, info -> diagnostics) plus field and
particle access.  It talks to a backend: the CUDA library by default; the
test suite plugs the CPU oracle in through the same interface.
"""
import ctypes as C
import weakref

import numpy as np

from . import abi, native


class PicError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{abi.STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class GpuBackend:
    """libpicgpu.so (CUDA, sm_103a)."""
    prefix = "picgpu_"
    name = "gpu"

    def __init__(self):
        self.lib = native.load()

    def create(self, mesh, cfg):
        h = C.c_void_p()
        st = self.lib.picgpu_create(C.byref(mesh), C.byref(cfg), C.byref(h))
        return st, h


class EnsembleBackend(GpuBackend):
    """libpicgpu.so with n_cases disjoint copies of the mesh in one context
    (picgpu_ensemble_create)."""
    name = "gpu-ensemble"

    def __init__(self, n_cases):
        super().__init__()
        self.n_cases = n_cases

    def create(self, mesh, cfg):
        h = C.c_void_p()
        st = self.lib.picgpu_ensemble_create(C.byref(mesh), self.n_cases, C.byref(cfg), C.byref(h))
        return st, h


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _i32(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int32))


def pinned_empty(shape, dtype):
    """An uninitialised numpy array in page-locked host memory
    (picgpu_host_alloc), freed with the array: transfers from and to it go
    straight to the DMA engine."""
    lib = native.load()
    dtype = np.dtype(dtype)
    nbytes = max(int(np.prod(shape)) * dtype.itemsize, 1)
    ptr = C.c_void_p()
    if lib.picgpu_host_alloc(nbytes, C.byref(ptr)) != abi.OK:
        raise MemoryError(f"picgpu_host_alloc({nbytes}) failed")
    buf = (C.c_char * nbytes).from_address(ptr.value)
    weakref.finalize(buf, lib.picgpu_host_free, ptr.value)
    return np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)


class Simulation:
    def __init__(self, mesh, cfg, backend=None, keepalive=()):
        self.backend = backend if backend is not None else GpuBackend()
        self.lib = self.backend.lib
        self.mesh_desc = mesh
        self.cfg = cfg
        self._keep = list(keepalive)
        self._h = None
        st, h = self.backend.create(mesh, cfg)
        self._h = h
        if st != abi.OK:
            msg = self._err()
            self.close()
            raise PicError(st, msg)

    # ---------------------------------------------------------------- util
    def _fn(self, name):
        return getattr(self.lib, self.backend.prefix + name)

    def _err(self):
        if not self._h:
            return ""
        e = self._fn("last_error")(self._h)
        return e.decode() if e else ""

    def _check(self, st):
        if st != abi.OK:
            raise PicError(st, self._err())

    def close(self):
        if self._h:
            self._fn("destroy")(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ----------------------------------------------------------- particles
    def set_particles(self, species, tet, bary, U):
        tet, tp = _i32(tet)
        bary, bp = _f64(np.reshape(bary, (-1, 3)))
        U, up = _f64(np.reshape(U, (-1, 3)))
        n = tet.shape[0]
        assert bary.shape[0] == n and U.shape[0] == n
        self._check(self._fn("set_particles")(self._h, species, n, tp, bp, up))

    def count(self, species):
        n = C.c_size_t()
        self._check(self._fn("count_particles")(self._h, species, C.byref(n)))
        return n.value

    def get_particles(self, species, out=None):
        """(tet, bary, U) of one species in storage order; `out` = three
        arrays to fill (int32 n, float64 n x 3, float64 n x 3, e.g. from
        pinned_empty), of at least the species' count."""
        cap = self.count(species)
        if out is None:
            tet = np.zeros(cap, np.int32)
            bary = np.zeros((cap, 3))
            U = np.zeros((cap, 3))
        else:
            tet, bary, U = out
            assert tet.dtype == np.int32 and bary.dtype == U.dtype == np.float64
            assert tet.flags.c_contiguous and bary.flags.c_contiguous and U.flags.c_contiguous
            cap = min(len(tet), len(bary), len(U))
        n = C.c_size_t()
        self._check(self._fn("get_particles")(
            self._h, species, cap, tet.ctypes.data_as(C.POINTER(C.c_int32)),
            bary.ctypes.data_as(C.POINTER(C.c_double)), U.ctypes.data_as(C.POINTER(C.c_double)),
            C.byref(n)))
        k = n.value
        return tet[:k], bary[:k], U[:k]

    def set_parcel_attributes(self, species, nParticle, chargeModifier):
        """Per-parcel nParticle and chargeModifier of one species, in the
        order of get_particles (picgpu_set_parcel_attributes)."""
        w, wp = _f64(nParticle)
        z = np.ascontiguousarray(chargeModifier, dtype=np.int32)
        assert w.shape[0] == z.shape[0]
        self._check(self._fn("set_parcel_attributes")(self._h, species, w.shape[0], wp,
                                                      z.ctypes.data_as(C.POINTER(C.c_int32))))

    def get_parcel_attributes(self, species):
        """(nParticle, chargeModifier) of one species, in the order of get_particles."""
        n = C.c_size_t()
        self._check(self._fn("get_parcel_attributes")(self._h, species, 0, None, None, C.byref(n)))
        w = np.zeros(n.value)
        z = np.zeros(n.value, np.int32)
        self._check(self._fn("get_parcel_attributes")(
            self._h, species, n.value, w.ctypes.data_as(C.POINTER(C.c_double)),
            z.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(n)))
        return w[:n.value], z[:n.value]

    def compute_field(self):
        """E from the current potential, no Poisson solve (picgpu_compute_field)."""
        self._check(self._fn("compute_field")(self._h))

    # ---------------------------------------------------------------- step
    def initialise_fields(self):
        self._check(self._fn("initialise_fields")(self._h))

    def set_injection(self, injectors):
        """SimpleInjection boundary models: a list of abi.Injection (empty
        removes them)."""
        arr = (abi.Injection * max(len(injectors), 1))(*injectors)
        self._check(self._fn("set_injection")(self._h, len(injectors), arr))

    def set_freestream(self, models):
        """FreeStream boundary models: a list of abi.FreeStream (empty removes
        them; the face accumulators restart at zero)."""
        arr = (abi.FreeStream * max(len(models), 1))(*models)
        self._check(self._fn("set_freestream")(self._h, len(models), arr))

    def set_emission(self, models):
        """EmissionModels (Thermionic, FowlerNordheim): a list of abi.Emission
        (empty removes them)."""
        arr = (abi.Emission * max(len(models), 1))(*models)
        self._check(self._fn("set_emission")(self._h, len(models), arr))

    def initialise(self, init):
        """picInitialise: place the particles of an abi.Init on the device (or
        in the oracle), compute the fields, optionally solve them and apply
        the leapfrog back-step; returns the abi.InitStats."""
        st = abi.InitStats()
        self._check(self._fn("initialise")(self._h, C.byref(init), C.byref(st)))
        return st

    def step(self, n=1):
        s = abi.StepStats()
        self._check(self._fn("step")(self._h, n, C.byref(s)))
        return s

    def step_graph(self, n, steps_per_graph):
        """n steps as CUDA-graph replays of steps_per_graph steps (FP32 form,
        MaxwellSolver none); the first call tunes the launch shapes."""
        s = abi.StepStats()
        self._check(self.lib.picgpu_step_graph(self._h, n, steps_per_graph, C.byref(s)))
        return s

    def graph_tuning(self, n_times=16):
        bps, blk = C.c_int(), C.c_int()
        t = np.zeros(n_times)
        self._check(self.lib.picgpu_graph_tuning(self._h, C.byref(bps), C.byref(blk),
                                                 t.ctypes.data_as(C.POINTER(C.c_double)), n_times))
        return bps.value, blk.value, t

    def set_case_efield(self, E):
        """Applied field per case of an ensemble, E[n_cases][3]."""
        e, ep = _f64(np.reshape(E, (-1, 3)))
        self._check(self.lib.picgpu_ensemble_set_efield(self._h, ep))

    def case_stats(self, species, n_cases):
        """Per case: count, sum U (3), sum |U|^2, and MCC ionisations."""
        out = np.zeros((n_cases, 5))
        iz = np.zeros(n_cases, np.int64)
        self._check(self.lib.picgpu_ensemble_case_stats(self._h, species, out.ctypes.data_as(C.POINTER(C.c_double)),
                                                        iz.ctypes.data_as(C.POINTER(C.c_int64))))
        return out, iz

    def move(self):
        s = abi.StepStats()
        self._check(self._fn("move")(self._h, C.byref(s)))
        return s

    def solve_poisson(self, rho, phi0=None):
        rho, rp = _f64(rho)
        phi = np.zeros_like(rho) if phi0 is None else np.array(phi0, dtype=np.float64, copy=True)
        s = abi.StepStats()
        self._check(self._fn("solve_poisson")(self._h, rp, phi.ctypes.data_as(C.POINTER(C.c_double)),
                                              C.byref(s)))
        return phi, s

    # -------------------------------------------------------------- fields
    def _field_len(self, which, n_cells, n_points):
        return {abi.FIELD_PHI: n_cells, abi.FIELD_E_CELL: 3 * n_cells, abi.FIELD_RHO: n_cells,
                abi.FIELD_E_POINT: 3 * n_points, abi.FIELD_SIGMA_V_MAX: n_cells,
                abi.FIELD_B_CELL: 3 * n_cells, abi.FIELD_PATCH_SIGMA: 6 + self.mesh_desc.n_boxes}[which]

    def sizes(self):
        """(n_cells, n_points) of the mesh."""
        if hasattr(self.backend, "sizes"):
            return self.backend.sizes(self._h)
        info = abi.MeshInfo()
        self._check(self.lib.picgpu_mesh_query(self._h, C.byref(info)))
        return info.n_cells, info.n_points

    def field(self, which):
        nc, npnt = self.sizes()
        n = self._field_len(which, nc, npnt)
        out = np.zeros(n)
        self._check(self._fn("get_field")(self._h, which, out.ctypes.data_as(C.POINTER(C.c_double)), n))
        if which in (abi.FIELD_E_CELL, abi.FIELD_E_POINT, abi.FIELD_B_CELL):
            out = out.reshape(-1, 3)
        return out

    def set_step_index(self, steps_done):
        """Continue a run after `steps_done` steps (restart from a time directory)."""
        self._check(self._fn("set_step_index")(self._h, int(steps_done)))

    def set_field(self, which, values):
        v, vp = _f64(np.ravel(values))
        self._check(self._fn("set_field")(self._h, which, vp, v.size))

    def diagnostics(self):
        d = abi.Diagnostics()
        fn = self._fn("diagnostics") if hasattr(self.lib, self.backend.prefix + "diagnostics") \
            else self._fn("diagnostics_compute")
        self._check(fn(self._h, C.byref(d)))
        return d

    # ------------------------------------------------------------ profiling
    def set_profiling(self, on=True):
        self._check(self.lib.picgpu_set_profiling(self._h, 1 if on else 0))

    def phase_times(self, reset=False):
        ms = (C.c_double * abi.PHASE_COUNT)()
        cnt = (C.c_int64 * abi.PHASE_COUNT)()
        self._check(self.lib.picgpu_phase_times(self._h, ms, cnt, abi.PHASE_COUNT, 1 if reset else 0))
        return {abi.PHASE_NAMES[i]: (ms[i], cnt[i]) for i in range(abi.PHASE_COUNT)}

    def kernel_launches(self):
        return int(self.lib.picgpu_kernel_launches(self._h))

    def synchronize(self):
        self._check(self.lib.picgpu_synchronize(self._h))

    def timer_start(self):
        self._check(self.lib.picgpu_timer_start(self._h))

    def timer_stop(self):
        ms = C.c_double()
        self._check(self.lib.picgpu_timer_stop(self._h, C.byref(ms)))
        return ms.value


class Mesh:
    """Host-only mesh handle (tet decomposition, locate, positions); no GPU needed."""

    def __init__(self, desc):
        self.lib = native.load()
        self._h = C.c_void_p()
        st = self.lib.picgpu_mesh_create(C.byref(desc), C.byref(self._h))
        if st != abi.OK:
            raise PicError(st, "invalid mesh description")
        info = abi.MeshInfo()
        self.lib.picgpu_mesh_info_get(self._h, C.byref(info))
        self.n_cells = info.n_cells
        self.n_points = info.n_points

    def close(self):
        if self._h:
            self.lib.picgpu_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def locate(self, xyz):
        xyz, xp = _f64(np.reshape(xyz, (-1, 3)))
        n = xyz.shape[0]
        tet = np.zeros(n, np.int32)
        bary = np.zeros((n, 3))
        self.lib.picgpu_mesh_locate(self._h, n, xp, tet.ctypes.data_as(C.POINTER(C.c_int32)),
                                    bary.ctypes.data_as(C.POINTER(C.c_double)))
        return tet, bary

    def position(self, tet, bary):
        tet, tp = _i32(tet)
        bary, bp = _f64(np.reshape(bary, (-1, 3)))
        out = np.zeros((tet.shape[0], 3))
        st = self.lib.picgpu_mesh_position(self._h, tet.shape[0], tp, bp,
                                           out.ctypes.data_as(C.POINTER(C.c_double)))
        if st != abi.OK:
            raise PicError(st, "tet index out of range")
        return out

    def cells(self):
        cc = np.zeros((self.n_cells, 3))
        vol = np.zeros(self.n_cells)
        self.lib.picgpu_mesh_cells(self._h, cc.ctypes.data_as(C.POINTER(C.c_double)),
                                   vol.ctypes.data_as(C.POINTER(C.c_double)))
        return cc, vol
