"""ctypes backend for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Used by tests/ and by bench.py's CPU-baseline leg as the checker and the
timed CPU restatement; the product package never imports it.
"""
import ctypes as C
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liboracle.so")

if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from picfoam_gb300 import abi  # noqa: E402
from picfoam_gb300.native import declare  # noqa: E402

PRECOND_JACOBI = 0
PRECOND_DIC = 1


def build():
    """Compile liboracle.so with its Makefile (no FMA contraction)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


_lib = None


def load():
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        lib.oracle_create.restype = C.c_int
        lib.oracle_create.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.Config), C.c_int,
                                      C.POINTER(C.c_void_p)]
        declare(lib, "oracle_")
        lib.oracle_diagnostics.restype = C.c_int
        lib.oracle_diagnostics.argtypes = [P, C.POINTER(abi.Diagnostics)]
        lib.oracle_set_precond.restype = C.c_int
        lib.oracle_set_precond.argtypes = [P, C.c_int]
        lib.oracle_mesh_query.restype = C.c_int
        lib.oracle_mesh_query.argtypes = [P, C.POINTER(abi.MeshInfo)]
        lib.oracle_mesh_selfcheck.restype = C.c_int
        lib.oracle_mesh_selfcheck.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(C.c_double), C.c_int]
        lib.oracle_move_seconds.restype = C.c_double
        lib.oracle_move_seconds.argtypes = [P]
        lib.oracle_philox4x32.restype = None
        lib.oracle_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.oracle_det_log.restype = C.c_double
        lib.oracle_det_log.argtypes = [C.c_double]
        lib.oracle_det_sin.restype = C.c_double
        lib.oracle_det_sin.argtypes = [C.c_double]
        lib.oracle_debye_length.restype = C.c_double
        lib.oracle_debye_length.argtypes = [P, C.c_int]
        F32P, F64P = C.POINTER(C.c_float), C.POINTER(C.c_double)
        i = C.c_int
        lib.oracle_unet_param_count.restype = C.c_size_t
        lib.oracle_unet_param_count.argtypes = []
        lib.oracle_unet_forward.restype = i
        lib.oracle_unet_forward.argtypes = [i, i, i, F32P, F32P, i, F64P]
        lib.oracle_unet_gradients.restype = i
        lib.oracle_unet_gradients.argtypes = [i, i, i, F32P, F32P, F32P, F32P, i, F64P, F64P]
        _lib = lib
    return _lib


class OracleBackend:
    prefix = "oracle_"
    name = "oracle"

    def __init__(self, nthreads=1, precond=PRECOND_JACOBI):
        self.lib = load()
        self.nthreads = nthreads
        self.precond = precond

    def create(self, mesh, cfg):
        h = C.c_void_p()
        st = self.lib.oracle_create(C.byref(mesh), C.byref(cfg), self.nthreads, C.byref(h))
        if st == 0:
            self.lib.oracle_set_precond(h, self.precond)
        return st, h

    def sizes(self, h):
        info = abi.MeshInfo()
        self.lib.oracle_mesh_query(h, C.byref(info))
        return info.n_cells, info.n_points

    def move_seconds(self, h):
        return self.lib.oracle_move_seconds(h)
