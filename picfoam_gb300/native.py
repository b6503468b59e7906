"""Loader of the CUDA library libpicgpu.so and its ctypes signatures.

The product has exactly one implementation of the hot path: the CUDA
kernels in libpicgpu.so.  If the library has not been built, load() raises;
there is no CPU fallback.
"""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
# PICGPU_LIB selects another build of the library (e.g. a variant build).
LIB_PATH = os.environ.get("PICGPU_LIB") or os.path.join(_HERE, "_build", "libpicgpu.so")

_lib = None

P = C.c_void_p
PP = C.POINTER(C.c_void_p)
I32P = C.POINTER(C.c_int32)
F64P = C.POINTER(C.c_double)
I64P = C.POINTER(C.c_int64)
SZP = C.POINTER(C.c_size_t)


def declare(lib, prefix, ctx_api=True):
    """Attach argtypes/restype for the ctx-level API under a symbol prefix."""
    def f(name, res, args):
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
        return fn

    i = C.c_int
    f("destroy", None, [P])
    f("last_error", C.c_char_p, [P])
    f("set_particles", i, [P, i, C.c_size_t, I32P, F64P, F64P])
    f("count_particles", i, [P, i, SZP])
    f("get_particles", i, [P, i, C.c_size_t, I32P, F64P, F64P, SZP])
    f("set_parcel_attributes", i, [P, i, C.c_size_t, F64P, I32P])
    f("get_parcel_attributes", i, [P, i, C.c_size_t, F64P, I32P, SZP])
    f("initialise_fields", i, [P])
    f("initialise", i, [P, C.POINTER(abi.Init), C.POINTER(abi.InitStats)])
    f("set_injection", i, [P, i, C.POINTER(abi.Injection)])
    f("set_freestream", i, [P, i, C.POINTER(abi.FreeStream)])
    f("set_emission", i, [P, i, C.POINTER(abi.Emission)])
    f("step", i, [P, i, C.POINTER(abi.StepStats)])
    f("move", i, [P, C.POINTER(abi.StepStats)])
    f("solve_poisson", i, [P, F64P, F64P, C.POINTER(abi.StepStats)])
    f("get_field", i, [P, i, F64P, C.c_size_t])
    f("set_field", i, [P, i, F64P, C.c_size_t])
    f("set_step_index", i, [P, C.c_int64])
    f("compute_field", i, [P])


def load():
    """Load libpicgpu.so (built by picfoam_gb300.build.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build the CUDA library first "
            "(python -c 'import picfoam_gb300.build as b; b.build()')")
    lib = C.CDLL(LIB_PATH)
    i = C.c_int
    lib.picgpu_create.restype = i
    lib.picgpu_create.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.Config), PP]
    declare(lib, "picgpu_")
    lib.picgpu_diagnostics_compute.restype = i
    lib.picgpu_diagnostics_compute.argtypes = [P, C.POINTER(abi.Diagnostics)]
    lib.picgpu_mesh_query.restype = i
    lib.picgpu_mesh_query.argtypes = [P, C.POINTER(abi.MeshInfo)]
    lib.picgpu_mesh_create.restype = i
    lib.picgpu_mesh_create.argtypes = [C.POINTER(abi.MeshDesc), PP]
    lib.picgpu_mesh_destroy.restype = None
    lib.picgpu_mesh_destroy.argtypes = [P]
    lib.picgpu_mesh_info_get.restype = i
    lib.picgpu_mesh_info_get.argtypes = [P, C.POINTER(abi.MeshInfo)]
    lib.picgpu_mesh_locate.restype = i
    lib.picgpu_mesh_locate.argtypes = [P, C.c_size_t, F64P, I32P, F64P]
    lib.picgpu_mesh_position.restype = i
    lib.picgpu_mesh_position.argtypes = [P, C.c_size_t, I32P, F64P, F64P]
    lib.picgpu_mesh_cells.restype = i
    lib.picgpu_mesh_cells.argtypes = [P, F64P, F64P]
    lib.picgpu_set_profiling.restype = i
    lib.picgpu_set_profiling.argtypes = [P, i]
    lib.picgpu_phase_times.restype = i
    lib.picgpu_phase_times.argtypes = [P, F64P, I64P, i, i]
    lib.picgpu_kernel_launches.restype = C.c_int64
    lib.picgpu_kernel_launches.argtypes = [P]
    lib.picgpu_synchronize.restype = i
    lib.picgpu_synchronize.argtypes = [P]
    lib.picgpu_timer_start.restype = i
    lib.picgpu_timer_start.argtypes = [P]
    lib.picgpu_timer_stop.restype = i
    lib.picgpu_timer_stop.argtypes = [P, F64P]
    lib.picgpu_solve_ldu_noalloc.restype = i
    lib.picgpu_solve_ldu_noalloc.argtypes = [i, P, P, P, P, P, C.c_double, i, C.POINTER(C.c_int),
                                             F64P, P]
    U16P = C.POINTER(C.c_uint16)
    F32P = C.POINTER(C.c_float)
    lib.picgpu_test_conv3d.restype = i
    lib.picgpu_test_conv3d.argtypes = [i, i, i, i, i, i, i, i, U16P, U16P, U16P, F32P]
    lib.picgpu_ensemble_create.restype = i
    lib.picgpu_ensemble_create.argtypes = [C.POINTER(abi.MeshDesc), i, C.POINTER(abi.Config), PP]
    lib.picgpu_ensemble_set_efield.restype = i
    lib.picgpu_ensemble_set_efield.argtypes = [P, F64P]
    lib.picgpu_ensemble_case_stats.restype = i
    lib.picgpu_ensemble_case_stats.argtypes = [P, i, F64P, I64P]
    lib.picgpu_step_graph.restype = i
    lib.picgpu_step_graph.argtypes = [P, i, i, C.POINTER(abi.StepStats)]
    lib.picgpu_graph_tuning.restype = i
    lib.picgpu_graph_tuning.argtypes = [P, C.POINTER(C.c_int), C.POINTER(C.c_int), F64P, i]
    lib.picgpu_unet_param_count.restype = C.c_size_t
    lib.picgpu_unet_param_count.argtypes = []
    lib.picgpu_unet_create.restype = i
    lib.picgpu_unet_create.argtypes = [i, i, i, C.c_uint64, PP]
    lib.picgpu_unet_destroy.restype = None
    lib.picgpu_unet_destroy.argtypes = [P]
    lib.picgpu_unet_set_weights.restype = i
    lib.picgpu_unet_set_weights.argtypes = [P, F32P]
    lib.picgpu_unet_get_weights.restype = i
    lib.picgpu_unet_get_weights.argtypes = [P, F32P]
    lib.picgpu_unet_forward.restype = i
    lib.picgpu_unet_forward.argtypes = [P, F32P, F32P]
    lib.picgpu_unet_gradients.restype = i
    lib.picgpu_unet_gradients.argtypes = [P, F32P, F32P, F32P, F32P, F64P]
    lib.picgpu_unet_train.restype = i
    lib.picgpu_unet_train.argtypes = [P, F32P, F32P, F32P, i, C.c_double, F64P]
    lib.picgpu_host_alloc.restype = i
    lib.picgpu_host_alloc.argtypes = [C.c_size_t, PP]
    lib.picgpu_host_free.restype = i
    lib.picgpu_host_free.argtypes = [P]
    _lib = lib
    return lib
