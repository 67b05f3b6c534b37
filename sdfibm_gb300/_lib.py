"""ctypes binding of libsdfibm_cuda.so (the C ABI of include/sdfibm_cuda.h and include/sdfibm_host.h).

The library is built in-tree by ``sdfibm_gb300.build``; importing the binding without it raises: there is no CPU
fallback for any entry point.
"""
import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsdfibm_cuda.so")
_lib = None

CUDA_SYMBOLS = [
    "sdfibm_options_default", "sdfibm_cuda_create", "sdfibm_cuda_interact", "sdfibm_cuda_interact_host",
    "sdfibm_cuda_interact_host64", "sdfibm_cuda_create_polymesh",
    "sdfibm_cuda_evolve", "sdfibm_cuda_fix_internal", "sdfibm_cuda_apply_forcing", "sdfibm_cuda_get_solids",
    "sdfibm_cuda_set_solids",
    "sdfibm_cuda_touched", "sdfibm_cuda_stats", "sdfibm_cuda_kernel_times", "sdfibm_cuda_last_error",
    "sdfibm_cuda_version",
    "sdfibm_cuda_destroy", "sdfibm_cuda_touched_noalloc", "sdfibm_cuda_set_fraction_model", "sdfibm_cuda_autotune",
    "sdfibm_cuda_tuning",
]
MLP_SYMBOLS = [
    "sdfibm_mlp_dataset", "sdfibm_mlp_forward", "sdfibm_mlp_loss_grad", "sdfibm_mlp_adam", "sdfibm_mlp_train",
]
HOST_SYMBOLS = [
    "sdfibm_host_make_shape", "sdfibm_host_make_motion", "sdfibm_host_make_forcer", "sdfibm_host_quat_from_euler_deg",
    "sdfibm_host_make_solid", "sdfibm_host_parse_soliddict", "sdfibm_host_euler_from_quat",
    "sdfibm_host_format_state", "sdfibm_host_write_restart", "sdfibm_host_soliddict_lookup",
    "sdfibm_host_format_mean_field", "sdfibm_host_parse_vofdict", "sdfibm_host_parse_blockmesh",
    "sdfibm_host_write_scalar_field", "sdfibm_host_soliddict_shape", "sdfibm_host_read_foam_list",
    "sdfibm_host_read_foam_faces", "sdfibm_host_uniform_mesh", "sdfibm_host_write_vector_field",
]


class LibraryMissing(ImportError):
    pass


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryMissing("%s is not built; run `python -m sdfibm_gb300.build` (needs nvcc)" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    P = C.POINTER
    L.sdfibm_options_default.argtypes = [P(abi.Options)]
    L.sdfibm_options_default.restype = None
    L.sdfibm_cuda_create.argtypes = [P(abi.MeshDesc), P(abi.SolidDesc), i32, P(abi.Options), vp, P(vp)]
    L.sdfibm_cuda_create_polymesh.argtypes = [vp, i64, vp, vp, i64, vp, vp, i64, i32, P(abi.SolidDesc), i32,
                                              P(abi.Options), vp, P(vp)]
    L.sdfibm_cuda_interact.argtypes = [vp, dbl, dbl, vp, vp, vp, vp, vp, vp]
    L.sdfibm_cuda_interact_host.argtypes = [vp, dbl, dbl, vp, vp, vp, vp, vp, vp]
    L.sdfibm_cuda_interact_host64.argtypes = [vp, dbl, dbl, vp, vp, vp, vp, vp, vp]
    L.sdfibm_cuda_evolve.argtypes = [vp, dbl, dbl]
    L.sdfibm_cuda_fix_internal.argtypes = [vp, vp, vp]
    L.sdfibm_cuda_apply_forcing.argtypes = [vp, dbl, vp, vp, vp, vp, vp]
    L.sdfibm_cuda_get_solids.argtypes = [vp, P(abi.SolidState), i32]
    L.sdfibm_cuda_set_solids.argtypes = [vp, P(abi.SolidState), i32]
    L.sdfibm_cuda_touched.argtypes = [vp, i32, vp, vp, i64, P(i64)]
    L.sdfibm_cuda_stats.argtypes = [vp, P(i64), i32]
    L.sdfibm_cuda_set_fraction_model.argtypes = [vp, vp, C.c_float, C.c_float]
    L.sdfibm_cuda_autotune.argtypes = [vp, dbl, vp, vp, vp, vp, vp, P(i32)]
    L.sdfibm_cuda_tuning.argtypes = [vp, P(i32), i32]
    L.sdfibm_cuda_kernel_times.argtypes = [vp, P(C.c_char_p), P(dbl), i32, P(i32)]
    L.sdfibm_cuda_touched_noalloc.argtypes = [P(abi.MeshDesc), P(abi.SolidDesc), vp, vp, vp, i64, vp]
    L.sdfibm_cuda_last_error.argtypes = [vp]
    L.sdfibm_cuda_last_error.restype = C.c_char_p
    L.sdfibm_cuda_version.restype = C.c_char_p
    L.sdfibm_cuda_destroy.argtypes = [vp]
    L.sdfibm_cuda_destroy.restype = None
    L.sdfibm_mlp_dataset.argtypes = [C.c_uint64, i64, P(abi.MlpDataDesc), vp, vp, vp, vp]
    L.sdfibm_mlp_forward.argtypes = [vp, vp, i64, i64, vp, vp]
    L.sdfibm_mlp_loss_grad.argtypes = [vp, vp, vp, i64, i64, vp, vp]
    L.sdfibm_mlp_adam.argtypes = [vp, vp, vp, vp, i32, C.c_float, vp]
    L.sdfibm_mlp_train.argtypes = [vp, vp, vp, i64, P(abi.MlpTrainDesc), vp, vp]
    L.sdfibm_abi_sizeof.argtypes = [C.c_int]
    L.sdfibm_abi_sizeof.restype = i64
    L.sdfibm_host_make_shape.argtypes = [i32, vp, vp, P(abi.ShapeDesc)]
    L.sdfibm_host_make_motion.argtypes = [i32, vp, vp]
    L.sdfibm_host_make_forcer.argtypes = [i32, vp, vp]
    L.sdfibm_host_quat_from_euler_deg.argtypes = [vp, vp]
    L.sdfibm_host_quat_from_euler_deg.restype = None
    L.sdfibm_host_make_solid.argtypes = [i32, P(abi.ShapeDesc), dbl, i32, vp, i32, vp, vp, vp, vp, vp,
                                         P(abi.SolidDesc)]
    L.sdfibm_host_parse_soliddict.argtypes = [C.c_char_p, dbl, P(abi.SolidDesc), i32, P(i32), P(abi.Options),
                                              P(i32), C.c_char_p, i32]
    L.sdfibm_host_euler_from_quat.argtypes = [vp, vp]
    L.sdfibm_host_euler_from_quat.restype = None
    L.sdfibm_host_format_state.argtypes = [dbl, i32, P(abi.SolidState), i32, C.c_char_p, i64, P(i64)]
    L.sdfibm_host_write_restart.argtypes = [C.c_char_p, P(abi.SolidState), i32, i32, i32, C.c_char_p, C.c_char_p,
                                            i64, P(i64), C.c_char_p, i32]
    L.sdfibm_host_soliddict_lookup.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, i64, P(i64)]
    L.sdfibm_host_format_mean_field.argtypes = [vp, i32, C.c_char_p, i64, P(i64)]
    L.sdfibm_host_parse_vofdict.argtypes = [C.c_char_p, i32, P(abi.SolidDesc), i32, P(i32), P(i32), C.c_char_p, i32]
    L.sdfibm_host_write_vector_field.argtypes = [C.c_char_p, i64, vp, i64, i32, i32, C.c_char_p, i64, P(i64),
                                                 C.c_char_p, i32]
    L.sdfibm_host_read_foam_list.argtypes = [C.c_char_p, i64, i32, vp, i64, P(i64), C.c_char_p, i32]
    L.sdfibm_host_read_foam_faces.argtypes = [C.c_char_p, i64, vp, i64, vp, i64, P(i64), P(i64), C.c_char_p, i32]
    L.sdfibm_host_uniform_mesh.argtypes = [vp, i64, i64, dbl, P(abi.MeshDesc), C.c_char_p, i32]
    L.sdfibm_host_soliddict_shape.argtypes = [C.c_char_p, C.c_char_p, P(abi.ShapeDesc), C.c_char_p, i32]
    L.sdfibm_host_parse_blockmesh.argtypes = [C.c_char_p, P(abi.MeshDesc), C.c_char_p, i32]
    L.sdfibm_host_write_scalar_field.argtypes = [C.c_char_p, i64, vp, i64, i32, i32, C.c_char_p, i64, P(i64),
                                                 C.c_char_p, i32]
    _lib = L
    return L
