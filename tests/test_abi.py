"""The C ABI library loads, exports every declared entry point, and its structs match the ctypes mirror (CPU)."""
import ctypes as C
import os
import re

from sdfibm_gb300 import abi
from sdfibm_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for h in ("sdfibm_cuda.h", "sdfibm_host.h", "sdfibm_mlp.h"):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\b(sdfibm_\w+)\s*\(", txt)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(cuda_lib):
    syms = declared_symbols()
    assert len(syms) >= 19
    for s in syms:
        assert hasattr(cuda_lib, s), s
    assert set(_lib.CUDA_SYMBOLS + _lib.HOST_SYMBOLS + _lib.MLP_SYMBOLS) <= set(syms)


def test_struct_layouts(cuda_lib):
    for i, t in enumerate((abi.MeshDesc, abi.ShapeDesc, abi.SolidDesc, abi.SolidState, abi.Options, abi.MlpDataDesc,
                           abi.MlpTrainDesc)):
        assert cuda_lib.sdfibm_abi_sizeof(i) == C.sizeof(t), t.__name__


def test_version_and_defaults(cuda_lib):
    assert b"sm_103a" in cuda_lib.sdfibm_cuda_version()
    o = abi.Options()
    cuda_lib.sdfibm_options_default(C.byref(o))
    assert o.rho_f == 1.0 and o.subsample_n == 10 and o.exact_forcing == 1 and o.collision_mode == 0


def test_bad_arguments_are_rejected_without_a_gpu(cuda_lib):
    h = C.c_void_p()
    bad = abi.mesh_desc((0, 1, 1), (0, 0, 0), (1, 1, 1))
    assert cuda_lib.sdfibm_cuda_create(C.byref(bad), None, 0, None, None, C.byref(h)) == abi.ERR_ARG
    assert cuda_lib.sdfibm_cuda_interact(None, 0.0, 1.0, None, None, None, None, None, None) == abi.ERR_ARG
    assert cuda_lib.sdfibm_mlp_forward(None, None, 0, 0, None, None) == abi.ERR_ARG
    assert cuda_lib.sdfibm_mlp_loss_grad(None, None, None, 0, 0, None, None) == abi.ERR_ARG
    assert cuda_lib.sdfibm_mlp_dataset(1, 0, None, None, None, None, None) == abi.ERR_ARG
    assert cuda_lib.sdfibm_mlp_train(None, None, None, 0, None, None, None) == abi.ERR_ARG
    assert cuda_lib.sdfibm_cuda_evolve(None, 0.0, 1.0) == abi.ERR_ARG
