"""GB300 (sm_103a) drop-in for sdfibm's fluid-solid coupling: SolidCloud::interact / evolve / fixInternal.

The compute path lives in libsdfibm_cuda.so (hand-written CUDA + C ABI, see include/sdfibm_cuda.h); this package
holds its ctypes binding and what surrounds it:
    cloud        SolidCloud (interact, evolve, fix_internal, mean_field, save_state, save_restart, ...)
    host         solid construction, the solidDict front end, cloud.out / meanfield.out / restart writers
    vof          the tool_vof smooth phase-field initializer
    foam_io      OpenFOAM polyMesh and field files
    learned      the learned cut-cell fraction (model files, training kernels); train_fraction trains one
    workloads    the synthetic benchmark workloads
    build        the in-tree build of the library
"""
from . import abi  # noqa: F401

__all__ = ["abi", "build", "cloud", "foam_io", "host", "learned", "vof", "workloads"]
