"""GB300 (sm_103a) drop-in for sdfibm's fluid-solid coupling: SolidCloud::interact / evolve / fixInternal.

The compute path lives in libsdfibm_cuda.so (hand-written CUDA + C ABI, see include/sdfibm_cuda.h); this package
holds its ctypes binding, the host-side construction of solids and the synthetic workloads.
"""
from . import abi  # noqa: F401

__all__ = ["abi", "build", "cloud", "host", "workloads"]
