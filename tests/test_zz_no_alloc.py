"""The allocation-free touched-cell query against the regular context path (collected last on purpose).

sdfibm_cuda_touched_noalloc serves callers that cannot call cudaMalloc (device memory owned by their own pool
allocator, or loops that cannot take cudaMalloc's device-wide synchronisation): it keeps its work space in a
file-scope device array instead of allocating.  Its answer must equal what sdfibm_cuda_touched returns after an
interact of a context holding the same solid, call after call (the array is reused and must be reset correctly).
"""
import ctypes as C

import numpy as np
import pytest

from sdfibm_gb300 import abi, workloads
from sdfibm_gb300.cloud import SolidCloud

pytestmark = pytest.mark.gpu


def _noalloc(lib, torch, mesh, solid, capacity):
    cells = torch.full((max(1, capacity),), -7, dtype=torch.int32, device="cuda")
    types = torch.zeros((max(1, capacity),), dtype=torch.int8, device="cuda")
    n = torch.full((1,), -99, dtype=torch.int64, device="cuda")
    rc = lib.sdfibm_cuda_touched_noalloc(C.byref(mesh), C.byref(solid), None, C.c_void_p(cells.data_ptr()),
                                         C.c_void_p(types.data_ptr()), capacity, C.c_void_p(n.data_ptr()))
    assert rc == abi.OK
    torch.cuda.synchronize()
    k = int(n.item())
    return k, cells.cpu().numpy()[:min(k, capacity)].astype(np.int64), types.cpu().numpy()[:min(k, capacity)]


def _context(w, solid):
    cloud = SolidCloud(w.mesh, [solid], w.opt)
    import torch
    f = cloud.new_fields()
    cloud.interact(0.0, w.dt, torch.from_numpy(w.U_numpy()).cuda(), f)
    out = cloud.touched(0)
    cloud.close()
    return out


def test_noalloc_matches_context_path_two_calls_in_a_row(cuda_lib, torch_cuda):
    w = workloads.poly3d_512(scale=0.125)
    # a large solid then a small one: the second call must not see anything left by the first
    order = sorted(range(len(w.solids)), key=lambda s: -w.solids[s].shape.radiusB)
    picks = [order[0], order[-1]]
    for s in picks:
        d = w.solids[s]
        ref_cells, ref_types = _context(w, d)
        n, cells, types = _noalloc(cuda_lib, torch_cuda, w.mesh, d, 1 << 16)
        assert n == len(ref_cells) and n > 0
        assert np.array_equal(cells, ref_cells)
        assert np.array_equal(types, ref_types)


def test_noalloc_2d_and_capacity_reporting(cuda_lib, torch_cuda):
    w = workloads.cylinder2d()
    d = w.solids[0]
    ref_cells, ref_types = _context(w, d)
    n, cells, types = _noalloc(cuda_lib, torch_cuda, w.mesh, d, 8)
    assert n == len(ref_cells)                       # full count even when the buffer is short
    assert np.array_equal(cells, ref_cells[:8]) and np.array_equal(types, ref_types[:8])
    n2, cells2, types2 = _noalloc(cuda_lib, torch_cuda, w.mesh, d, 1024)
    assert n2 == n and np.array_equal(cells2, ref_cells) and np.array_equal(types2, ref_types)


def test_noalloc_rejects_oversized_bbox(cuda_lib, torch_cuda):
    from sdfibm_gb300.host import make_shape, make_solid
    mesh = abi.mesh_desc((128, 128, 128), (0, 0, 0), (1 / 128,) * 3)
    big = make_solid(0, make_shape("Sphere", radius=0.45), 1.0, (0.5, 0.5, 0.5))  # ~120^3 bbox cells
    n = torch_cuda.zeros((1,), dtype=torch_cuda.int64, device="cuda")
    cells = torch_cuda.zeros((16,), dtype=torch_cuda.int32, device="cuda")
    types = torch_cuda.zeros((16,), dtype=torch_cuda.int8, device="cuda")
    rc = cuda_lib.sdfibm_cuda_touched_noalloc(C.byref(mesh), C.byref(big), None, C.c_void_p(cells.data_ptr()),
                                              C.c_void_p(types.data_ptr()), 16, C.c_void_p(n.data_ptr()))
    assert rc == abi.ERR_CAPACITY


def test_noalloc_allocates_nothing_and_counts_without_buffers(cuda_lib, torch_cuda):
    """After a first call (which, under lazy module loading, is when the driver reserves the array), ten more calls
    leave the device's free memory unchanged; a call with capacity 0 and no output buffers still reports the
    count."""
    w = workloads.poly3d_512(scale=0.125)
    d = w.solids[0]
    ref_cells, _ = _context(w, d)
    n = torch_cuda.full((1,), -99, dtype=torch_cuda.int64, device="cuda")
    cells = torch_cuda.zeros((1 << 16,), dtype=torch_cuda.int32, device="cuda")
    types = torch_cuda.zeros((1 << 16,), dtype=torch_cuda.int8, device="cuda")

    def call(capacity, with_buffers=True):
        return cuda_lib.sdfibm_cuda_touched_noalloc(
            C.byref(w.mesh), C.byref(d), None, C.c_void_p(cells.data_ptr()) if with_buffers else None,
            C.c_void_p(types.data_ptr()) if with_buffers else None, capacity, C.c_void_p(n.data_ptr()))

    assert call(1 << 16) == abi.OK
    torch_cuda.cuda.synchronize()
    free0 = torch_cuda.cuda.mem_get_info()[0]
    alloc0 = torch_cuda.cuda.memory_allocated()
    for _ in range(10):
        assert call(1 << 16) == abi.OK
    torch_cuda.cuda.synchronize()
    assert torch_cuda.cuda.mem_get_info()[0] == free0
    assert torch_cuda.cuda.memory_allocated() == alloc0
    assert int(n.item()) == len(ref_cells)
    n.fill_(-99)
    assert call(0, with_buffers=False) == abi.OK
    torch_cuda.cuda.synchronize()
    assert int(n.item()) == len(ref_cells)
