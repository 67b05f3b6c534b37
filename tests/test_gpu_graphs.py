"""CUDA-graph replay of interact and evolve (options.graphs = 1) gives the fields of direct launches bit for bit, and
their forces and solid states up to the order of FP64 atomic sums, over steps whose time and dt change; the
autotuner keeps results."""
import copy

import numpy as np
import pytest

from sdfibm_gb300 import abi, workloads
from sdfibm_gb300.cloud import SolidCloud

pytestmark = pytest.mark.gpu


def _run(torch, w, graphs, steps):
    s = torch.cuda.Stream()
    opt = copy.copy(w.opt)
    opt.graphs = graphs
    U = torch.from_numpy(w.U_numpy()).cuda()
    torch.cuda.synchronize()
    cloud = SolidCloud(w.mesh, w.solids, opt, stream=s)
    with torch.cuda.stream(s):
        f = cloud.new_fields()
    s.synchronize()
    out = []
    t = 0.0
    for i in range(steps):
        dt = w.dt * (1.0 + 0.1 * i)  # a changing step size exercises the replayed parameter node
        out.append(cloud.interact(t, dt, U, f))
        cloud.evolve(t, dt)
        t += dt
    s.synchronize()
    fields = {k: v.cpu().numpy() for k, v in f.items()}
    st = [np.array(list(x.pos) + list(x.vel) + list(x.quat) + list(x.omega)) for x in cloud.states()]
    launches = cloud.stats()["launches"]
    cloud.close()
    return out, fields, st, launches


@pytest.mark.parametrize("cfg", ["sedimentation2d", "poly3d_256"])
def test_graph_replay_is_bit_identical(cuda_lib, torch_cuda, cfg):
    if cfg == "sedimentation2d":
        w = workloads.sedimentation2d(scale=0.125, ncircles=12)
    else:
        w = workloads.poly3d_256(scale=0.25, collision=abi.COLLISION_SPHERES)
        w.opt.fraction_method = abi.FRACTION_SUBSAMPLE
    a = _run(torch_cuda, w, 0, 4)
    b = _run(torch_cuda, w, 1, 4)
    # forces sum FP64 atomics from many warps: equal up to the order of those sums
    for x, y in zip(a[0], b[0]):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-14)
    for k in a[1]:
        assert np.array_equal(a[1][k], b[1][k]), k
    for x, y in zip(a[2], b[2]):
        np.testing.assert_allclose(x, y, rtol=1e-12, atol=1e-14)
    assert a[3] == b[3] > 0


def test_autotune_keeps_results(cuda_lib, torch_cuda):
    """The autotuner only changes the launch configuration (classify work-item size, CTA counts): fields and forces
    equal an untuned context's, and a second context of the same shape takes the choice from the cache."""
    torch = torch_cuda
    w = workloads.poly3d_256(scale=0.25)
    w.opt.fraction_method = abi.FRACTION_SUBSAMPLE
    U = torch.from_numpy(w.U_numpy()).cuda()
    a = SolidCloud(w.mesh, w.solids, w.opt)
    b = SolidCloud(w.mesh, w.solids, w.opt)
    fa, fb = a.new_fields(), b.new_fields()
    chosen = b.autotune(w.dt, U, fb)
    assert chosen in (2, 4, 8, 16, 32)
    assert b.stats()["work_items"] >= 1
    FTa = a.interact(0.0, w.dt, U, fa)
    FTb = b.interact(0.0, w.dt, U, fb)
    for k in fa:
        assert torch.equal(fa[k], fb[k]), k
    np.testing.assert_allclose(FTa, FTb, rtol=1e-12, atol=1e-14)
    t = b.tuning()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert t["classify_tiles_per_item"] == chosen and t["from_cache"] == 0
    for k in ("classify_ctas", "subsample_ctas", "couple_ctas", "mlp_ctas", "refgeo_ctas"):
        assert t[k] > 0 and t[k] % sms == 0, (k, t)
    c = SolidCloud(w.mesh, w.solids, w.opt)
    fc = c.new_fields()
    assert c.autotune(w.dt, U, fc) == chosen
    tc = c.tuning()
    assert tc["from_cache"] == 1 and {k: v for k, v in tc.items() if k != "from_cache"} == \
        {k: v for k, v in t.items() if k != "from_cache"}
    FTc = c.interact(0.0, w.dt, U, fc)
    for k in fa:
        assert torch.equal(fa[k], fc[k]), k
    np.testing.assert_allclose(FTa, FTc, rtol=1e-12, atol=1e-14)
    a.close()
    b.close()
    c.close()
