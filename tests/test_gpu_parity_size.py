"""GPU coupling against the FP64 oracle at the benchmarked sizes.

  * the 256^3 mesh with 4096 spheres and ellipsoids at full size, REF-GEO and SUBSAMPLE 10^3;
  * the 512^3 / 16384-solid workload at half scale per axis (256^3 mesh, 2048 spheres / ellipsoids / boxes at the same
    r/h), two coupled steps with collisions;
  * the 1024^2 sedimentation workload (4 walls, 100 circles) over 200 coupled steps with collisions and motion
    (SolidCloud::interact then SolidCloud::evolve, solidcloud.cpp:435-464, 477-562): at steps 1, 50, 100 and 200 the
    two runs' solid states are compared (their drift), the oracle takes the GPU's states, and the interact of that
    step is checked against the full coupling contract.
Contract: touched sets, types and Ct bit-exact; As, Ts, Fs per cell within 1e-5 relative; force and torque per
solid within 1e-6 normwise (gpu_helpers).
"""
import numpy as np
import pytest

from gpu_helpers import check_interact, run_pair
from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi, workloads
from sdfibm_gb300.cloud import SolidCloud

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method", [abi.FRACTION_REFGEO, abi.FRACTION_SUBSAMPLE])
def test_poly3d_256_full_size(cuda_lib, torch_cuda, method):
    w = workloads.poly3d_256()
    w.opt.fraction_method = method
    r = run_pair(torch_cuda, w)
    s = check_interact(w, r)
    assert s["coupling_cells"] > 1_000_000
    r["gpu"].close()


def test_poly3d_512_half_scale_two_steps(cuda_lib, torch_cuda):
    """Two coupled steps with collisions: the contract on each interact, the evolved states in between within the
    drift the FP32 fractions allow.  Before the second interact the oracle takes the GPU's states, so that the
    second comparison runs on the same inputs (the forcing of a cell is U - u_s, which can cancel: a 1e-7 difference
    of the states would show there as a large relative difference of Fs)."""
    torch = torch_cuda
    w = workloads.poly3d_512(scale=0.5)
    assert w.mesh.nx == 256 and len(w.solids) == 2048
    r = run_pair(torch, w, steps=1)
    check_interact(w, r)
    gpu, orc = r["gpu"], r["orc"]
    gpu.evolve(0.0, w.dt)
    orc.evolve(0.0, w.dt)
    xg, vg, og, _ = _states(gpu)
    xo, vo, oo, _ = _states(orc)
    assert np.abs(xg - xo).max() <= 1e-9 and np.abs(vg - vo).max() <= 1e-6 * (1 + np.abs(vo).max())
    orc.set_state(gpu.states())
    FTg = gpu.interact(w.dt, w.dt, r["Ud"], r["fd"])
    FTo = orc.interact(w.dt, w.dt, r["Uo"], r["fo"])
    torch.cuda.synchronize()
    r["FT"] = [(FTg, FTo)]
    check_interact(w, r)
    gpu.close()


def _states(cloud):
    st = cloud.states() if hasattr(cloud, "states") else cloud.get_state()
    return (np.array([s.pos[:] for s in st]), np.array([s.vel[:] for s in st]), np.array([s.omega[:] for s in st]),
            np.array([s.quat[:] for s in st]))


def test_sedimentation2d_full_size_200_steps(cuda_lib, torch_cuda):
    torch = torch_cuda
    w = workloads.sedimentation2d()
    assert w.mesh.nx == 1024 and len(w.solids) == 104
    Uh = w.U_numpy()
    gpu = SolidCloud(w.mesh, w.solids, w.opt)
    orc = OracleCloud(w.mesh, w.solids, w.opt, faithful=False)
    Ud = torch.from_numpy(Uh).cuda()
    Uo = Uh.astype(np.float64).reshape(-1).copy()
    fd, fo = gpu.new_fields(), orc.new_fields()
    t = 0.0
    checked = []
    moved = 0.0
    x0 = _states(orc)[0]
    for step in range(1, 201):
        if step in (1, 50, 100, 200):
            # the states after step - 1 coupled steps: the drift of the two runs (FP32 fractions and forcing against
            # FP64 feed slightly different forces into the integrator), then the oracle takes the GPU's states so
            # that the checked interact runs on the same inputs
            xg, vg, og, qg = _states(gpu)
            xo, vo, oo, qo = _states(orc)
            assert np.abs(xg - xo).max() <= 1e-8, (step, np.abs(xg - xo).max())
            assert np.abs(qg - qo).max() <= 1e-7, (step, np.abs(qg - qo).max())
            assert np.abs(vg - vo).max() <= 1e-6 * (1.0 + np.abs(vo).max()), (step, np.abs(vg - vo).max())
            assert np.abs(og - oo).max() <= 1e-5 * (1.0 + np.abs(oo).max()), (step, np.abs(og - oo).max())
            orc.set_state(gpu.states())
            moved = np.abs(xo - x0).max()
        FTg = gpu.interact(t, w.dt, Ud, fd)
        FTo = orc.interact(t, w.dt, Uo, fo)
        if step in (1, 50, 100, 200):
            torch.cuda.synchronize()
            check_interact(w, dict(gpu=gpu, orc=orc, fd=fd, fo=fo, FT=[(FTg, FTo)], Ud=Ud, Uo=Uo))
            checked.append(step)
        gpu.evolve(t, w.dt)
        orc.evolve(t, w.dt)
        t += w.dt
    assert checked == [1, 50, 100, 200]
    assert moved > 1e-3  # the circles did move over the run
    gpu.close()
