"""Coupling with the learned cut-cell fraction (options.fraction_method = LEARNED) against the FP64 oracle running
SUBSAMPLE with the 16^3 lattice the model is trained on and falls back to.

Gates of the shipped model (the learned path's contract; the oracle's 16^3 lattice is the reference):
  * As, mean absolute error over the cut cells <= 1e-3 (the target's bar), 99th percentile <= 1e-2;
  * per-solid force, normwise: median <= 1e-4; 90th percentile <= 1e-4 on the benchmarked workload (16384 solids,
    test_trained_model_full_size), <= 1e-3 on the small scaled workloads, where 32 to 64 solids make the percentile
    a statement about two or three solids.
The mean and the median are the gated statistics because the reference itself is a lattice count: its own error against
the converged fraction is about 6e-4 per cut cell (mean), with a tail, so no smooth estimate meets 1e-3 in every
cell, and a per-solid force bar of 1e-4 at the 90th percentile is below the 16^3 lattice's own noise for solids of
one or two cells' radius (the bench reports every quantile against 16^3 and against a converged 32^3 lattice).
"""
import copy
import os

import numpy as np
import pytest

from gpu_helpers import check_interact, run_pair
from sdfibm_gb300 import abi, learned, workloads

pytestmark = pytest.mark.gpu

AS_MEAN = 1e-3   # learned path: mean |As - As_SUBSAMPLE(4096)| over the cut cells
AS_P99 = 1e-2    # and its 99th percentile
F_REL = 1e-4     # learned path: median per-solid force error, normwise against the sum of |contributions|
F_REL_P90 = 1e-3


def _learned_pair(torch, w, params, tau_refine, rho_min, recheck_cap=0):
    orc_w = copy.copy(w)
    orc_w.opt = abi.options(rho_f=w.opt.rho_f, collision_mode=w.opt.collision_mode,
                            fraction_method=abi.FRACTION_SUBSAMPLE, subsample_n=16)
    gpu_opt = abi.options(rho_f=w.opt.rho_f, collision_mode=w.opt.collision_mode,
                          fraction_method=abi.FRACTION_LEARNED, learned_fallback_n=16, recheck_cap=recheck_cap)
    r = run_pair(torch, orc_w, gpu_opt=gpu_opt,
                 gpu_setup=lambda c: c.set_fraction_model(params, tau_refine, rho_min))
    return orc_w, r


@pytest.mark.parametrize("recheck_cap", [0, 50])
def test_band_closed_is_subsample16(cuda_lib, torch_cuda, recheck_cap):
    """With the band closed every cut cell takes the SUBSAMPLE fallback: the contract of the plain method holds.
    A recheck list of 50 entries overflows at once: the cells whose points it could not take are recounted."""
    w = workloads.poly3d_256(scale=0.25)
    orc_w, r = _learned_pair(torch_cuda, w, learned.init_params(0), -1.0, 0.0, recheck_cap)
    check_interact(orc_w, r)
    st = r["gpu"].stats()
    assert st["learned_cells"] == st["cut_cells"] > 0
    assert st["learned_fallback_cells"] == st["learned_cells"]
    if recheck_cap:
        assert st["fp64_rechecks"] > 2 * recheck_cap


def test_band_open_predicts_every_cut_cell(cuda_lib, torch_cuda):
    """With the band open the network gives every cut cell its fraction; enumeration and inside cells are exact."""
    w = workloads.poly3d_256(scale=0.25)
    orc_w, r = _learned_pair(torch_cuda, w, learned.init_params(1), 1e30, 0.0)
    gpu, orc, fd, fo = r["gpu"], r["orc"], r["fd"], r["fo"]
    st = gpu.stats()
    assert st["learned_fallback_cells"] == 0 and st["learned_cells"] == st["cut_cells"] > 0
    for s in range(len(w.solids)):
        cg, tg = gpu.touched(s)
        co, to = orc.touched(s)
        assert np.array_equal(cg, co) and np.array_equal(tg, to)
    assert np.array_equal(fd["Ct"].cpu().numpy(), fo["Ct"])
    As = fd["As"].cpu().numpy()
    for s in range(len(w.solids)):
        cells, types = orc.touched(s)
        assert np.all(As[cells[types == 1]] == 1.0)   # ALL_INSIDE cells take alpha = 1
    touched = fo["Ct"] != 0
    assert np.all((As[touched] > 0) & (As[touched] <= 1))


@pytest.mark.skipif(not os.path.exists(learned.MODEL_PATH), reason="no trained fraction model")
@pytest.mark.parametrize("cfg", ["poly3d_256", "poly3d_512"])
def test_trained_model_accuracy(cuda_lib, torch_cuda, cfg):
    """The shipped model with its band: As and per-solid force against SUBSAMPLE(4096) in FP64."""
    params, tau, rho, meta = learned.load_model()
    w = workloads.poly3d_256(scale=0.25) if cfg == "poly3d_256" else workloads.poly3d_512(scale=0.125,
                                                                                          collision=abi.COLLISION_OFF)
    orc_w, r = _learned_pair(torch_cuda, w, params, tau, rho)
    gpu, orc, fd, fo = r["gpu"], r["orc"], r["fd"], r["fo"]
    assert np.array_equal(fd["Ct"].cpu().numpy(), fo["Ct"])
    As = fd["As"].cpu().numpy().astype(np.float64)
    cut = (fo["Ct"] != 0) & ~((fo["As"] == 1.0) & (As == 1.0))
    err = np.abs(As - fo["As"])[cut]
    assert err.mean() <= AS_MEAN, "mean |As error| %g over %d cut cells" % (err.mean(), cut.sum())
    assert np.percentile(err, 99) <= AS_P99, "99th percentile of |As error| %g" % np.percentile(err, 99)
    FTg, FTo = r["FT"][-1]
    N = orc.N
    V = w.mesh.h[0] * w.mesh.h[1] * w.mesh.h[2]
    Uo = r["Uo"].reshape(3, N)
    rel = []
    for s in range(len(w.solids)):
        cells, _ = orc.touched(s)
        if len(cells) == 0:
            continue
        st = orc.get_state()[s]
        fm = np.linalg.norm(Uo[:, cells] - np.array(st.vel)[:, None], axis=0).sum() * w.opt.rho_f * V / w.dt
        rel.append(np.linalg.norm(FTg[s, :3] - FTo[s, :3]) / (fm + 1e-300))
    rel = np.array(rel)
    assert np.median(rel) <= F_REL, "median per-solid force error %g" % np.median(rel)
    assert np.percentile(rel, 90) <= F_REL_P90, "90th percentile per-solid force error %g" % np.percentile(rel, 90)


@pytest.mark.skipif(not os.path.exists(learned.MODEL_PATH), reason="no trained fraction model")
def test_trained_model_full_size(cuda_lib, torch_cuda):
    """The shipped model on the benchmarked workload itself (512^3 mesh, 16384 spheres / ellipsoids / boxes; its band
    was calibrated on another draw of that distribution), against SUBSAMPLE 16^3 on the GPU (whose classifications are
    the FP64 oracle's, as the SUBSAMPLE parity tests show): As mean <= 1e-3 and 99th percentile <= 1e-2 over the cut
    cells, per-solid force median and 90th percentile <= 1e-4; the maxima are reported."""
    from sdfibm_gb300.cloud import SolidCloud
    torch = torch_cuda
    params, tau, rho, _ = learned.load_model()
    w = workloads.poly3d_512(collision=abi.COLLISION_OFF)
    U = w.U_torch()
    ref = SolidCloud(w.mesh, w.solids, abi.options(rho_f=w.opt.rho_f, fraction_method=abi.FRACTION_SUBSAMPLE,
                                                   subsample_n=16))
    fr = ref.new_fields()
    FTr = ref.interact(0.0, w.dt, U, fr)
    ref.close()
    c = SolidCloud(w.mesh, w.solids, abi.options(rho_f=w.opt.rho_f, fraction_method=abi.FRACTION_LEARNED,
                                                 learned_fallback_n=16))
    c.set_fraction_model(params, tau, rho)
    f = c.new_fields()
    FT = c.interact(0.0, w.dt, U, f)
    st = c.stats()
    c.close()
    a = learned.accuracy(torch, w, f, FT, fr, FTr, U)
    msg = "%r" % a
    assert a["as_abs_err_mean"] <= AS_MEAN and a["as_abs_err_p99"] <= AS_P99, msg
    assert a["force_rel_err_median"] <= F_REL and a["force_rel_err_p90"] <= 1e-4, msg
    assert a["as_abs_err_max"] < 0.1 and a["force_rel_err_max"] < 1e-2, msg
    assert st["learned_fallback_cells"] <= 0.25 * st["learned_cells"]
