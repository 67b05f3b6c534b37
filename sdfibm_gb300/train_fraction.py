"""Trains the learned cut-cell fraction model on the GPU and writes sdfibm_gb300/data/fraction_mlp.npz.

    python -m sdfibm_gb300.train_fraction [--train 16000000] [--test 1000000] [--epochs 120] [--out PATH]

Steps, all through libsdfibm_cuda.so:
  1. labelled cut cells (sdfibm_mlp_dataset): random spheres, ellipsoids, boxes, planes, circle and ellipse prisms
     under random rotation and translation, cell size / radius log-uniform in [hr_min, hr_max], label = fraction of
     a 16^3 lattice of isInside samples (SUBSAMPLE with 4096 samples, FP64 inside tests); the model's inputs and
     prior come from the same device code as in the coupling path;
  2. Adam on the mean squared error, every gradient from the tensor-core forward + backward kernels
     (sdfibm_mlp_train);
  3. held-out cells of the same distribution: the model's error against the label, and the error of its prior alone
     (the 4^3 sub-cell planar reconstruction, network output zero), per shape family;
  4. the confidence band, calibrated on a coupling workload that the benchmark does not use: the 512^3 workload's
     distribution of spheres / ellipsoids / boxes drawn with another seed (16384 solids on 512^3).  For a grid of
     (tau_refine, rho_min) the learned step's As and per-solid force are compared with a SUBSAMPLE 16^3 step; the band
     kept is the one with the smallest fallback share whose As mean, As 99th percentile and per-solid force median
     and 90th percentile stay within the limits.  The force limits default to 0.9 of the contract's 1e-4: the 90th
     percentile moves by a few per cent between draws of the same distribution, and a band chosen exactly at the
     limit on one draw can land above it on another;
  5. the model file, with the training record (data description, losses, held-out errors, calibration table,
     timings) in `meta`.
"""
import argparse
import json
import time

import numpy as np

from . import learned

TAU_GRID = (1e30, 0.1, 0.05, 0.04, 0.03, 0.02, 0.01, 0.005)
RHO_GRID = (0.0, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5, 4.0, 4.5, 5.0, 6.0)


def band_score(torch, feat):
    """|P4 - P2| of the clamped reconstructions from feature records [17, n] (the formula of in_band in mlp.cuh)."""
    return (torch.sigmoid(feat[16].double()) - torch.sigmoid(feat[15].double())).abs()


def heldout_report(torch, params, tf, tl, rec):
    """Errors of the model and of its prior alone on held-out cells, overall and per shape family."""
    pred = learned.forward(torch, params, tf)
    p0 = params.clone()
    p0[-65:] = 0.0  # network output zero: the prior alone
    prior = learned.forward(torch, p0, tf)
    err, err0 = (pred - tl).abs().double(), (prior - tl).abs().double()
    qs = torch.tensor([0.5, 0.9, 0.99, 0.999], dtype=torch.float64, device=err.device)
    q = torch.quantile(err[:1 << 22], qs).tolist()
    out = dict(mean_abs=err.mean().item(), max_abs=err.max().item(), q50=q[0], q90=q[1], q99=q[2], q999=q[3],
               prior_only_mean_abs=err0.mean().item(),
               prior_only_q99=torch.quantile(err0[:1 << 22], 0.99).item())
    fam = {}
    from . import abi
    names = {abi.SHAPE_SPHERE: "sphere", abi.SHAPE_ELLIPSOID: "ellipsoid", abi.SHAPE_BOX: "box",
             abi.SHAPE_PLANE: "plane", abi.SHAPE_CIRCLE: "cylinder", abi.SHAPE_ELLIPSE: "elliptic_cylinder"}
    types = rec[:, 0].round().long()
    for t, nm in names.items():
        m = types == t
        if m.any():
            fam[nm] = dict(cells=int(m.sum()), mean_abs=err[m].mean().item(), prior_only=err0[m].mean().item())
    out["per_family"] = fam
    return out


def calibrate_band(torch, params_np, limits, scale=1.0, seed=6):
    """Band on a coupling workload the benchmark does not use; returns (tau_refine, rho_min, table)."""
    from . import abi, workloads
    from .cloud import SolidCloud
    w = workloads.poly3d_512(scale=scale, seed=seed, collision=abi.COLLISION_OFF)
    U = w.U_torch()
    ref = SolidCloud(w.mesh, w.solids, abi.options(rho_f=w.opt.rho_f, fraction_method=abi.FRACTION_SUBSAMPLE,
                                                   subsample_n=16))
    fr = ref.new_fields()
    FTr = ref.interact(0.0, w.dt, U, fr)
    ref.close()
    cloud = SolidCloud(w.mesh, w.solids, abi.options(rho_f=w.opt.rho_f, fraction_method=abi.FRACTION_LEARNED,
                                                     learned_fallback_n=16))
    fl = cloud.new_fields()
    table = []
    for tau in TAU_GRID:
        for rho in RHO_GRID:
            cloud.set_fraction_model(params_np, tau, rho)
            FT = cloud.interact(0.0, w.dt, U, fl)
            st = cloud.stats()
            acc = learned.accuracy(torch, w, fl, FT, fr, FTr, U)
            acc.update(tau_refine=tau, rho_min=rho,
                       fallback_share=st["learned_fallback_cells"] / max(1, st["learned_cells"]))
            table.append(acc)
    cloud.close()
    ok = [r for r in table if r["as_abs_err_mean"] <= limits["mean"] and r["as_abs_err_p99"] <= limits["q99"] and
          r["force_rel_err_median"] <= limits["force_median"] and r["force_rel_err_p90"] <= limits["force_p90"]]
    why = "As mean, As p99, force median and force p90 within the limits"
    if not ok:
        ok = [r for r in table if r["as_abs_err_mean"] <= limits["mean"] and r["as_abs_err_p99"] <= limits["q99"]]
        why = "no band met the force limit; As mean and p99 within the limits"
    if not ok:
        ok = [min(table, key=lambda r: r["as_abs_err_mean"])]
        why = "no band met the As limits; the band with the lowest As mean"
    best = min(ok, key=lambda r: (r["fallback_share"], -r["tau_refine"]))
    return best["tau_refine"], best["rho_min"], dict(
        workload="poly3d_512 distribution, seed %d, scale %g: %dx%dx%d mesh, %d solids" % (
            seed, scale, w.mesh.nx, w.mesh.ny, w.mesh.nz, len(w.solids)),
        reference="SUBSAMPLE 16^3 (4096 samples) step of the same workload", limits=limits, chosen_because=why,
        chosen=best, table=table)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--train", type=int, default=16_000_000)
    ap.add_argument("--test", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=120)
    ap.add_argument("--batch", type=int, default=32768)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--hr-min", type=float, default=0.05)
    ap.add_argument("--hr-max", type=float, default=1.5)
    ap.add_argument("--n-sub", type=int, default=16)
    ap.add_argument("--families", default="all", help="all, or a comma list of sphere,ellipsoid,box,plane,cylinder,"
                                                        "elliptic_cylinder")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--band-mean", type=float, default=1e-3)
    ap.add_argument("--band-p99", type=float, default=1e-2)
    ap.add_argument("--band-force", type=float, default=0.9e-4, help="limit of the per-solid force error median")
    ap.add_argument("--band-force-p90", type=float, default=0.9e-4, help="limit of its 90th percentile")
    ap.add_argument("--no-calibrate", action="store_true")
    ap.add_argument("--out", default=learned.MODEL_PATH)
    a = ap.parse_args(argv)
    import torch
    torch.cuda.init()
    from . import abi
    names = dict(sphere=abi.MLP_SPHERE, ellipsoid=abi.MLP_ELLIPSOID, box=abi.MLP_BOX, plane=abi.MLP_PLANE,
                 cylinder=abi.MLP_CYLINDER, elliptic_cylinder=abi.MLP_ELLIPTIC_CYL)
    fam = learned.ALL_FAMILIES if a.families == "all" else sum(names[x] for x in a.families.split(","))
    dkw = dict(hr=(a.hr_min, a.hr_max), n_sub=a.n_sub, families=fam)
    t0 = time.time()
    feat, label, _ = learned.make_dataset(torch, a.train, seed=a.seed, **dkw)
    tf, tl, rec = learned.make_dataset(torch, a.test, seed=a.seed + 1, recipe=True, **dkw)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    p = torch.from_numpy(learned.init_params(a.seed)).cuda()
    t0 = time.time()
    losses = learned.train(torch, p, feat, label, epochs=a.epochs, batch=a.batch, lr=a.lr,
                           warmup_steps=min(500, a.train // a.batch))
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del feat, label
    held = heldout_report(torch, p, tf, tl, rec)
    score = band_score(torch, tf)
    curve = []
    err = (learned.forward(torch, p, tf) - tl).abs().double()
    for qq in (0.5, 0.8, 0.9, 0.95, 0.99, 1.0):
        t = torch.quantile(score[:1 << 22], qq).item()
        e = err[score <= t]
        curve.append(dict(accepted=(score <= t).double().mean().item(), tau_refine=t, mean=e.mean().item(),
                          q99=torch.quantile(e[:1 << 22], 0.99).item()))
    params_np = p.cpu().numpy()
    tau, rho, calib = (1e30, 0.0, None)
    if not a.no_calibrate:
        tau, rho, calib = calibrate_band(torch, params_np, dict(mean=a.band_mean, q99=a.band_p99,
                                                                force_median=a.band_force,
                                                                force_p90=a.band_force_p90))
    meta = dict(model="sigmoid(logit(P4) + network(16 inputs)): P4/P2 the 4^3/2^3 sub-cell planar reconstructions "
                      "of the 5^3 distance stencil",
                data=dict(train=a.train, test=a.test, seed=a.seed, hr=[a.hr_min, a.hr_max], n_sub=a.n_sub,
                          families=a.families, z_axis_frac=0.25),
                train=dict(epochs=a.epochs, batch=a.batch, lr=a.lr, loss_per_epoch=[float(x) for x in losses],
                           seconds=t_train, data_seconds=t_data),
                test=held, band_curve_on_test=curve,
                band=dict(tau_refine=tau, rho_min=rho, fallback_n=16, calibration=calib))
    learned.save_model(params_np, tau, rho, meta, a.out)
    print(json.dumps(dict(test=held, band=dict(tau_refine=tau, rho_min=rho,
                                              chosen=calib["chosen"] if calib else None),
                          train_seconds=t_train, final_loss=float(losses[-1]))))


if __name__ == "__main__":
    main()
