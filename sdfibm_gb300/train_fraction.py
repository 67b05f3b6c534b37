"""Trains the learned cut-cell fraction model on the GPU and writes sdfibm_gb300/data/fraction_mlp.npz.

    python -m sdfibm_gb300.train_fraction [--train 10000000] [--test 1000000] [--epochs 40] [--out PATH]

Steps, all through libsdfibm_cuda.so:
  1. labelled cut cells (sdfibm_mlp_dataset): random spheres, ellipsoids, boxes, planes, circle and ellipse
     prisms under random rotation and translation, cell size / radius log-uniform in [hr_min, hr_max], label =
     fraction of a 16^3 lattice of isInside samples (SUBSAMPLE with 4096 samples);
  2. Adam on the mean squared error, every gradient from the tensor-core forward + backward kernels
     (sdfibm_mlp_train);
  3. the confidence band: on held-out cells, the largest (tau_twist, tau_grad) box whose accepted cells keep the
     mean absolute error at most --band-mean and the 99th percentile at most --band-p99;
  4. the model file, with the training record (data description, losses, held-out errors, timings) in `meta`.
"""
import argparse
import json
import time

import numpy as np

from . import learned


def band_scores(torch, feat):
    """(twist sum, | |trilinear gradient| - 1 |) of every cell; the formulas of in_band in mlp.cuh."""
    f = feat[:8]
    tw = ((f[0] - f[1] - f[2] + f[3]).abs() + (f[4] - f[5] - f[6] + f[7]).abs() + (f[0] - f[1] - f[4] + f[5]).abs() +
          (f[2] - f[3] - f[6] + f[7]).abs() + (f[0] - f[2] - f[4] + f[6]).abs() + (f[1] - f[3] - f[5] + f[7]).abs())
    gx = 0.25 * (((f[1] - f[0]) + (f[3] - f[2])) + ((f[5] - f[4]) + (f[7] - f[6])))
    gy = 0.25 * (((f[2] - f[0]) + (f[3] - f[1])) + ((f[6] - f[4]) + (f[7] - f[5])))
    gz = 0.25 * (((f[4] - f[0]) + (f[5] - f[1])) + ((f[6] - f[2]) + (f[7] - f[3])))
    return tw, ((gx * gx + gy * gy + gz * gz).sqrt() - 1.0).abs()


def calibrate(torch, err, tw, gd, mean_max, p99_max):
    """Largest accepted fraction over a grid of (tau_twist, tau_grad) quantiles meeting both error limits."""
    qs = torch.tensor([0.5, 0.6, 0.7, 0.8, 0.85, 0.9, 0.93, 0.95, 0.97, 0.98, 0.99, 0.995, 0.999, 1.0],
                      device=err.device)
    tws = torch.quantile(tw[:1 << 20].double(), qs.double()).float()
    gds = torch.quantile(gd[:1 << 20].double(), qs.double()).float()
    best = (0.0, 0.0, 0.0, float("nan"), float("nan"))
    for a in tws.tolist():
        for b in gds.tolist():
            acc = (tw <= a) & (gd <= b)
            frac = acc.float().mean().item()
            if frac <= best[0]:
                continue
            e = err[acc]
            if e.numel() == 0:
                continue
            m = e.mean().item()
            p = torch.quantile(e[:1 << 22].double(), 0.99).item()
            if m <= mean_max and p <= p99_max:
                best = (frac, a, b, m, p)
    return best


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--train", type=int, default=10_000_000)
    ap.add_argument("--test", type=int, default=1_000_000)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--batch", type=int, default=32768)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--hr-min", type=float, default=0.01)
    ap.add_argument("--hr-max", type=float, default=1.5)
    ap.add_argument("--n-sub", type=int, default=16)
    ap.add_argument("--families", default="all", help="all, or a comma list of sphere,ellipsoid,box,plane,cylinder,"
                                                        "elliptic_cylinder")
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--band-mean", type=float, default=7e-4)
    ap.add_argument("--band-p99", type=float, default=1e-2)
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
    tf, tl, _ = learned.make_dataset(torch, a.test, seed=a.seed + 1, **dkw)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    p = torch.from_numpy(learned.init_params(a.seed)).cuda()
    t0 = time.time()
    losses = learned.train(torch, p, feat, label, epochs=a.epochs, batch=a.batch, lr=a.lr,
                           warmup_steps=min(500, a.train // a.batch))
    torch.cuda.synchronize()
    t_train = time.time() - t0
    pred = learned.forward(torch, p, tf)
    err = (pred - tl).abs()
    # the planar prior alone (network output zero)
    p0 = p.clone()
    p0[-65:] = 0.0
    err0 = (learned.forward(torch, p0, tf) - tl).abs()
    tw, gd = band_scores(torch, tf)
    frac, tau_tw, tau_gd, m_acc, p_acc = calibrate(torch, err, tw, gd, a.band_mean, a.band_p99)
    # error of the accepted cells against the fraction accepted, twist limit only
    curve = []
    for qq in (0.3, 0.5, 0.7, 0.8, 0.9, 0.95, 0.99, 1.0):
        t = torch.quantile(tw[:1 << 20].double(), qq).item()
        e = err[tw <= t].double()
        curve.append(dict(accepted=(tw <= t).float().mean().item(), tau_twist=t, mean=e.mean().item(),
                          q99=torch.quantile(e[:1 << 22], 0.99).item(),
                          q999=torch.quantile(e[:1 << 22], 0.999).item(),
                          prior_only_mean=err0[tw <= t].double().mean().item()))
    q = torch.quantile(err[:1 << 22].double(), torch.tensor([0.5, 0.9, 0.99, 0.999], dtype=torch.float64,
                                                            device=err.device)).tolist()
    meta = dict(data=dict(train=a.train, test=a.test, seed=a.seed, hr=[a.hr_min, a.hr_max], n_sub=a.n_sub,
                          families=a.families, z_axis_frac=0.25),
                train=dict(epochs=a.epochs, batch=a.batch, lr=a.lr, loss_per_epoch=[float(x) for x in losses],
                           seconds=t_train, data_seconds=t_data),
                test=dict(mean_abs=err.mean().item(), max_abs=err.max().item(), q50=q[0], q90=q[1], q99=q[2],
                          q999=q[3], prior_only_mean_abs=err0.mean().item()),
                model="sigmoid(logit(planar fraction) + gate * network), gate = twist / (1 + twist)",
                band=dict(tau_twist=tau_tw, tau_grad=tau_gd, accepted=frac, accepted_mean_abs=m_acc,
                          accepted_q99=p_acc, limits=dict(mean=a.band_mean, q99=a.band_p99), curve=curve))
    learned.save_model(p.cpu().numpy(), tau_tw, tau_gd, meta, a.out)
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
