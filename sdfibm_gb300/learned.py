"""Host side of the learned cut-cell fraction (include/sdfibm_mlp.h): training data, forward, gradient, training,
and the model file.

Every function calls libsdfibm_cuda.so; tensors are CUDA torch tensors (torch only holds device memory and the
stream).  Feature records are [17, n] float32 (structure of arrays: the 16 network inputs, then the prior
logit(P4)), labels and predictions [n] float32, parameters [5313] float32 in the layout W1[64][16], b1, W2[64][64],
b2, w3, b3.  The model: a = sigmoid(prior + network(inputs)), see include/sdfibm_mlp.h.
"""
import ctypes as C
import json
import os

import numpy as np

from . import abi
from ._lib import load

MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "fraction_mlp.npz")
ALL_FAMILIES = (abi.MLP_SPHERE | abi.MLP_ELLIPSOID | abi.MLP_BOX | abi.MLP_PLANE | abi.MLP_CYLINDER |
                abi.MLP_ELLIPTIC_CYL)


class MlpError(RuntimeError):
    def __init__(self, status, what):
        super().__init__("%s failed with status %d" % (what, status))
        self.status = status


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _stream(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _check(rc, what):
    if rc != abi.OK:
        raise MlpError(rc, what)


def data_desc(hr=(0.01, 1.5), families=ALL_FAMILIES, n_sub=16, z_axis_frac=0.25):
    d = abi.MlpDataDesc()
    d.hr_min, d.hr_max = float(hr[0]), float(hr[1])
    d.families = int(families)
    d.n_sub = int(n_sub)
    d.z_axis_frac = float(z_axis_frac)
    return d


def make_dataset(torch, n, seed, recipe=False, **kw):
    """n labelled cut cells on the GPU: (feature records [17, n], labels [n], recipe [n, 20] float64 or None)."""
    feat = torch.empty((abi.MLP_NFEAT, n), dtype=torch.float32, device="cuda")
    label = torch.empty(n, dtype=torch.float32, device="cuda")
    rec = torch.empty((n, 20), dtype=torch.float64, device="cuda") if recipe else None
    d = data_desc(**kw)
    _check(load().sdfibm_mlp_dataset(C.c_uint64(seed), n, C.byref(d), _ptr(feat), _ptr(label), _ptr(rec),
                                     _stream(torch)), "sdfibm_mlp_dataset")
    return feat, label, rec


def forward(torch, params, feat):
    n = feat.shape[1]
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    _check(load().sdfibm_mlp_forward(_ptr(params), _ptr(feat), feat.stride(0), n, _ptr(out), _stream(torch)),
           "sdfibm_mlp_forward")
    return out


def loss_grad(torch, params, feat, label):
    """(mean loss, gradient [4993]) of loss = mean((a - label)^2) over the cells."""
    n = feat.shape[1]
    g = torch.empty(abi.MLP_NPARAM + 1, dtype=torch.float32, device="cuda")
    _check(load().sdfibm_mlp_loss_grad(_ptr(params), _ptr(feat), _ptr(label), feat.stride(0), n, _ptr(g),
                                       _stream(torch)), "sdfibm_mlp_loss_grad")
    g = g.cpu().numpy()
    return float(g[-1]) / n, g[:-1].copy()


def adam(torch, params, grad, m, v, t, lr):
    _check(load().sdfibm_mlp_adam(_ptr(params), _ptr(grad), _ptr(m), _ptr(v), int(t), C.c_float(lr), _stream(torch)),
           "sdfibm_mlp_adam")


def train(torch, params, feat, label, epochs=10, batch=16384, lr=2e-3, lr_final_frac=0.02, warmup_steps=200):
    """Trains `params` (device tensor) in place; returns the mean loss of every epoch."""
    d = abi.MlpTrainDesc()
    d.epochs, d.batch, d.lr, d.lr_final_frac, d.warmup_steps = int(epochs), int(batch), float(lr), \
        float(lr_final_frac), int(warmup_steps)
    losses = np.zeros(epochs, dtype=np.float32)
    _check(load().sdfibm_mlp_train(_ptr(params), _ptr(feat), _ptr(label), feat.shape[1], C.byref(d),
                                   losses.ctypes.data_as(C.c_void_p), _stream(torch)), "sdfibm_mlp_train")
    return losses


def init_params(seed=0):
    """Fan-in scaled uniform initialisation (zero biases), output layer small: the model starts near its prior."""
    rng = np.random.default_rng(seed)
    n_in = abi.MLP_NIN
    W1 = rng.uniform(-1, 1, (64, n_in)) * np.sqrt(3.0 / n_in)
    W2 = rng.uniform(-1, 1, (64, 64)) * np.sqrt(3.0 / 64)
    w3 = rng.uniform(-1, 1, 64) * np.sqrt(3.0 / 64) * 0.1
    return np.concatenate([W1.ravel(), np.zeros(64), W2.ravel(), np.zeros(64), w3, [0.0]]).astype(np.float32)


def save_model(params, tau_refine, rho_min, meta, path=MODEL_PATH):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez(path, params=np.asarray(params, np.float32), tau_refine=np.float32(tau_refine),
             rho_min=np.float32(rho_min), meta=json.dumps(meta))


def load_model(path=MODEL_PATH):
    """(params float32 [5313], tau_refine, rho_min, meta dict) of a trained model file: the network and its
    confidence band (|P4 - P2| limit, smallest solid bounding radius in cells)."""
    z = np.load(path)
    return z["params"].astype(np.float32), float(z["tau_refine"]), float(z["rho_min"]), json.loads(str(z["meta"]))


def accuracy(torch, w, f, FT, fr, FTr, U, reference="SUBSAMPLE 16^3 (4096 samples), same step"):
    """As of a coupling step (fields f, force/torque FT) against a reference step (fr, FTr) of workload w on the same
    velocity U: absolute As error over the cut cells (mean and quantiles) and the per-solid force error, normwise
    against rho_f / dt * volume * (|U| rms + |v| + |omega| r_B), the magnitude of the sum of the cell contributions
    (median, 90th percentile, max)."""
    touched = fr["Ct"] != 0
    cut = touched & ~((fr["As"] == 1.0) & (f["As"] == 1.0))
    err = (f["As"] - fr["As"]).abs()[cut].double()
    q = torch.quantile(err[: 1 << 24], torch.tensor([0.5, 0.99, 0.999], dtype=torch.float64, device=err.device))
    u_rms = float(U.square().mean().sqrt())
    rel = []
    for s, d in enumerate(w.solids):
        v = np.linalg.norm(np.array(d.vel[:])) + np.linalg.norm(np.array(d.omega[:])) * d.shape.radiusB
        scale = w.opt.rho_f / w.dt * d.shape.volume * (u_rms + v)
        rel.append(np.linalg.norm(FT[s, :3] - FTr[s, :3]) / scale)
    rel = np.array(rel)
    return {"reference": reference, "cut_cells": int(cut.sum()),
            "as_abs_err_mean": float(err.mean()), "as_abs_err_p50": float(q[0]), "as_abs_err_p99": float(q[1]),
            "as_abs_err_p999": float(q[2]), "as_abs_err_max": float(err.max()),
            "force_rel_err_median": float(np.median(rel)), "force_rel_err_p90": float(np.percentile(rel, 90)),
            "force_rel_err_max": float(rel.max())}
