"""Learned cut-cell fraction on the GPU (tcgen05 kernels of mlp.cu through include/sdfibm_mlp.h) against the CPU
oracle of the model (oracle/mlp_oracle.py) and of the training cells (oracle_sample_cell)."""
import numpy as np
import pytest

from oracle import mlp_oracle as MO
from oracle import oracle as O
from sdfibm_gb300 import abi, learned

pytestmark = pytest.mark.gpu

FWD_ABS = 2e-5      # predicted fraction, GPU vs oracle (same roundings; FP32 accumulation order, fast exp)
GRAD_REL = 2e-2     # normwise per parameter block (BF16 roundings of dZ can flip by one unit in the last place)


def _params(seed, bias=0.1):
    p = learned.init_params(seed)
    rng = np.random.default_rng(seed + 100)
    p[MO.OFF_B1:MO.OFF_W2] = rng.normal(0, bias, 64)
    p[MO.OFF_B2:MO.OFF_W3] = rng.normal(0, bias, 64)
    p[MO.OFF_B3] = 0.3
    return p


def test_dataset_matches_oracle(cuda_lib, torch_cuda):
    """Generated cells against the oracle: labels exactly (FP64 inside tests on both sides), inputs and prior within
    the FP32 rounding of the device's stencil (distances from FP32 local coordinates, FP32 sub-cell planes)."""
    torch = torch_cuda
    n = 2048  # 64 warps: every family drawn (the family is chosen per warp)
    feat, label, rec = learned.make_dataset(torch, n, seed=7, recipe=True, n_sub=8)
    feat, label, rec = feat.cpu().numpy(), label.cpu().numpy(), rec.cpu().numpy()
    assert feat.shape == (abi.MLP_NFEAT, n)
    types = set()
    phis = []
    for i in range(n):
        phi, cnt = O.sample_cell(rec[i], 8)
        assert 0 < rec[i, 17] < 8, "cell %d is not cut" % i
        assert label[i] == np.float32(cnt / 512.0), "label of cell %d: %r vs %r" % (i, label[i], cnt / 512.0)
        phis.append(phi)
        types.add(int(rec[i, 0]))
    ref = MO.features(np.array(phis))
    # distance inputs: FP32 local coordinates of points up to ~20 cells from the origin (the inputs need 1e-4: BF16
    # hi + lo pairs keep about 16 bits)
    d = np.abs(feat[:15].T - ref[:, :15]) / (1 + np.abs(ref[:, :15]))
    assert d.max() <= 1e-4, "distance inputs: max scaled difference %g" % d.max()
    # P2 and P4 through their logits: compare the fractions.  A sub-cell's fraction moves by the distances' FP32
    # rounding over the sub-cell's width (h/2 for P2) and by the fast reciprocals of the closed form: about 2e-5
    sig = lambda z: 1.0 / (1.0 + np.exp(-z.astype(np.float64)))
    assert np.abs(sig(feat[15]) - sig(ref[:, 15])).max() <= 5e-5
    assert np.abs(sig(feat[16]) - sig(ref[:, 16])).max() <= 5e-5
    assert types == {abi.SHAPE_SPHERE, abi.SHAPE_ELLIPSOID, abi.SHAPE_BOX, abi.SHAPE_PLANE, abi.SHAPE_CIRCLE,
                     abi.SHAPE_ELLIPSE}
    # the prior is a good estimate already: planes are exact up to the 8^3 label's own lattice error
    plane = rec[:, 0] == abi.SHAPE_PLANE
    assert np.abs(sig(feat[16][plane]) - label[plane]).mean() < 5e-3


def test_forward_matches_oracle(cuda_lib, torch_cuda):
    torch = torch_cuda
    n = 1000  # 8 tiles, the last one partial
    feat, _, _ = learned.make_dataset(torch, n, seed=11)
    p = _params(3)
    out = learned.forward(torch, torch.from_numpy(p).cuda(), feat).cpu().numpy()
    X = feat.cpu().numpy().T
    ref = MO.forward(p, X)
    err = np.abs(out - ref)
    assert err.max() <= FWD_ABS, "max |GPU - oracle| = %g at cell %d" % (err.max(), int(err.argmax()))
    # the hi/lo split matters: single-BF16 inputs are several times further off
    Xb = X.copy()
    Xb[:, :MO.N_IN] = MO.bf16(X[:, :MO.N_IN])
    lo = MO.forward(p, Xb)
    assert np.abs(lo - ref).max() > 3 * err.max()


def test_forward_strided_features(cuda_lib, torch_cuda):
    torch = torch_cuda
    feat, _, _ = learned.make_dataset(torch, 4096, seed=12)
    p = torch.from_numpy(_params(4)).cuda()
    full = learned.forward(torch, p, feat)
    part = learned.forward(torch, p, feat[:, 100:1300])  # stride 4096, 1200 cells
    assert torch.equal(full[100:1300], part)


def test_loss_grad_matches_oracle(cuda_lib, torch_cuda):
    torch = torch_cuda
    n = 1000
    feat, label, _ = learned.make_dataset(torch, n, seed=13)
    p = _params(5)
    loss, g = learned.loss_grad(torch, torch.from_numpy(p).cuda(), feat, label)
    lref, gref = MO.loss_grad(p, feat.cpu().numpy().T, label.cpu().numpy().astype(np.float64))
    assert abs(loss - lref) <= 1e-5 * (1 + lref)
    blocks = {"W1": (MO.OFF_W1, MO.OFF_B1), "b1": (MO.OFF_B1, MO.OFF_W2), "W2": (MO.OFF_W2, MO.OFF_B2),
              "b2": (MO.OFF_B2, MO.OFF_W3), "w3": (MO.OFF_W3, MO.OFF_B3), "b3": (MO.OFF_B3, MO.N_PARAM)}
    for name, (a, b) in blocks.items():
        rel = np.linalg.norm(g[a:b] - gref[a:b]) / (np.linalg.norm(gref[a:b]) + 1e-30)
        assert rel <= GRAD_REL, "%s gradient: relative error %g" % (name, rel)


def test_gradient_of_many_tiles_per_cta(cuda_lib, torch_cuda):
    """More tiles than SMs: each CTA accumulates several tiles in tensor memory before its single flush."""
    torch = torch_cuda
    n = 128 * 700
    feat, label, _ = learned.make_dataset(torch, n, seed=14, n_sub=4)
    p = _params(6)
    loss, g = learned.loss_grad(torch, torch.from_numpy(p).cuda(), feat, label)
    lref, gref = MO.loss_grad(p, feat.cpu().numpy().T, label.cpu().numpy().astype(np.float64))
    assert abs(loss - lref) <= 1e-4 * (1 + lref)
    assert np.linalg.norm(g - gref) / np.linalg.norm(gref) <= GRAD_REL


def test_adam_step_matches_oracle(cuda_lib, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(2)
    p = _params(7)
    g = rng.normal(0, 1e-2, MO.N_PARAM + 1).astype(np.float32)
    m = rng.normal(0, 1e-3, MO.N_PARAM).astype(np.float32)
    v = np.abs(rng.normal(0, 1e-4, MO.N_PARAM)).astype(np.float32)
    pd, gd, md, vd = (torch.from_numpy(x.copy()).cuda() for x in (p, g, m, v))
    learned.adam(torch, pd, gd, md, vd, 3, 1e-3)
    pr, mr, vr = MO.adam_step(p, g[:-1], m, v, 3, 1e-3)
    np.testing.assert_allclose(pd.cpu().numpy(), pr, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(md.cpu().numpy(), mr, rtol=1e-6, atol=1e-9)


def test_training_lowers_the_error(cuda_lib, torch_cuda):
    torch = torch_cuda
    feat, label, _ = learned.make_dataset(torch, 1 << 18, seed=21)
    tf, tl, _ = learned.make_dataset(torch, 1 << 15, seed=22)
    p = torch.from_numpy(learned.init_params(1)).cuda()
    before = (learned.forward(torch, p, tf) - tl).abs().mean().item()
    p0 = p.clone()
    p0[-65:] = 0.0  # network output zero: the prior alone (4^3 sub-cell planar reconstruction)
    prior_only = (learned.forward(torch, p0, tf) - tl).abs().mean().item()
    losses = learned.train(torch, p, feat, label, epochs=10, batch=4096, lr=2e-3, warmup_steps=50)
    after = (learned.forward(torch, p, tf) - tl).abs().mean().item()
    assert np.all(np.isfinite(losses)) and losses[-1] < losses[0]
    # what the trained network gains over the model without it (the sub-cell planar prior)
    assert after < 0.7 * prior_only and after < before, (before, prior_only, after, losses)
