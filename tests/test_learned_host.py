"""Host-side parts of the learned cut-cell fraction, on CPU: the confidence-band scores (the formulas of the device's
in_band), the band calibration of the trainer, and the shipped model file."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

# the 8 vertices of a unit cell in cellPoints order (x fastest, then y, then z)
CORNERS = np.array([[i, j, k] for k in (0, 1) for j in (0, 1) for i in (0, 1)], dtype=np.float64)


def _features(phi):
    f = torch.zeros((11, phi.shape[1]), dtype=torch.float32)
    f[:8] = torch.from_numpy(phi.astype(np.float32))
    return f


def test_band_scores_of_planes_and_spheres():
    from sdfibm_gb300.train_fraction import band_scores
    rng = np.random.default_rng(0)
    n = rng.normal(size=(3, 500))
    n /= np.linalg.norm(n, axis=0)
    d = rng.uniform(-0.8, 0.8, 500)
    phi = CORNERS @ n + d                                    # a plane's signed distance, in cell sizes
    tw, gd = band_scores(torch, _features(phi))
    assert tw.abs().max().item() < 1e-5 and gd.max().item() < 1e-5   # no twist, unit gradient
    # spheres through the cell centre, seen along a diagonal: twisted, more so the smaller the radius
    u = np.ones(3) / np.sqrt(3.0)
    tws = []
    for r in (1.5, 3.0, 12.0):
        centre = np.array([0.5, 0.5, 0.5]) - r * u
        phi = np.linalg.norm(CORNERS - centre, axis=1)[:, None] - r
        tws.append(band_scores(torch, _features(phi))[0].item())
    assert tws[0] > tws[1] > tws[2] > 0


def test_band_scores_match_the_oracle():
    """The trainer's scores and the oracle's restatement of the device's in_band give the same FP32 values."""
    from oracle import mlp_oracle
    from sdfibm_gb300.train_fraction import band_scores
    feat = np.random.default_rng(2).normal(size=(11, 4096)).astype(np.float32)
    tw, gd = band_scores(torch, torch.from_numpy(feat))
    tw_o, gd_o = mlp_oracle.band_scores(feat.T)
    assert np.allclose(tw.numpy(), tw_o, rtol=1e-6, atol=1e-6) and np.allclose(gd.numpy(), gd_o, rtol=1e-6, atol=1e-6)


def test_calibration_keeps_the_error_limits():
    from sdfibm_gb300.train_fraction import calibrate
    g = torch.Generator().manual_seed(1)
    n = 200000
    tw = torch.rand(n, generator=g)
    gd = torch.rand(n, generator=g) * 0.1
    # the error grows with the twist: cells above 0.5 are far off
    err = torch.where(tw < 0.5, 2e-4 * torch.rand(n, generator=g), 5e-2 * torch.ones(n))
    frac, a, b, m, p = calibrate(torch, err, tw, gd, 1e-3, 1e-2)
    acc = (tw <= a) & (gd <= b)
    assert 0.3 < frac <= 0.5 + 1e-3 and abs(acc.float().mean().item() - frac) < 1e-6
    assert err[acc].mean().item() <= 1e-3 and m <= 1e-3 and p <= 1e-2
    # limits that nothing meets leave the band empty
    assert calibrate(torch, err, tw, gd, 1e-9, 1e-9)[0] == 0.0


def test_shipped_model_file():
    from sdfibm_gb300 import abi, learned
    params, tau_twist, tau_grad, meta = learned.load_model()
    assert params.dtype == np.float32 and params.shape == (abi.MLP_NPARAM,) and np.isfinite(params).all()
    assert tau_twist > 0 and tau_grad > 0 and "band" in meta


def test_model_file_round_trip(tmp_path):
    from sdfibm_gb300 import learned
    p = learned.init_params(3)
    learned.save_model(p, 0.25, 0.05, {"note": "test"}, path=str(tmp_path / "m.npz"))
    q, a, b, meta = learned.load_model(str(tmp_path / "m.npz"))
    assert np.array_equal(p, q) and a == np.float32(0.25) and b == np.float32(0.05) and meta == {"note": "test"}
