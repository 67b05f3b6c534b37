"""SolidCloud::calcMeanField / writeMeanField: the mean of U around every solid over the cells a sampler shape in the
solid's pose touches, weighted by the REF-GEO fraction.

The library computes it with the coupling itself: the sampler-shaped solids at rest, with rho_f = 1 and dt = 1,
receive the force sum(alpha V U), and a pass on U = 1 gives sum(alpha V).  The CPU tests show on the oracle that this
identity reproduces the oracle's direct restatement of calcMeanField (same cells, same Ct writes); the GPU test runs
it through libsdfibm_cuda.so against that restatement."""
import numpy as np
import pytest

from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi
from sdfibm_gb300 import workloads as W
from sdfibm_gb300.host import StateFile, format_mean_field, make_shape


def _case(name):
    if name == "poly3d":
        w = W.poly3d_256(scale=0.25)
        sampler = make_shape("Sphere", radius=0.03)
    else:
        w = W.sedimentation2d(scale=0.5)
        sampler = make_shape("Circle", radius=0.06)
    # a mean flow plus noise, so that the means are O(1)
    rng = np.random.default_rng(5)
    U = (rng.standard_normal((3, w.ncells)) * 0.05).astype(np.float32)
    U += np.array([1.0, -0.5, 0.25], np.float32)[:, None]
    return w, sampler, U


def _sampler_solids(w, sampler):
    out = []
    for d in w.solids:
        e = abi.SolidDesc.from_buffer_copy(d)
        e.shape = sampler
        for a in range(3):
            e.vel[a] = 0.0
            e.omega[a] = 0.0
        out.append(e)
    return out


@pytest.mark.parametrize("name", ["poly3d", "sedimentation2d"])
def test_forcing_identity_on_the_oracle(name):
    w, sampler, U = _case(name)
    Uo = U.astype(np.float64).reshape(-1)
    oc = OracleCloud(w.mesh, w.solids, w.opt, faithful=True)
    Ct = np.zeros(oc.N, np.int32)
    direct = oc.mean_field(sampler, Uo, Ct)
    sc = OracleCloud(w.mesh, _sampler_solids(w, sampler), abi.options(rho_f=1.0), faithful=False)
    f = sc.new_fields()
    F = sc.interact(0.0, 1.0, Uo, f)
    Wt = sc.interact(0.0, 1.0, np.ones_like(Uo), f)
    assert np.abs(F[:, :3] / Wt[:, :1] - direct).max() < 1e-13
    # the same cells, and the Ct the reference leaves behind
    assert np.array_equal(f["Ct"], Ct) and (Ct != 0).sum() > 100


def test_uniform_field_and_volume():
    w, sampler, _ = _case("poly3d")
    oc = OracleCloud(w.mesh, w.solids, w.opt, faithful=False)
    U = np.repeat(np.array([0.3, -0.7, 1.1])[:, None], oc.N, axis=1).reshape(-1)
    m = oc.mean_field(sampler, U)
    assert np.allclose(m, [0.3, -0.7, 1.1], rtol=1e-14, atol=0)
    # sum(alpha V) of a sampler of radius 6.4 cells away from the walls: the sphere's volume, less the REF-GEO
    # fraction's first-order deficit on cut cells (about 1.5 % at this radius, 15 % at 2 cells)
    big = make_shape("Sphere", radius=0.1)
    sc = OracleCloud(w.mesh, _sampler_solids(w, big), abi.options(rho_f=1.0), faithful=False)
    f = sc.new_fields()
    vol = sc.interact(0.0, 1.0, np.ones(3 * oc.N), f)[:, 0]
    inner = [i for i, d in enumerate(w.solids) if all(0.1 < d.pos[a] < 0.9 for a in range(3))]
    assert len(inner) > 10
    ratio = vol[inner] / (4.0 / 3.0 * np.pi * 0.1 ** 3)
    assert ratio.min() > 0.97 and ratio.max() < 1.0


def test_mean_field_file(cuda_lib, tmp_path):
    m = np.array([[1.0, -2.5e-3, 3.0], [0.0, 1e10, -1e-10]])
    assert format_mean_field(m) == " ".join("%.6e" % v for v in m.reshape(-1)) + " \n"
    sf = StateFile(str(tmp_path / "cloud.out"), write_frequency=2, mean_field_path=str(tmp_path / "meanfield.out"))
    assert sf.keeps_mean_field
    st = [abi.SolidState(), abi.SolidState()]
    for s in st:
        s.quat[0] = 1.0
    for k in range(3):
        sf.save(0.1 * k, st, m * (k + 1))
    sf.close()
    # cloud.out on calls 0 and 2, the mean field on every call
    assert len(open(tmp_path / "cloud.out").read().splitlines()) == 4
    lines = open(tmp_path / "meanfield.out").read().splitlines()
    assert len(lines) == 3 and lines[2] == format_mean_field(3 * m)[:-1]


class _OracleSamplerContext:
    """Stands in for the sampler-shaped SolidCloud on CPU: the same calls, answered by the oracle."""

    def __init__(self, w, sampler):
        self.oc = OracleCloud(w.mesh, _sampler_solids(w, sampler), abi.options(rho_f=1.0), faithful=False)

    def set_states(self, st):
        self.oc.set_state((abi.SolidState * len(st))(*st))

    def new_fields(self, device="cpu"):
        import torch
        N = self.oc.N
        return dict(As=torch.zeros(N, dtype=torch.float64), Fs=torch.zeros(3 * N, dtype=torch.float64),
                    Ts=torch.zeros(N, dtype=torch.float64), Ct=torch.zeros(N, dtype=torch.int32))

    def interact(self, time, dt, U, fields):
        fo = {k: v.numpy() for k, v in fields.items()}
        return self.oc.interact(time, dt, U.numpy().astype(np.float64).reshape(-1), fo)

    def close(self):
        pass


def test_mean_field_host_logic():
    """SolidCloud.mean_field's host logic (states at rest, the two passes, the Ct merge) on CPU tensors, the sampler
    context answered by the oracle; the moving solids' velocities must not reach the forcing."""
    torch = pytest.importorskip("torch")
    from sdfibm_gb300.cloud import SolidCloud
    w, sampler, U = _case("poly3d")
    main = OracleCloud(w.mesh, w.solids, w.opt, faithful=False)
    fo = main.new_fields()
    Uo = U.astype(np.float64).reshape(-1)
    main.interact(0.0, w.dt, Uo, fo)
    assert max(abs(s.vel[0]) for s in main.get_state()) > 0
    cloud = SolidCloud.__new__(SolidCloud)
    cloud.time = 0.0
    cloud._sampler = (sampler, _OracleSamplerContext(w, sampler))
    cloud._sampler_fields = None
    cloud.states = lambda: list(main.get_state())
    Ct = torch.from_numpy(fo["Ct"].copy())
    m = cloud.mean_field(torch.from_numpy(U), Ct)
    ref = main.mean_field(sampler, Uo, fo["Ct"])
    assert np.abs(m - ref).max() < 1e-13
    assert np.array_equal(Ct.numpy(), fo["Ct"])
    # before the next interact the sampler's cells return to 0, as the reference's dense reset leaves them
    sampled = cloud._sampler_ct[1].numpy().copy()
    assert sampled.sum() > 100
    other = Ct.clone()
    cloud._clear_sampler_ct(other.clone())      # another field: untouched, and the mark is consumed
    assert cloud._sampler_ct is None
    cloud._sampler_ct = (Ct, torch.from_numpy(sampled))
    cloud._clear_sampler_ct(Ct)
    assert (Ct.numpy()[sampled] == 0).all() and np.array_equal(Ct.numpy()[~sampled], other.numpy()[~sampled])


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["poly3d", "sedimentation2d"])
def test_mean_field_gpu(cuda_lib, torch_cuda, name):
    torch = torch_cuda
    from sdfibm_gb300.cloud import SolidCloud
    w, sampler, U = _case(name)
    gpu = SolidCloud(w.mesh, w.solids, w.opt)
    Ud = torch.from_numpy(U).cuda()
    f = gpu.new_fields()
    gpu.interact(0.0, w.dt, Ud, f)
    gpu.set_sampler(sampler)
    m = gpu.mean_field(Ud, f["Ct"])
    Ctg = f["Ct"].cpu().numpy()
    gpu.close()

    oc = OracleCloud(w.mesh, w.solids, w.opt, faithful=False)
    fo = oc.new_fields()
    Uo = U.astype(np.float64).reshape(-1)
    oc.interact(0.0, w.dt, Uo, fo)
    ref = oc.mean_field(sampler, Uo, fo["Ct"])
    # the fractions of the cut cells agree within 1e-5 relative, so the weighted means within 1e-5 normwise
    err = np.linalg.norm(m - ref, axis=1) / np.linalg.norm(ref, axis=1)
    assert err.max() < 1e-5, err.max()
    assert np.array_equal(Ctg, fo["Ct"])
