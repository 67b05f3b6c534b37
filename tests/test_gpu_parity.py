"""GPU coupling (libsdfibm_cuda.so through its C ABI) against the FP64 oracle on the same seeded inputs."""
import math

import numpy as np
import pytest

from gpu_helpers import check_interact, run_pair
from sdfibm_gb300 import abi, workloads
from sdfibm_gb300.host import make_shape, make_solid, mask_motion
from sdfibm_gb300.workloads import Workload, random_quaternions

pytestmark = pytest.mark.gpu


def test_cylinder2d(cuda_lib, torch_cuda):
    w = workloads.cylinder2d()
    r = run_pair(torch_cuda, w)
    s = check_interact(w, r)
    assert s["coupling_cells"] == 94


@pytest.mark.parametrize("method", [abi.FRACTION_REFGEO, abi.FRACTION_SUBSAMPLE])
def test_sedimentation2d_scaled(cuda_lib, torch_cuda, method):
    w = workloads.sedimentation2d(scale=0.25)
    w.opt.fraction_method = method
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


@pytest.mark.parametrize("method", [abi.FRACTION_REFGEO, abi.FRACTION_SUBSAMPLE])
def test_poly3d_256_scaled(cuda_lib, torch_cuda, method):
    w = workloads.poly3d_256(scale=0.25)
    w.opt.fraction_method = method
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


def test_poly3d_512_scaled(cuda_lib, torch_cuda):
    w = workloads.poly3d_512(scale=0.125)
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


def _zoo(twod, seed):
    """Every registered shape, random pose and com, some solids crossing the mesh boundary, tiny and thin ones."""
    rng = np.random.default_rng(seed)
    n = 48
    if twod:
        mesh = abi.mesh_desc((n, n, 1), (-1.0, -1.0, -0.5), (2.0 / n, 2.0 / n, 1.0), twod=1)
    else:
        mesh = abi.mesh_desc((n, n, n), (-1.0, -1.0, -1.0), (2.0 / n,) * 3, twod=0)
    h = 2.0 / n
    shapes = [("Circle", dict(radius=0.3)), ("Ellipse", dict(radiusa=0.35, radiusb=0.12)),
              ("Rectangle", dict(radiusa=0.3, radiusb=0.1)), ("Circle_Tail", dict(radius=0.15, ratio=2.0, thickness=0.06)),
              ("Circle_TwoTail", dict(radius=0.15, ratio=2.0, thickness=0.08)), ("Circle", dict(radius=0.3 * h)),
              ("Rectangle", dict(radiusa=0.5, radiusb=0.2 * h))]
    if not twod:
        shapes += [("Sphere", dict(radius=0.3)), ("Ellipsoid", dict(radiusa=0.1, radiusb=0.25, radiusc=0.4)),
                   ("Box", dict(radiusa=0.1, radiusb=0.2, radiusc=0.3)), ("Sphere", dict(radius=0.4 * h)),
                   ("Box", dict(radiusa=0.45, radiusb=0.15 * h, radiusc=0.15 * h))]
    solids = []
    for i, (t, kw) in enumerate(shapes):
        com = (0.0, 0.0, 0.0) if i % 3 == 0 else tuple(rng.uniform(-0.05, 0.05, 3) * (1, 1, 0 if twod else 1))
        sh = make_shape(t, com=com, **kw)
        pos = rng.uniform(-1.1, 1.1, 3)
        if twod:
            pos[2] = 0.0
        d = make_solid(i, sh, 1.2, pos, vel=rng.normal(0, 0.1, 3), omega=rng.normal(0, 1.0, 3) * ((0, 0, 1) if twod else 1))
        if twod:
            th = rng.uniform(0, 2 * math.pi)
            q = (math.cos(th / 2), 0.0, 0.0, math.sin(th / 2))
        else:
            q = random_quaternions(rng, 1)[0]
        for c in range(4):
            d.quat[c] = float(q[c])
        solids.append(d)
    # a plane cutting the mesh obliquely
    pl = make_solid(len(solids), make_shape("Plane"), 1.0, (0.2, -0.5, 0.0), (0, 0, 25.0),
                    motion=mask_motion("b000000"))
    solids.append(pl)
    opt = abi.options(rho_f=1.3)
    return Workload("zoo%d" % (2 if twod else 3), mesh, solids, opt, 0.01, (0.2, -0.1, 0.05), 0.1, seed)


@pytest.mark.parametrize("twod", [True, False])
@pytest.mark.parametrize("method", [abi.FRACTION_REFGEO, abi.FRACTION_SUBSAMPLE])
def test_shape_zoo(cuda_lib, torch_cuda, twod, method):
    w = _zoo(twod, 11 if twod else 12)
    w.opt.fraction_method = method
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


@pytest.mark.parametrize("method", [abi.FRACTION_REFGEO, abi.FRACTION_SUBSAMPLE])
def test_filter_threshold_vertices(cuda_lib, torch_cuda, method):
    """Surfaces 1e-8 away from mesh vertices: the vertex distances sit at the reference's filter threshold
    (|phi| < 1e-8 -> -1e-8, sdf.h:147-150), where the FP32 and two-float paths hand over to the FP64 sequence."""
    n = 32
    h = 1.0 / n
    mesh = abi.mesh_desc((n, n, n), (0.0, 0.0, 0.0), (h,) * 3, twod=0)
    solids = []
    for i, (t, kw, pos) in enumerate([
            ("Sphere", dict(radius=6 * h + 1e-8), (8 * h, 8 * h, 8 * h)),
            ("Sphere", dict(radius=5 * h - 1e-8), (24 * h, 8 * h, 8 * h)),
            ("Box", dict(radiusa=4 * h + 1e-8, radiusb=3 * h - 1e-8, radiusc=5 * h), (8 * h, 24 * h, 8 * h)),
            ("Ellipsoid", dict(radiusa=4 * h + 1e-8, radiusb=6 * h, radiusc=5 * h - 1e-8), (24 * h, 24 * h, 8 * h)),
            ("Sphere", dict(radius=7 * h), (16 * h, 16 * h, 23 * h))]):
        solids.append(make_solid(i, make_shape(t, **kw), 1.2, pos, vel=(0.1, 0.0, 0.0), omega=(0.0, 0.0, 0.5)))
    opt = abi.options(rho_f=1.0, fraction_method=method)
    w = Workload("threshold", mesh, solids, opt, 0.01, (0.1, 0.0, 0.0), 0.1, 3)
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


@pytest.mark.parametrize("cfg", ["poly3d_256", "sedimentation2d", "zoo3", "zoo2"])
def test_mixed_precision_forcing(cuda_lib, torch_cuda, cfg):
    """exact_forcing = 0: FP64 only for the rigid-body velocity and U - us, FP32 after; same contract."""
    if cfg == "poly3d_256":
        w = workloads.poly3d_256(scale=0.25)
    elif cfg == "sedimentation2d":
        w = workloads.sedimentation2d(scale=0.25)
    else:
        w = _zoo(cfg == "zoo2", 13)
    w.opt.exact_forcing = 0
    w.opt.fraction_method = abi.FRACTION_SUBSAMPLE
    r = run_pair(torch_cuda, w)
    check_interact(w, r)


def test_sparse_reset_and_repeat(cuda_lib, torch_cuda):
    """Three interacts with motion in between: the sparse reset leaves exactly the fields a dense reset gives."""
    w = workloads.sedimentation2d(scale=0.125, ncircles=12)
    r = run_pair(torch_cuda, w, steps=3, evolve=True)
    check_interact(w, r)


def _cluster(exact, twod):
    """Solids overlapping in a cluster (cells touched by two to four solids), some crossing the high corner of a mesh
    whose cell count is not a multiple of 8, moving about two cells per step."""
    rng = np.random.default_rng(21 if twod else 22)
    if twod:
        n = (45, 37, 1)
        mesh = abi.mesh_desc(n, (0.0, 0.0, -0.5), (1.0 / 45, 1.0 / 45, 1.0), twod=1)
        kinds = [("Circle", dict(radius=0.09)), ("Ellipse", dict(radiusa=0.12, radiusb=0.05)),
                 ("Rectangle", dict(radiusa=0.1, radiusb=0.04))]
    else:
        n = (37, 29, 23)
        mesh = abi.mesh_desc(n, (0.0, 0.0, 0.0), (1.0 / 37,) * 3, twod=0)
        kinds = [("Sphere", dict(radius=0.09)), ("Ellipsoid", dict(radiusa=0.12, radiusb=0.05, radiusc=0.07)),
                 ("Box", dict(radiusa=0.1, radiusb=0.04, radiusc=0.06))]
    hi = np.array([n[0] / 37 if not twod else 1.0, n[1] / (37 if not twod else 45), n[2] / 37 if not twod else 0.0])
    centre = 0.45 * hi
    solids = []
    for i in range(10):
        t, kw = kinds[i % 3]
        if i < 7:
            pos = centre + rng.uniform(-0.08, 0.08, 3)
        else:  # at the high corner: the last chunk of the mesh is partly outside it
            pos = hi - rng.uniform(0.0, 0.05, 3)
        if twod:
            pos[2] = 0.0
        vel = rng.normal(0, 3.0, 3) * ((1, 1, 0) if twod else 1)
        om = rng.normal(0, 5.0, 3) * ((0, 0, 1) if twod else 1)
        solids.append(make_solid(i, make_shape(t, **kw), 1.1, pos, vel=vel, omega=om))
    opt = abi.options(rho_f=1.2, fraction_method=abi.FRACTION_SUBSAMPLE, exact_forcing=exact)
    return Workload("cluster", mesh, solids, opt, 0.01, (0.3, -0.2, 0.1), 0.2, 5)


@pytest.mark.parametrize("twod", [False, True])
@pytest.mark.parametrize("exact", [1, 0])
def test_clustered_solids_shared_cells(cuda_lib, torch_cuda, twod, exact):
    """Cells shared by several solids (their FP64 sums through the shared table), chunks of 8 cells split between
    solids and untouched cells, the partial last chunk of the mesh, and cells left behind by fast motion (the sparse
    reset outside the chunks written this call), over three coupled steps."""
    w = _cluster(exact, twod)
    assert w.ncells % 8 != 0
    r = run_pair(torch_cuda, w, steps=3, evolve=True, sync_states=not exact)
    check_interact(w, r)
    touched = np.concatenate([r["orc"].touched(s)[0] for s in range(len(w.solids))])
    _, cnt = np.unique(touched, return_counts=True)
    assert (cnt > 1).sum() > 20 and cnt.max() >= 3
    assert (touched == w.ncells - 1).any() or (touched >= w.ncells - 8).any()


def test_fix_internal(cuda_lib, torch_cuda):
    w = workloads.cylinder2d(scale=0.5)
    w.solids[0].vel[0] = 0.3
    w.solids[0].omega[2] = 0.7
    r = run_pair(torch_cuda, w, steps=2, evolve=True, fix=True)
    Ug = r["Ud"].cpu().numpy().astype(np.float64).reshape(-1)
    assert np.abs(Ug - r["Uo"]).max() <= 1e-6 * np.abs(r["Uo"]).max()


@pytest.mark.parametrize("cfg", ["poly3d_512", "sedimentation2d"])
def test_apply_forcing(cuda_lib, torch_cuda, cfg):
    """The solver's forcing update on device fields after each of three moving steps: U -= Fs dt and
    T = (1 - As) T + Ts equal the dense FP64 update of every cell, rounded once to FP32; other fields are refused."""
    from sdfibm_gb300.cloud import SolidCloud
    torch = torch_cuda
    w = workloads.poly3d_512(scale=0.0625) if cfg == "poly3d_512" else workloads.sedimentation2d(scale=0.125)
    N = w.ncells
    c = SolidCloud(w.mesh, w.solids, w.opt)
    f = c.new_fields()
    U = torch.from_numpy(w.U_numpy()).cuda()
    T = torch.from_numpy(np.random.default_rng(4).uniform(0.0, 2.0, N).astype(np.float32)).cuda()
    t = 0.0
    for step in range(3):
        c.interact(t, w.dt, U, f)
        U0, T0 = U.cpu().numpy().astype(np.float64), T.cpu().numpy().astype(np.float64)
        As, Fs, Ts = (f[k].cpu().numpy().astype(np.float64) for k in ("As", "Fs", "Ts"))
        c.apply_forcing(w.dt, f, U, T if step != 1 else None)
        Ue = (U0.reshape(-1) - Fs.reshape(-1) * w.dt).astype(np.float32)
        assert np.array_equal(U.cpu().numpy().reshape(-1), Ue), step
        Te = ((1.0 - As) * T0 + Ts).astype(np.float32) if step != 1 else T0.astype(np.float32)
        assert np.array_equal(T.cpu().numpy(), Te), step
        assert (As > 0).sum() > 0
        c.evolve(t, w.dt)
        t += w.dt
    g = c.new_fields()
    with pytest.raises(RuntimeError):
        c.apply_forcing(w.dt, g, U, T)
    c.close()


def test_interact_host_matches_device(cuda_lib, torch_cuda):
    from sdfibm_gb300.cloud import SolidCloud
    w = workloads.poly3d_512(scale=0.0625)
    U = w.U_numpy()
    a = SolidCloud(w.mesh, w.solids, w.opt)
    b = SolidCloud(w.mesh, w.solids, w.opt)
    fd = a.new_fields()
    FTa = a.interact(0.0, w.dt, torch_cuda.from_numpy(U).cuda(), fd)
    N = w.ncells
    fh = dict(As=np.zeros(N, np.float32), Fs=np.zeros(3 * N, np.float32), Ts=np.zeros(N, np.float32),
              Ct=np.zeros(N, np.int32))
    FTb = b.interact_host(0.0, w.dt, U, fh)
    assert np.array_equal(fd["As"].cpu().numpy(), fh["As"])
    assert np.array_equal(fd["Ct"].cpu().numpy(), fh["Ct"])
    assert np.allclose(FTa, FTb, rtol=1e-12, atol=1e-14)
    assert b.stats()["host_sparse"] == 0


@pytest.mark.parametrize("cfg", ["poly3d_512", "sedimentation2d"])
def test_interact_host_pinned_in_place(cuda_lib, torch_cuda, cfg):
    """Page-locked host fields over several moving steps: only the changed cells are written back; the host fields
    equal the device path's after every step, and a buffer change falls back to a whole copy."""
    from sdfibm_gb300.cloud import SolidCloud
    torch = torch_cuda
    w = workloads.poly3d_512(scale=0.0625) if cfg == "poly3d_512" else workloads.sedimentation2d(scale=0.125)
    N = w.ncells
    U = torch.from_numpy(w.U_numpy()).pin_memory()
    a = SolidCloud(w.mesh, w.solids, w.opt)
    b = SolidCloud(w.mesh, w.solids, w.opt)
    fd = a.new_fields()
    Ud = U.cuda()

    def pinned():
        return {"As": torch.full((N,), 7.0).pin_memory(), "Fs": torch.full((3 * N,), 7.0).pin_memory(),
                "Ts": torch.full((N,), 7.0).pin_memory(), "Ct": torch.full((N,), 7, dtype=torch.int32).pin_memory()}

    fh = pinned()
    hn = {k: v.numpy() for k, v in fh.items()}
    t = 0.0
    for step in range(4):
        if step == 3:  # other host buffers: one whole copy
            fh = pinned()
            hn = {k: v.numpy() for k, v in fh.items()}
        FTa = a.interact(t, w.dt, Ud, fd)
        FTb = b.interact_host(t, w.dt, U.numpy(), hn)
        for k in ("As", "Fs", "Ts", "Ct"):
            assert np.array_equal(fd[k].cpu().numpy().reshape(-1), hn[k]), (step, k)
        assert np.allclose(FTa, FTb, rtol=1e-12, atol=1e-14)
        st = b.stats()
        assert st["host_sparse"] == (1 if step in (1, 2) else 0), step
        if st["host_sparse"]:
            assert 0 < st["host_d2h_bytes"] < 24 * N
            # a page-locked U is read in place at the coupling cells (REF-GEO, or when copying it in whole outlasts
            # the fraction kernels) or copied in whole
            in_place = 12 * st["coupling_cells"]
            assert st["host_h2d_bytes"] == in_place or (w.opt.fraction_method != abi.FRACTION_REFGEO and
                                                         st["host_h2d_bytes"] == 12 * N)
        a.evolve(t, w.dt)
        b.evolve(t, w.dt)
        t += w.dt


@pytest.mark.parametrize("pinned", [True, False])
def test_interact_host64_matches_device(cuda_lib, torch_cuda, pinned):
    """FP64 host fields in OpenFOAM's layout (U and Fs one x,y,z triple per cell, Ct as doubles), page-locked (read
    and written in place) or pageable (staged): every step equals the device-field path on the same U, and a change
    of buffers writes every cell again."""
    from sdfibm_gb300.cloud import SolidCloud
    torch = torch_cuda
    w = workloads.poly3d_512(scale=0.0625)
    N = w.ncells
    U32 = w.U_numpy()                                    # [3][N] FP32
    U64 = np.ascontiguousarray(U32.T.astype(np.float64))  # [N][3]: the FP32 values, exactly
    a = SolidCloud(w.mesh, w.solids, w.opt)
    b = SolidCloud(w.mesh, w.solids, w.opt)
    fd = a.new_fields()
    Ud = torch.from_numpy(U32).cuda()

    def host(shape, fill):
        t = torch.full(shape, fill, dtype=torch.float64)
        return (t.pin_memory() if pinned else t).numpy()

    def fields():
        return {"As": host((N,), 7.0), "Fs": host((N, 3), 7.0), "Ts": host((N,), 7.0), "Ct": host((N,), 7.0)}

    Uh = torch.from_numpy(U64)
    Uh = (Uh.pin_memory() if pinned else Uh).numpy()
    hn = fields()
    t = 0.0
    for step in range(4):
        if step == 3:
            hn = fields()
        FTa = a.interact(t, w.dt, Ud, fd)
        FTb = b.interact_host64(t, w.dt, Uh, hn)
        assert np.array_equal(fd["As"].cpu().numpy().astype(np.float64), hn["As"]), step
        assert np.array_equal(fd["Ts"].cpu().numpy().astype(np.float64), hn["Ts"]), step
        assert np.array_equal(fd["Ct"].cpu().numpy().astype(np.float64), hn["Ct"]), step
        assert np.array_equal(fd["Fs"].cpu().numpy().astype(np.float64).T, hn["Fs"]), step
        assert np.allclose(FTa, FTb, rtol=1e-12, atol=1e-14)
        st = b.stats()
        assert st["host_sparse"] == (1 if pinned and step in (1, 2) else 0), step
        if st["host_sparse"]:
            assert st["host_h2d_bytes"] == 24 * st["coupling_cells"]
            assert 0 < st["host_d2h_bytes"] < 48 * N
        a.evolve(t, w.dt)
        b.evolve(t, w.dt)
        t += w.dt
    a.close()
    b.close()
