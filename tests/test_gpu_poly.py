"""The unstructured-mesh path (sdfibm_cuda_create_polymesh) on the GPU against the FP64 oracle's polyMesh path on the
same OpenFOAM lists, and against the As the reference ships for re200 on its graded multi-block mesh.

Meshes come from tests/polymesh_gen.py: the re200 blockMeshDict (9 graded blocks, 78400 cells), a single block
with jiggled interior points (general hexahedra with non-planar faces) in 3-D, and a single uniform block (the
uniform path's own mesh written as a polyMesh).  Contract as for the uniform path: touched sets and types exact,
As / Ts / Fs per cell within 1e-5 relative, force and torque within 1e-6 normwise.
"""
import numpy as np
import pytest

from conftest import golden
from oracle.oracle import Lowering, OracleCloud
from polymesh_gen import block_mesh, jiggle, uniform_block
from sdfibm_gb300 import abi
from sdfibm_gb300.cloud import SolidCloud

pytestmark = pytest.mark.gpu

L = Lowering


def _pair(torch, poly, solids, opt, U, dt, steps=1, twod=False, evolve=False):
    pts, fo, fl, ow, nb, nc = poly
    gpu = SolidCloud.from_polymesh(pts, fo, fl, ow, nb, solids, opt, twod=twod)
    box = abi.mesh_desc((1, 1, 1), (0, 0, 0), (1, 1, 1), twod=int(twod))
    orc = OracleCloud(box, solids, opt, faithful=False, polymesh=(pts, fo, fl, ow, nb))
    assert gpu.ncells == orc.N == nc
    fd, fo_ = gpu.new_fields(), orc.new_fields()
    Ud = torch.from_numpy(U.astype(np.float32)).cuda()
    Uo = U.astype(np.float32).astype(np.float64).reshape(-1)
    t = 0.0
    for _ in range(steps):
        FTg = gpu.interact(t, dt, Ud, fd)
        FTo = orc.interact(t, dt, Uo, fo_)
        if evolve:
            gpu.evolve(t, dt)
            orc.evolve(t, dt)
        t += dt
    return gpu, orc, fd, fo_, FTg, FTo, Uo


def _check(gpu, orc, fd, fo, FTg, FTo, Uo, dt, rho_f, S, vol_mean):
    N = orc.N
    for s in range(S):
        cg, tg = gpu.touched(s)
        co, to = orc.touched(s)
        assert np.array_equal(cg, co), "touched cells of solid %d differ (%d vs %d)" % (s, len(cg), len(co))
        assert np.array_equal(tg, to), "cell types of solid %d differ" % s
    assert np.array_equal(fd["Ct"].cpu().numpy(), fo["Ct"])
    for k in ("As", "Ts"):
        g = fd[k].cpu().numpy().astype(np.float64)
        assert (np.abs(g - fo[k]) <= 1e-5 * np.abs(fo[k]) + 1e-9).all(), k
    g = fd["Fs"].cpu().numpy().astype(np.float64).reshape(3, N)
    o = fo["Fs"].reshape(3, N)
    assert (np.abs(g - o) <= 1e-5 * np.abs(o) + 1e-7 * np.abs(o).max()).all()
    # force / torque: normwise against the sum over the solid's cells of the magnitudes of the contributions,
    # rho_f |Fs| V, with the cell volume bounded by twice the mean (the jiggled meshes stay within that)
    Vmax = 2.0 * vol_mean
    Fo = fo["Fs"].reshape(3, N)
    for s in range(S):
        cells, _ = orc.touched(s)
        scale = rho_f * Vmax * np.linalg.norm(Fo[:, cells], axis=0).sum() if len(cells) else 0.0
        assert np.linalg.norm(FTg[s, :3] - FTo[s, :3]) <= 1e-6 * scale + 1e-12 * np.abs(FTo[s, :3]).max(), s


def test_poly_re200_multiblock_against_the_shipped_As(cuda_lib, torch_cuda):
    """initialCorrect (interact(0, 1)) of the re200 case on its 9-block graded mesh: the library's unstructured path
    equals the oracle on the same mesh, and both reproduce the As the reference ships (the centre block's cells; the
    cell the shipped field holds at 1.0 against the serial algorithm's 0.6685 is reported, as in the uniform test)."""
    g = golden("re200_blocks.npz")
    poly = block_mesh(g["vertices"], g["hexes"], g["counts"], g["grading"])
    solid = L.make_solid(0, L.make_shape("Circle", radius=1.0), 1.0, (0, 0, 0), motion=L.mask_motion("b000000"))
    N = poly[5]
    gpu, orc, fd, fo, FTg, FTo, Uo = _pair(torch_cuda, poly, [solid], abi.options(rho_f=1.0), np.zeros((3, N)), 1.0,
                                           twod=True)
    _check(gpu, orc, fd, fo, FTg, FTo, Uo, 1.0, 1.0, 1, vol_mean=0.0)
    As = fd["As"].cpu().numpy().astype(np.float64)
    assert (np.delete(As, np.arange(20800, 20800 + 14400)) == 0).all()
    centre = As[20800:20800 + 14400].reshape(120, 120)
    ref = golden("re200_As.npz")["As"].reshape(120, 120)
    mask = np.ones_like(ref, dtype=bool)
    mask[50, 57] = False
    assert (np.abs(centre - ref)[mask] <= 1e-5 * ref[mask] + 1e-9).all()
    assert (centre > 1e-9).sum() >= 344 and 0.6 < centre[50, 57] < 0.7
    gpu.close()


@pytest.mark.parametrize("seed", [1, 2])
def test_poly_jiggled_hexahedra_3d(cuda_lib, torch_cuda, seed):
    """General hexahedra (interior points moved by up to 30 % of a cell, faces no longer planar), spheres, ellipsoids
    and boxes crossing each other and the mesh boundary, two coupled steps with motion."""
    n = 20
    h = 1.0 / n
    pts, fo, fl, ow, nb, nc = uniform_block((n, n, n), (0, 0, 0), (h, h, h))
    pts = jiggle(pts, 0.3 * h, seed)
    rng = np.random.default_rng(seed)
    solids = []
    kinds = [("Sphere", dict(radius=0.18)), ("Ellipsoid", dict(radiusa=0.1, radiusb=0.2, radiusc=0.15)),
             ("Box", dict(radiusa=0.1, radiusb=0.15, radiusc=0.08)), ("Sphere", dict(radius=0.3 * h))]
    for i, (t, kw) in enumerate(kinds):
        d = L.make_solid(i, L.make_shape(t, **kw), 1.3, rng.uniform(0.15, 0.85, 3), tuple(rng.uniform(0, 90, 3)),
                         vel=rng.normal(0, 0.1, 3), omega=rng.normal(0, 1.0, 3))
        solids.append(d)
    U = rng.normal(0, 0.1, (3, nc))
    opt = abi.options(rho_f=1.1)
    gpu, orc, fd, fo, FTg, FTo, Uo = _pair(torch_cuda, (pts, fo, fl, ow, nb, nc), solids, opt, U, 0.01, steps=2,
                                           evolve=True)
    _check(gpu, orc, fd, fo, FTg, FTo, Uo, 0.01, 1.1, len(solids), vol_mean=h ** 3)
    assert gpu.stats()["coupling_cells"] > 100
    # fixInternal with the mesh's cell centres
    Ud = torch_cuda.from_numpy(U.astype(np.float32)).cuda()
    gpu.fix_internal(fd["Ct"], Ud)
    Uf = orc.fix_internal(fo["Ct"], Uo)
    assert np.abs(Ud.cpu().numpy().astype(np.float64).reshape(-1) - Uf).max() <= 1e-6
    gpu.close()


def test_poly_uniform_block_matches_the_uniform_path(cuda_lib, torch_cuda):
    """The uniform path's mesh written as a polyMesh: the unstructured path gives the uniform path's touched sets and
    fields (cell centres from the pyramid decomposition agree with the closed form to rounding)."""
    torch = torch_cuda
    n, origin, h = (24, 20, 16), (-1.0, -0.8, -0.6), (2 / 24, 1.6 / 20, 1.2 / 16)
    pts, fo, fl, ow, nb, nc = uniform_block(n, origin, h)
    solids = [L.make_solid(0, L.make_shape("Sphere", radius=0.4), 1.0, (0.05, 0.02, -0.03), vel=(0.1, 0, 0),
                           omega=(0, 0, 1)),
              L.make_solid(1, L.make_shape("Box", radiusa=0.2, radiusb=0.3, radiusc=0.25), 1.0, (0.5, 0.3, 0.1),
                           (10, 20, 30))]
    opt = abi.options(rho_f=1.0)
    U = np.random.default_rng(0).normal(size=(3, nc)).astype(np.float32)
    a = SolidCloud(abi.mesh_desc(n, origin, h), solids, opt)
    b = SolidCloud.from_polymesh(pts, fo, fl, ow, nb, solids, opt)
    fa, fb = a.new_fields(), b.new_fields()
    Ud = torch.from_numpy(U).cuda()
    FTa = a.interact(0.0, 0.01, Ud, fa)
    FTb = b.interact(0.0, 0.01, Ud, fb)
    for s in range(2):
        ca, ta = a.touched(s)
        cb, tb = b.touched(s)
        assert np.array_equal(ca, cb) and np.array_equal(ta, tb)
    assert torch.equal(fa["Ct"], fb["Ct"])
    assert (fa["As"] - fb["As"]).abs().max().item() <= 1e-5
    assert np.abs(FTa - FTb).max() <= 1e-5 * np.abs(FTa).max()
    # host fields (FP32 planes and FP64 in OpenFOAM's layout) through whole-field copies
    hf = {"As": np.zeros(nc, np.float32), "Fs": np.zeros(3 * nc, np.float32), "Ts": np.zeros(nc, np.float32),
          "Ct": np.zeros(nc, np.int32)}
    FTh = b.interact_host(0.0, 0.01, U, hf)
    assert np.array_equal(hf["As"], fb["As"].cpu().numpy())
    np.testing.assert_allclose(FTh, FTb, rtol=1e-9, atol=1e-12 * np.abs(FTb).max())
    h64 = {"As": np.zeros(nc), "Fs": np.zeros((nc, 3)), "Ts": np.zeros(nc), "Ct": np.zeros(nc)}
    b.interact_host64(0.0, 0.01, np.ascontiguousarray(U.T.astype(np.float64)), h64)
    assert np.array_equal(h64["As"], fb["As"].cpu().numpy().astype(np.float64))
    assert np.array_equal(h64["Ct"], fb["Ct"].cpu().numpy().astype(np.float64))
    a.close()
    b.close()
