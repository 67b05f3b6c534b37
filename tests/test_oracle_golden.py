"""The oracle pinned against the reference's shipped artefacts (CPU), and the library against the same artefacts
(GPU)."""
import numpy as np
import pytest

from conftest import golden
from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi
from sdfibm_gb300.host import make_shape, make_solid, mask_motion

# cell (j=50, i=57) of the re200 centre block holds 1.0 in the shipped field while the shipped serial algorithm gives
# 0.6685 for every possible vertex order: it is excluded and reported (see the fixture script).
RE200_FLAGGED = [(50, 57)]


def re200_case(faithful=True):
    g = golden("re200_As.npz")
    mesh = abi.mesh_desc((120, 120, 1), g["origin"], g["h"], twod=1)
    solid = make_solid(0, make_shape("Circle", radius=1.0), 1.0, (0, 0, 0), motion=mask_motion("b000000"))
    oc = OracleCloud(mesh, [solid], abi.options(rho_f=1.0), faithful=faithful)
    f = oc.new_fields()
    oc.interact(0.0, 1.0, np.zeros(3 * oc.N), f)   # SolidCloud::initialCorrect = interact(0, 1)
    return g["As"].reshape(120, 120), f["As"].reshape(120, 120)


def test_re200_golden_As():
    ref, got = re200_case()
    mask = np.ones_like(ref, dtype=bool)
    for j, i in RE200_FLAGGED:
        mask[j, i] = False
    d = np.abs(ref - got)
    # 346 cells bit-for-bit up to 1e-12; 5 cells where blockMesh's point coordinates put a vertex on the circle to
    # rounding hold As < 1e-9 in the shipped field and 0 here
    assert d[mask].max() < 1e-9
    assert (d[mask] < 1e-12).sum() >= 346
    assert (got > 0).sum() == 346 and (ref > 0).sum() == 352
    assert (got == 1).sum() == 276 and (ref == 1).sum() == 276
    # the flagged cell is a genuine cut cell in the serial algorithm
    assert 0.6 < got[50, 57] < 0.7 and ref[50, 57] == 1.0


def test_re200_total_area():
    ref, got = re200_case()
    assert abs((got * 0.01).sum() - 3.1352207447) < 1e-9
    assert abs((ref * 0.01).sum() - 3.1385353449) < 1e-9


def test_falling_ellipse_uniform_matches_polymesh():
    """The implicit uniform mesh (closed-form geometry, OpenFOAM ordering) reproduces the oracle run on the
    reference's own OpenFOAM polyMesh of examples/falling_ellipse."""
    g = golden("falling_ellipse.npz")
    shape = make_shape("Ellipse", radiusa=0.3, radiusb=0.15)
    solid = make_solid(0, shape, 2.0, (0.5, 3.5, 0.0), (0.0, 0.0, -45.0), motion=mask_motion("b111111"))
    mesh = abi.mesh_desc((100, 200, 1), (0.0, 0.0, -0.5), (0.02, 0.02, 1.0), twod=1)
    oc = OracleCloud(mesh, [solid], abi.options(rho_f=1.0), faithful=False)
    N = oc.N
    rng = np.random.default_rng(int(g["U_seed"]))
    U = (rng.standard_normal((3, N), dtype=np.float32) * np.float32(g["U_std"])).astype(np.float64)
    f = oc.new_fields()
    FT = oc.interact(0.0, float(g["dt"]), U, f)
    cells, types = oc.touched(0)
    assert np.array_equal(cells, g["cells"]) and np.array_equal(types, g["types"])
    assert np.abs(f["As"][cells] - g["As"]).max() < 1e-12
    assert np.abs(f["Fs"].reshape(3, N)[:, cells] - g["Fs"]).max() < 1e-9
    assert np.abs(FT - g["FT"]).max() < 1e-12 * np.abs(g["FT"]).max() + 1e-15


@pytest.mark.gpu
def test_re200_golden_on_the_gpu(cuda_lib, torch_cuda):
    """The library's initialCorrect pass (interact(0, 1), REF-GEO) against the As the reference ships for re200: the
    same cells as the oracle, FP32 fractions within the coupling tolerance of the shipped FP64 values."""
    torch = torch_cuda
    from sdfibm_gb300.cloud import SolidCloud
    g = golden("re200_As.npz")
    mesh = abi.mesh_desc((120, 120, 1), g["origin"], g["h"], twod=1)
    solid = make_solid(0, make_shape("Circle", radius=1.0), 1.0, (0, 0, 0), motion=mask_motion("b000000"))
    cloud = SolidCloud(mesh, [solid], abi.options(rho_f=1.0))
    f = cloud.new_fields()
    cloud.interact(0.0, 1.0, torch.zeros((3, 14400), dtype=torch.float32, device="cuda"), f)
    got = f["As"].cpu().numpy().astype(np.float64).reshape(120, 120)
    cells, _ = cloud.touched(0)
    cloud.close()
    _, orc = re200_case(faithful=False)
    assert len(cells) == (orc > 0).sum() == 346
    ref = g["As"].reshape(120, 120)
    mask = np.ones_like(ref, dtype=bool)
    for j, i in RE200_FLAGGED:
        mask[j, i] = False
    # the 5 cells at blockMesh rounding level hold < 1e-9 in the shipped field and 0 here, as in the oracle
    assert (np.abs(got - ref)[mask] <= 1e-5 * ref[mask] + 1e-9).all()
    # 344 cells above 1e-9 (two cut cells hold 3.5e-11 in FP64), 276 of them at 1
    assert (got > 1e-9).sum() == 344 and (got == 1).sum() == 276
    assert 0.6 < got[50, 57] < 0.7


@pytest.mark.gpu
def test_falling_ellipse_golden_on_the_gpu(cuda_lib, torch_cuda):
    """The library on the uniform form of examples/falling_ellipse against the oracle's run on the reference's own
    polyMesh: touched cells and types exact, As and Fs within the coupling tolerance, force and torque within 1e-6."""
    torch = torch_cuda
    from sdfibm_gb300.cloud import SolidCloud
    g = golden("falling_ellipse.npz")
    shape = make_shape("Ellipse", radiusa=0.3, radiusb=0.15)
    solid = make_solid(0, shape, 2.0, (0.5, 3.5, 0.0), (0.0, 0.0, -45.0), motion=mask_motion("b111111"))
    mesh = abi.mesh_desc((100, 200, 1), (0.0, 0.0, -0.5), (0.02, 0.02, 1.0), twod=1)
    N = 20000
    rng = np.random.default_rng(int(g["U_seed"]))
    U = rng.standard_normal((3, N), dtype=np.float32) * np.float32(g["U_std"])
    cloud = SolidCloud(mesh, [solid], abi.options(rho_f=1.0))
    f = cloud.new_fields()
    FT = cloud.interact(0.0, float(g["dt"]), torch.from_numpy(U).cuda(), f)
    cells, types = cloud.touched(0)
    As = f["As"].cpu().numpy().astype(np.float64)
    Fs = f["Fs"].cpu().numpy().astype(np.float64).reshape(3, N)
    cloud.close()
    assert np.array_equal(cells, g["cells"]) and np.array_equal(types, g["types"])
    assert (np.abs(As[cells] - g["As"]) <= 1e-5 * np.abs(g["As"]) + 1e-9).all()
    assert (np.abs(Fs[:, cells] - g["Fs"]) <= 1e-5 * np.abs(g["Fs"]) + 1e-7 * np.abs(g["Fs"]).max()).all()
    # force and torque normwise within 1e-6 of the sum of the per-cell contributions' magnitudes (the coupling's bar)
    V = 0.02 * 0.02 * 1.0
    i, j = cells % 100, cells // 100
    r = np.stack([(i + 0.5) * 0.02 - 0.5, (j + 0.5) * 0.02 - 3.5, np.zeros(len(cells))])
    dF = g["Fs"] * V
    scale_f = np.linalg.norm(dF, axis=0).sum()
    scale_t = np.linalg.norm(np.cross(r.T, dF.T), axis=1).sum()
    assert np.linalg.norm(FT[0, :3] - g["FT"][0, :3]) <= 1e-6 * scale_f
    assert np.linalg.norm(FT[0, 3:] - g["FT"][0, 3:]) <= 1e-6 * scale_t


def test_polymesh_generator_single_block_equals_the_uniform_mesh():
    """tests/polymesh_gen.py writes the uniform mesh as OpenFOAM lists: the oracle's polyMesh path on them gives the
    uniform path's touched sets and fields (to the rounding of the triangle-fan face geometry)."""
    from oracle.oracle import Lowering as L
    from polymesh_gen import uniform_block
    n, origin, h = (24, 20, 16), (-1.0, -0.8, -0.6), (2 / 24, 1.6 / 20, 1.2 / 16)
    pts, fo, fl, ow, nb, nc = uniform_block(n, origin, h)
    sol = [L.make_solid(0, L.make_shape("Sphere", radius=0.4), 1.0, (0.05, 0.02, -0.03), vel=(0.1, 0, 0),
                        omega=(0, 0, 1)),
           L.make_solid(1, L.make_shape("Box", radiusa=0.2, radiusb=0.3, radiusc=0.25), 1.0, (0.5, 0.3, 0.1),
                        (10, 20, 30))]
    opt = abi.options(rho_f=1.0)
    ou = OracleCloud(abi.mesh_desc(n, origin, h), sol, opt, faithful=False)
    op = OracleCloud(abi.mesh_desc(n, origin, h), sol, opt, faithful=False, polymesh=(pts, fo, fl, ow, nb))
    U = np.random.default_rng(0).normal(size=3 * nc)
    fu, fp = ou.new_fields(), op.new_fields()
    FTu = ou.interact(0.0, 0.01, U, fu)
    FTp = op.interact(0.0, 0.01, U, fp)
    for s in range(2):
        cu, tu = ou.touched(s)
        cp, tp = op.touched(s)
        assert np.array_equal(cu, cp) and np.array_equal(tu, tp)
    assert np.abs(fu["As"] - fp["As"]).max() < 1e-12
    assert np.abs(FTu - FTp).max() < 1e-12 * np.abs(FTu).max()


def test_re200_multiblock_mesh_reproduces_the_shipped_As():
    """The re200 case on its own 9-block graded mesh (rebuilt from the reference's blockMeshDict by
    tests/polymesh_gen.py) through the oracle's polyMesh path: every cell outside the centre block stays 0 and the
    centre block reproduces the shipped As (the flagged cell aside) to 1e-9."""
    from oracle.oracle import Lowering as L
    from polymesh_gen import block_mesh
    g = golden("re200_blocks.npz")
    pts, fo, fl, ow, nb, nc = block_mesh(g["vertices"], g["hexes"], g["counts"], g["grading"])
    assert nc == 78400
    solid = L.make_solid(0, L.make_shape("Circle", radius=1.0), 1.0, (0, 0, 0), motion=L.mask_motion("b000000"))
    oc = OracleCloud(abi.mesh_desc((1, 1, 1), (0, 0, 0), (1, 1, 1), twod=1), [solid], abi.options(rho_f=1.0),
                     faithful=False, polymesh=(pts, fo, fl, ow, nb))
    f = oc.new_fields()
    oc.interact(0.0, 1.0, np.zeros(3 * oc.N), f)
    As = f["As"]
    assert (np.delete(As, np.arange(20800, 20800 + 14400)) == 0).all()
    centre = As[20800:20800 + 14400].reshape(120, 120)
    ref = golden("re200_As.npz")["As"].reshape(120, 120)
    mask = np.ones_like(ref, dtype=bool)
    for j, i in RE200_FLAGGED:
        mask[j, i] = False
    assert np.abs(centre - ref)[mask].max() < 1e-9
    assert (centre > 1e-9).sum() >= 344 and 0.6 < centre[50, 57] < 0.7
