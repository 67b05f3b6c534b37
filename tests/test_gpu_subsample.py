"""SUBSAMPLE lattice counts of the convex 3-D shapes against the oracle's exhaustive FP64 count: spheres, ellipsoids
of large aspect ratio and boxes in random poses, sizes from below a cell to many cells, lattices of 2 to 16 samples
per axis (runs along lattice columns from 5 per axis, 4 x 4 x 4 blocks at 16).  A count differing by one sample
moves As by at least 1/16^3 and fails the 1e-5 tolerance."""
import numpy as np
import pytest

from gpu_helpers import check_interact, run_pair
from sdfibm_gb300 import abi
from sdfibm_gb300.host import make_shape, make_solid
from sdfibm_gb300.workloads import Workload, random_quaternions

pytestmark = pytest.mark.gpu


def _convex_zoo(seed, n_solids=18):
    rng = np.random.default_rng(seed)
    n = 40
    h = 2.0 / n
    mesh = abi.mesh_desc((n, n, n), (-1.0, -1.0, -1.0), (h,) * 3, twod=0)
    solids = []
    quats = random_quaternions(rng, n_solids)
    for i in range(n_solids):
        size = h * np.exp(rng.uniform(np.log(0.4), np.log(8.0)))
        kind = i % 3
        if kind == 0:
            sh = make_shape("Sphere", radius=size)
        elif kind == 1:
            ab = np.exp(rng.uniform(0.0, np.log(6.0), 2))
            sh = make_shape("Ellipsoid", radiusa=size, radiusb=size * ab[0], radiusc=size / ab[1])
        else:
            ab = np.exp(rng.uniform(np.log(0.2), np.log(4.0), 2))
            com = tuple(rng.uniform(-0.3, 0.3, 3) * size)
            sh = make_shape("Box", radiusa=size, radiusb=size * ab[0], radiusc=size * ab[1], com=com)
        d = make_solid(i, sh, 1.2, rng.uniform(-0.8, 0.8, 3), vel=rng.normal(0, 0.1, 3), omega=rng.normal(0, 1, 3))
        for c in range(4):
            d.quat[c] = float(quats[i, c])
        solids.append(d)
    # an axis-aligned box and sphere centred on lattice planes: columns parallel to faces and tangent runs
    solids.append(make_solid(n_solids, make_shape("Box", radiusa=3 * h, radiusb=2 * h, radiusc=2.5 * h), 1.2,
                             (0.5 * h, -0.5, 0.25 * h), vel=(0.1, 0, 0)))
    solids.append(make_solid(n_solids + 1, make_shape("Sphere", radius=4 * h), 1.2, (-0.5, 0.5, 0.0)))
    opt = abi.options(rho_f=1.0, fraction_method=abi.FRACTION_SUBSAMPLE)
    return Workload("convex_zoo", mesh, solids, opt, 0.01, (0.1, -0.2, 0.05), 0.1, seed)


@pytest.mark.parametrize("n", [2, 5, 7, 10, 16])
def test_convex_lattice_counts(cuda_lib, torch_cuda, n):
    w = _convex_zoo(30 + n)
    w.opt.subsample_n = n
    r = run_pair(torch_cuda, w)
    s = check_interact(w, r)
    assert s["coupling_cells"] > 1000


def test_recheck_list_overflow(cuda_lib, torch_cuda):
    """A recheck list of 20 entries: the undecided points it cannot take are re-evaluated in place."""
    import copy
    w = _convex_zoo(40)
    w.opt.subsample_n = 10
    gpu_opt = copy.copy(w.opt)
    gpu_opt.recheck_cap = 20
    r = run_pair(torch_cuda, w, gpu_opt=gpu_opt)
    check_interact(w, r)
    assert r["gpu"].stats()["fp64_rechecks"] > 40
