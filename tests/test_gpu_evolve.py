"""Solid side of the time step on the GPU (SolidCloud::evolve: forcers, AB2 fluid force, gravity, collisions,
motions, Solid::move) against the FP64 oracle: the full rigid-body state after several steps."""
import math

import numpy as np
import pytest

from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi
from sdfibm_gb300.cloud import SolidCloud
from sdfibm_gb300.host import make_forcer, make_motion, make_shape, make_solid, mask_motion
from sdfibm_gb300.workloads import random_quaternions

pytestmark = pytest.mark.gpu

STATE_REL = 1e-9   # positions, velocities, quaternions, forces: the same FP64 sequence up to the order of pair sums
# rho_f = 0 removes the fluid force (its FP32 fractions would differ at 1e-7), leaving FP64 physics on both sides


def _evolve_pair(torch, mesh, solids, opt, dt, steps, U=None):
    gpu = SolidCloud(mesh, solids, opt)
    orc = OracleCloud(mesh, solids, opt, faithful=False)
    N = int(mesh.nx) * int(mesh.ny) * int(mesh.nz)
    Uh = np.zeros((3, N), np.float32) if U is None else U
    Ud = torch.from_numpy(Uh).cuda()
    Uo = Uh.astype(np.float64).reshape(-1)
    fd, fo = gpu.new_fields(), orc.new_fields()
    t = 0.0
    for _ in range(steps):
        gpu.interact(t, dt, Ud, fd)
        orc.interact(t, dt, Uo, fo)
        gpu.evolve(t, dt)
        orc.evolve(t, dt)
        t += dt
    torch.cuda.synchronize()
    return gpu.states(), orc.get_state(), orc.last_pairs()


def _compare(sg, so, fields=("pos", "quat", "vel", "omega", "force", "torque")):
    for i, (a, b) in enumerate(zip(sg, so)):
        for f in fields:
            x = np.array(getattr(a, f)[:])
            y = np.array(getattr(b, f)[:])
            scale = max(1.0, np.abs(y).max())
            assert np.abs(x - y).max() <= STATE_REL * scale, "solid %d %s: %s vs %s" % (i, f, x, y)


def _cluster(rng, n, box, rmin, rmax, big=None):
    """n spheres with lognormal-ish radii packed so that many overlap (contacts in every sub-step)."""
    pos = rng.uniform(box[0], box[1], (n, 3))
    r = np.exp(rng.uniform(math.log(rmin), math.log(rmax), n))
    if big is not None:
        r[0] = big
    return pos, r


def test_collisions_spheres_mode_polydisperse(cuda_lib, torch_cuda):
    """Bounding-sphere contacts of a polydisperse cluster (one large solid spans many fine-grid cells) and a plane."""
    rng = np.random.default_rng(5)
    mesh = abi.mesh_desc((32, 32, 32), (0.0, 0.0, 0.0), (1.0 / 32,) * 3)
    pos, r = _cluster(rng, 160, (0.2, 0.8), 0.01, 0.05, big=0.18)
    quat = random_quaternions(rng, len(r))
    solids = []
    for i in range(len(r)):
        kind = i % 3
        if kind == 0:
            sh = make_shape("Sphere", radius=r[i])
        elif kind == 1:
            sh = make_shape("Ellipsoid", radiusa=r[i], radiusb=0.7 * r[i], radiusc=0.5 * r[i])
        else:
            sh = make_shape("Box", radiusa=0.5 * r[i], radiusb=0.4 * r[i], radiusc=0.3 * r[i])
        d = make_solid(i, sh, 1.5, pos[i], vel=rng.normal(0, 0.05, 3), omega=rng.normal(0, 1, 3))
        for c in range(4):
            d.quat[c] = float(quat[i, c])
        solids.append(d)
    solids.append(make_solid(len(solids), make_shape("Plane"), 1.0, (0.5, 0.25, 0.5), (0, 0, 0),
                             motion=mask_motion("b000000")))
    opt = abi.options(rho_f=0.0, collision_mode=abi.COLLISION_SPHERES, gravity=(0, -1.0, 0))
    sg, so, pairs = _evolve_pair(torch_cuda, mesh, solids, opt, 1e-3, 3)
    assert pairs > 100
    _compare(sg, so)


def test_collisions_reference_mode_walls(cuda_lib, torch_cuda):
    """The reference's contact table: circles against circles and against the four walls (2-D)."""
    rng = np.random.default_rng(6)
    mesh = abi.mesh_desc((64, 64, 1), (0.0, 0.0, -0.5), (1.0 / 64, 1.0 / 64, 1.0), twod=1)
    solids = []
    walls = [((0.0, 0.5, 0.0), (0, 0, -90)), ((1.0, 0.5, 0.0), (0, 0, 90)), ((0.5, 0.0, 0.0), (0, 0, 0)),
             ((0.5, 1.0, 0.0), (0, 0, 180))]
    for i, (p, e) in enumerate(walls):
        solids.append(make_solid(i, make_shape("Plane"), 1.0, p, e, motion=mask_motion("b000000")))
    pos = np.zeros((60, 3))
    pos[:, :2] = rng.uniform(0.03, 0.97, (60, 2))
    for i in range(60):
        sh = make_shape("Circle", radius=float(rng.uniform(0.03, 0.06)))
        solids.append(make_solid(len(solids), sh, 1.5, pos[i], vel=(*rng.normal(0, 0.1, 2), 0.0),
                                 omega=(0, 0, rng.normal(0, 1))))
    opt = abi.options(rho_f=0.0, collision_mode=abi.COLLISION_REFERENCE, gravity=(0, -1.0, 0))
    sg, so, pairs = _evolve_pair(torch_cuda, mesh, solids, opt, 1e-3, 3)
    assert pairs > 60
    _compare(sg, so)


def test_collisions_outside_the_grid_are_ignored(cuda_lib, torch_cuda):
    """The reference's UGrid never pairs solids whose centre lies off the grid; overlapping pairs there stay free."""
    mesh = abi.mesh_desc((16, 16, 16), (0.0, 0.0, 0.0), (1.0 / 16,) * 3)
    solids = [make_solid(0, make_shape("Sphere", radius=0.1), 1.5, (-0.05, 0.5, 0.5)),
              make_solid(1, make_shape("Sphere", radius=0.1), 1.5, (-0.05, 0.6, 0.5)),
              make_solid(2, make_shape("Sphere", radius=0.1), 1.5, (0.5, 0.5, 0.5)),
              make_solid(3, make_shape("Sphere", radius=0.1), 1.5, (0.5, 0.62, 0.5))]
    opt = abi.options(rho_f=0.0, collision_mode=abi.COLLISION_SPHERES)
    sg, so, _ = _evolve_pair(torch_cuda, mesh, solids, opt, 1e-3, 1)
    _compare(sg, so)
    # the pair on the grid pushed itself apart (the contact is stiff: it may have separated by the last sub-step);
    # the pair off the grid kept its rest state
    assert np.allclose(sg[0].vel[:], 0.0) and np.allclose(sg[1].vel[:], 0.0)
    assert not np.allclose(sg[2].vel[:], 0.0) and not np.allclose(sg[3].vel[:], 0.0)


def test_motions_and_forcers(cuda_lib, torch_cuda):
    """Every motion and forcer, without collisions (the one-launch path), over several steps."""
    mesh = abi.mesh_desc((16, 16, 16), (0.0, 0.0, 0.0), (1.0 / 16,) * 3)
    rng = np.random.default_rng(7)
    motions = [None, make_motion("Motion000002", 2.0), make_motion("Motion110002", 3.0),
               make_motion("Motion222000", 0.1, -0.2, 0.05), make_motion("MotionSineDirectional", 0.1, 2.0, 0, 1, 0),
               mask_motion("b101010"), make_motion("MotionRotor", 4.0, 0.1, 0.3, 0.5), make_motion("MotionOpenClose")]
    forcers = [None, make_forcer("Constant", 0.1, -0.2, 0.3, 0.01, 0.02, -0.03),
               make_forcer("Spring", 0.5, 0.5, 0.5, 2.0, 0.05), make_forcer("Magnetic", 0, 1, 0, 0.3, 2.0)]
    solids = []
    for i in range(len(motions) * len(forcers)):
        sh = make_shape("Ellipsoid", radiusa=0.05, radiusb=0.04, radiusc=0.03)
        d = make_solid(i, sh, 1.3, rng.uniform(0.2, 0.8, 3), euler_deg=rng.uniform(0, 90, 3),
                       vel=rng.normal(0, 0.1, 3), omega=rng.normal(0, 1, 3), motion=motions[i % len(motions)],
                       forcer=forcers[i // len(motions)])
        solids.append(d)
    opt = abi.options(rho_f=0.0, collision_mode=abi.COLLISION_OFF, gravity=(0, 0, -9.81))
    U = (np.random.default_rng(8).standard_normal((3, 16 ** 3)) * 0.1).astype(np.float32)
    sg, so, _ = _evolve_pair(torch_cuda, mesh, solids, opt, 0.01, 4, U=U)
    _compare(sg, so)
