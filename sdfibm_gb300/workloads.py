"""Seeded synthetic workloads of the five coupling configurations (uniform hex meshes, FP32 fields).

  cylinder2d      400x200x1 on [-10,30]x[-10,10]x[-0.5,0.5], one circle r=0.5 at the origin (on_twod), v=w=0,
                  rho_s=1, rho_f=1, U=(1,0,0)+N(0,0.05^2) per component (seed 1), dt=0.005
  sedimentation2d 1024x1024x1 on [0,1]^2x[-0.5,0.5], 4 wall planes listed first (normals into the fluid,
                  Motion01Mask b000000) then 100 circles r=0.03 placed with gap >= 0.01 (seed 2), v~N(0,0.1^2),
                  w_z~N(0,1), rho_s=1.5, Motion01Mask b110001, U~N(0,0.1^2), g=(0,-10,0), dt=1e-3, collisions
  poly3d_256      256^3 on [0,1]^3, 4096 solids (half Sphere, half Ellipsoid), r~LogNormal(ln 0.01, 0.4), ellipsoid
                  axes r*(1,U[1,3],U[1,3]), uniform random orientations, non-overlapping bounding spheres,
                  v~N(0,0.05^2), rho_s=1.5, U~N(0,0.1^2), dt=1e-3
  poly3d_512      512^3 on [0,1]^3, 16384 solids (Sphere / Ellipsoid / Box, a third each), r~LogNormal(ln 0.004, 0.5),
                  half extents / axes r*(1,U[1,3],U[1,3]), random orientations, non-overlapping, v~N(0,0.05^2),
                  rho_s=1.5, U~N(0,0.1^2), dt=1e-3, soft-sphere collisions on bounding spheres
The sedimentation radius is 0.03: 100 circles of radius 0.05 with a 0.01 gap cannot be placed in the unit square
(they would cover 95% of it, more than the densest hexagonal packing).
A ``scale`` < 1 shrinks meshes and solid counts for tests while keeping the per-solid resolution (r/h); ``seed``
draws another instance of the same distribution (the learned fraction's band is calibrated on one that the
benchmark does not use).
The reference's public benchmark inputs are not used: these seeded inputs stand in for them.
Every builder takes ``lower``: the object whose make_shape / make_solid / mask_motion build the solids (default: the
C++ lowering of include/sdfibm_host.h, i.e. sdfibm_gb300.host); any lowering with the same signatures that restates
the reference's constructors gives the same descriptors bit for bit.
"""
import math

import numpy as np

from . import abi


def _host_lowering():
    from . import host
    return host


class Workload:
    def __init__(self, name, mesh, solids, opt, dt, u_mean, u_std, u_seed):
        self.name = name
        self.mesh = mesh
        self.solids = solids
        self.opt = opt
        self.dt = dt
        self.u_mean = np.asarray(u_mean, dtype=np.float64)
        self.u_std = u_std
        self.u_seed = u_seed

    @property
    def ncells(self):
        return int(self.mesh.nx) * int(self.mesh.ny) * int(self.mesh.nz)

    def U_numpy(self):
        """FP32 velocity field [3][N] (host)."""
        rng = np.random.default_rng(self.u_seed)
        N = self.ncells
        U = rng.standard_normal((3, N), dtype=np.float32) * np.float32(self.u_std)
        U += self.u_mean.astype(np.float32)[:, None]
        return U

    def U_torch(self, device="cuda"):
        """FP32 velocity field [3][N] generated on the device (large meshes)."""
        import torch
        g = torch.Generator(device=device)
        g.manual_seed(int(self.u_seed))
        U = torch.randn((3, self.ncells), generator=g, device=device, dtype=torch.float32) * float(self.u_std)
        U += torch.tensor(self.u_mean, dtype=torch.float32, device=device)[:, None]
        return U


def random_quaternions(rng, n):
    """Uniform random unit quaternions (w, x, y, z), Shoemake's method."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(u1) * np.cos(2 * np.pi * u3), np.sqrt(1 - u1) * np.sin(2 * np.pi * u2),
                  np.sqrt(1 - u1) * np.cos(2 * np.pi * u2), np.sqrt(u1) * np.sin(2 * np.pi * u3)], axis=1)
    return q / np.linalg.norm(q, axis=1, keepdims=True)


def place_spheres(rng, radii, lo, hi, gap, twod=False, max_tries=20000):
    """Random sequential placement of non-overlapping spheres (largest first) inside [lo+r, hi-r]."""
    n = len(radii)
    order = np.argsort(-radii)
    pos = np.zeros((n, 3))
    placed_p, placed_r = [], []
    cell = max(2 * radii.max() + gap, 1e-9)
    grid = {}
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    for idx in order:
        r = radii[idx]
        ok = False
        for _ in range(max_tries):
            p = lo + r + rng.random(3) * (hi - lo - 2 * r)
            if twod:
                p[2] = 0.0
            key = tuple(np.floor(p / cell).astype(int))
            clash = False
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in ((0,) if twod else (-1, 0, 1)):
                        for j in grid.get((key[0] + dx, key[1] + dy, key[2] + dz), ()):
                            if np.linalg.norm(placed_p[j] - p) < placed_r[j] + r + gap:
                                clash = True
                                break
                        if clash:
                            break
                    if clash:
                        break
                if clash:
                    break
            if not clash:
                ok = True
                break
        if not ok:
            raise RuntimeError("could not place solid %d (r=%g)" % (idx, r))
        grid.setdefault(key, []).append(len(placed_p))
        placed_p.append(p)
        placed_r.append(r)
        pos[idx] = p
    return pos


def cylinder2d(scale=1.0, lower=None):
    L = lower or _host_lowering()
    nx, ny = max(8, int(round(400 * scale))), max(4, int(round(200 * scale)))
    mesh = abi.mesh_desc((nx, ny, 1), (-10.0, -10.0, -0.5), (40.0 / nx, 20.0 / ny, 1.0), twod=1)
    shape = L.make_shape("Circle", radius=0.5)
    solids = [L.make_solid(0, shape, 1.0, (0.0, 0.0, 0.0))]
    opt = abi.options(rho_f=1.0)
    return Workload("cylinder2d", mesh, solids, opt, 0.005, (1.0, 0.0, 0.0), 0.05, 1)


def sedimentation2d(scale=1.0, ncircles=None, collision=abi.COLLISION_REFERENCE, lower=None):
    L = lower or _host_lowering()
    n = max(16, int(round(1024 * scale)))
    mesh = abi.mesh_desc((n, n, 1), (0.0, 0.0, -0.5), (1.0 / n, 1.0 / n, 1.0), twod=1)
    rng = np.random.default_rng(2)
    nc = ncircles if ncircles is not None else 100
    r = 0.03
    pos = place_spheres(rng, np.full(nc, r), (0, 0, 0), (1, 1, 0), 0.01, twod=True)
    wall = L.make_shape("Plane")
    walls = [((0.0, 0.5, 0.0), (0, 0, -90.0)), ((1.0, 0.5, 0.0), (0, 0, 90.0)),
             ((0.5, 0.0, 0.0), (0, 0, 0.0)), ((0.5, 1.0, 0.0), (0, 0, 180.0))]
    fixed = L.mask_motion("b000000")
    planar = L.mask_motion("b110001")
    solids = [L.make_solid(i, wall, 1.5, p, e, motion=fixed) for i, (p, e) in enumerate(walls)]
    circle = L.make_shape("Circle", radius=r)
    vel = rng.normal(0.0, 0.1, (nc, 2))
    om = rng.normal(0.0, 1.0, nc)
    for i in range(nc):
        solids.append(L.make_solid(len(solids), circle, 1.5, pos[i], vel=(vel[i, 0], vel[i, 1], 0.0),
                                 omega=(0.0, 0.0, om[i]), motion=planar))
    opt = abi.options(rho_f=1.0, gravity=(0.0, -10.0, 0.0), collision_mode=collision)
    return Workload("sedimentation2d", mesh, solids, opt, 1e-3, (0.0, 0.0, 0.0), 0.1, 3)


def _poly3d(name, n, nsolids, r_median, sigma, kinds, seed, collision, lower):
    L = lower or _host_lowering()
    mesh = abi.mesh_desc((n, n, n), (0.0, 0.0, 0.0), (1.0 / n,) * 3, twod=0)
    rng = np.random.default_rng(seed)
    r = np.exp(rng.normal(math.log(r_median), sigma, nsolids))
    a = rng.uniform(1.0, 3.0, nsolids)
    b = rng.uniform(1.0, 3.0, nsolids)
    kind = np.array([kinds[i % len(kinds)] for i in range(nsolids)])
    factor = np.where(kind == "Sphere", 1.0, np.where(kind == "Ellipsoid", np.maximum(a, b), np.sqrt(1 + a * a + b * b)))
    # the lognormal tail is clipped so that every bounding sphere fits a fifth of the unit box (this only bites on
    # the few-solid test configurations; the full-size draws stay below 0.15)
    r = np.minimum(r, 0.2 / factor)
    bound = r * factor
    pos = place_spheres(rng, bound, (0, 0, 0), (1, 1, 1), 0.0)
    quat = random_quaternions(rng, nsolids)
    vel = rng.normal(0.0, 0.05, (nsolids, 3))
    solids = []
    for i in range(nsolids):
        if kind[i] == "Sphere":
            sh = L.make_shape("Sphere", radius=r[i])
        elif kind[i] == "Ellipsoid":
            sh = L.make_shape("Ellipsoid", radiusa=r[i], radiusb=r[i] * a[i], radiusc=r[i] * b[i])
        else:
            sh = L.make_shape("Box", radiusa=r[i], radiusb=r[i] * a[i], radiusc=r[i] * b[i])
        d = L.make_solid(i, sh, 1.5, pos[i], vel=vel[i])
        for c in range(4):
            d.quat[c] = float(quat[i, c])
        solids.append(d)
    opt = abi.options(rho_f=1.0, collision_mode=collision)
    return Workload(name, mesh, solids, opt, 1e-3, (0.0, 0.0, 0.0), 0.1, seed + 100)


def poly3d_256(scale=1.0, collision=abi.COLLISION_OFF, lower=None, seed=4):
    n = max(16, int(round(256 * scale)))
    ns = max(4, int(round(4096 * scale ** 3)))
    return _poly3d("poly3d_256", n, ns, 0.01 * 256 / n, 0.4, ["Sphere", "Ellipsoid"], seed, collision, lower)


def poly3d_512(scale=1.0, collision=abi.COLLISION_SPHERES, lower=None, seed=5):
    n = max(16, int(round(512 * scale)))
    ns = max(6, int(round(16384 * scale ** 3)))
    return _poly3d("poly3d_512", n, ns, 0.004 * 512 / n, 0.5, ["Sphere", "Ellipsoid", "Box"], seed, collision, lower)


CONFIGS = {"cylinder2d": cylinder2d, "sedimentation2d": sedimentation2d, "poly3d_256": poly3d_256,
           "poly3d_512": poly3d_512}
