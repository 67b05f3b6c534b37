"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle (oracle/oracle.cpp).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference legs may import this module; the
product (sdfibm_gb300) never does.  The oracle restates sdfibm's coupling path; see oracle.cpp's header for the
reference files it follows.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from sdfibm_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = os.path.join(_HERE, "liboracle.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(_HERE, f) for f in ("oracle.cpp", "oracle_math.h", "oracle_mesh.h", "oracle_shapes.h")]
    newest = max(os.path.getmtime(s) for s in srcs)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < newest:
        subprocess.check_call(["sh", os.path.join(_HERE, "build.sh")])
    return _LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB)
        vp = C.c_void_p
        L.oracle_create_uniform.restype = vp
        L.oracle_create_uniform.argtypes = [C.POINTER(abi.MeshDesc), C.POINTER(abi.SolidDesc), C.c_int,
                                            C.POINTER(abi.Options), C.c_int]
        L.oracle_create_polymesh.restype = vp
        L.oracle_create_polymesh.argtypes = [vp, C.c_int64, vp, vp, C.c_int64, vp, vp, C.c_int64, C.c_int,
                                             C.POINTER(abi.SolidDesc), C.c_int, C.POINTER(abi.Options)]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_ncells.restype = C.c_int64
        L.oracle_ncells.argtypes = [vp]
        L.oracle_interact.argtypes = [vp, C.c_double, C.c_double] + [vp] * 6
        L.oracle_last_seconds.restype = C.c_double
        L.oracle_last_seconds.argtypes = [vp]
        L.oracle_last_pairs.restype = C.c_int64
        L.oracle_last_pairs.argtypes = [vp]
        L.oracle_touched.restype = C.c_int64
        L.oracle_touched.argtypes = [vp, C.c_int, vp, vp, C.c_int64]
        L.oracle_evolve.argtypes = [vp, C.c_double, C.c_double]
        L.oracle_fix_internal.argtypes = [vp, vp, vp]
        L.oracle_get_state.argtypes = [vp, C.POINTER(abi.SolidState), C.c_int]
        L.oracle_set_state.argtypes = [vp, C.POINTER(abi.SolidState), C.c_int]
        L.oracle_cell_centre.argtypes = [vp, C.c_int64, vp]
        L.oracle_cell_fraction.restype = C.c_double
        L.oracle_cell_fraction.argtypes = [vp, C.c_int, C.c_int64, C.c_int]
        L.oracle_make_shape.argtypes = [C.c_int, vp, vp, C.POINTER(abi.ShapeDesc)]
        L.oracle_quat_from_euler.argtypes = [vp, vp]
        L.oracle_world2local.argtypes = [vp, vp, vp, vp]
        L.oracle_phi01.argtypes = [C.POINTER(abi.SolidDesc), vp]
        L.oracle_phi.restype = C.c_double
        L.oracle_phi.argtypes = [C.POINTER(abi.SolidDesc), vp]
        L.oracle_interact_threads.argtypes = [vp, C.c_double] + [vp] * 6 + [C.c_int]
        L.oracle_sample_cell.restype = C.c_int64
        L.oracle_sample_cell.argtypes = [C.POINTER(abi.ShapeDesc), vp, vp, C.c_double, C.c_int, vp]
        L.oracle_mean_field.argtypes = [vp, C.POINTER(abi.ShapeDesc), vp, vp, vp]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def make_shape(type_id, raw, com=(0.0, 0.0, 0.0)):
    r = np.zeros(8)
    r[:len(raw)] = raw
    c = np.asarray(com, dtype=np.float64)
    s = abi.ShapeDesc()
    if lib().oracle_make_shape(type_id, _p(r), _p(c), C.byref(s)) != 0:
        raise ValueError("bad shape")
    return s


def sample_cell(recipe, n_sub):
    """Recomputes one generated training cell from its FP64 recipe (the 20-value record of sdfibm_mlp_dataset):
    returns (phi / h at the cell's 5 x 5 x 5 lattice [125], inside count of the n_sub^3 lattice)."""
    r = np.asarray(recipe, dtype=np.float64)
    s = abi.ShapeDesc()
    s.type = int(r[0])
    for k in range(8):
        s.p[k] = r[1 + k]
    q = np.ascontiguousarray(r[9:13])
    o = np.ascontiguousarray(r[13:16])
    phi = np.zeros(125)
    cnt = lib().oracle_sample_cell(C.byref(s), _p(q), _p(o), float(r[16]), int(n_sub), _p(phi))
    return phi, int(cnt)


def quat_from_euler_deg(euler_deg):
    a = np.radians(np.asarray(euler_deg, dtype=np.float64))
    q = np.zeros(4)
    lib().oracle_quat_from_euler(_p(a), _p(q))
    return q


class OracleCloud:
    """SolidCloud restated in FP64 on the CPU (faithful or fast mode)."""

    def __init__(self, mesh, solids, opt, faithful=True, polymesh=None):
        L = lib()
        self.nsolids = len(solids)
        self._solids = (abi.SolidDesc * max(1, len(solids)))(*solids)
        self.mesh = mesh
        if polymesh is None:
            self.h = L.oracle_create_uniform(C.byref(mesh), self._solids, len(solids), C.byref(opt), int(faithful))
        else:
            pts, off, lab, own, nei = polymesh
            self._keep = (np.ascontiguousarray(pts, np.float64), np.ascontiguousarray(off, np.int32),
                          np.ascontiguousarray(lab, np.int32), np.ascontiguousarray(own, np.int32),
                          np.ascontiguousarray(nei, np.int32))
            p, o, la, ow, ne = self._keep
            self.h = L.oracle_create_polymesh(_p(p), len(p), _p(o), _p(la), len(o) - 1, _p(ow), _p(ne), len(ne),
                                              int(mesh.twod), self._solids, len(solids), C.byref(opt))
        if not self.h:
            raise RuntimeError("oracle create failed")
        self.N = L.oracle_ncells(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def new_fields(self):
        N = self.N
        return dict(As=np.zeros(N), Fs=np.zeros(3 * N), Ts=np.zeros(N), Ct=np.zeros(N, np.int32))

    def interact(self, time, dt, U, fields):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        FT = np.zeros(6 * self.nsolids)
        rc = lib().oracle_interact(self.h, time, dt, _p(U), _p(fields["As"]), _p(fields["Fs"]), _p(fields["Ts"]),
                                   _p(fields["Ct"]), _p(FT))
        if rc != 0:
            raise RuntimeError("oracle interact failed")
        return FT.reshape(self.nsolids, 6)

    def interact_threads(self, dt, U, fields, nthreads):
        """interact with the solids spread over nthreads host threads (CPU timing on all cores)."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        FT = np.zeros(6 * self.nsolids)
        rc = lib().oracle_interact_threads(self.h, dt, _p(U), _p(fields["As"]), _p(fields["Fs"]), _p(fields["Ts"]),
                                           _p(fields["Ct"]), _p(FT), int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle interact failed")
        return FT.reshape(self.nsolids, 6)

    def last_seconds(self):
        return lib().oracle_last_seconds(self.h)

    def last_pairs(self):
        return lib().oracle_last_pairs(self.h)

    def touched(self, s):
        n = lib().oracle_touched(self.h, s, None, None, 0)
        cells = np.zeros(max(n, 1), np.int64)
        types = np.zeros(max(n, 1), np.int8)
        lib().oracle_touched(self.h, s, _p(cells), _p(types), n)
        return cells[:n], types[:n]

    def evolve(self, time, dt):
        lib().oracle_evolve(self.h, time, dt)

    def fix_internal(self, Ct, U):
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1).copy()
        lib().oracle_fix_internal(self.h, _p(np.ascontiguousarray(Ct, np.int32)), _p(U))
        return U

    def get_state(self):
        st = (abi.SolidState * self.nsolids)()
        lib().oracle_get_state(self.h, st, self.nsolids)
        return st

    def set_state(self, st):
        """Solid states from a ctypes array or a sequence of abi.SolidState (e.g. SolidCloud.states())."""
        if not isinstance(st, C.Array):
            st = (abi.SolidState * max(1, self.nsolids))(*st)
        lib().oracle_set_state(self.h, st, self.nsolids)

    def mean_field(self, sampler, U, Ct=None):
        """SolidCloud::calcMeanField of U for every solid with the sampler shape: (S, 3).  Ct (int32, updated in
        place) receives the reference's writes for the visited cells."""
        U = np.ascontiguousarray(U, dtype=np.float64).reshape(-1)
        out = np.zeros(3 * max(1, self.nsolids))
        if Ct is not None:
            assert Ct.dtype == np.int32 and Ct.flags.c_contiguous
        lib().oracle_mean_field(self.h, C.byref(sampler), _p(U), _p(Ct) if Ct is not None else None, _p(out))
        return out[:3 * self.nsolids].reshape(self.nsolids, 3)

    def cell_fraction(self, s, c, method):
        return lib().oracle_cell_fraction(self.h, s, c, method)


class Lowering:
    """The solid construction of the reference (shape constructors, quaternion(XYZ, euler), Solid::setMaterial)
    through the oracle's own restatement, with the call signatures of sdfibm_gb300.host.  The CPU reference leg of
    the benchmark builds its workload with this, so that it maps no library of the product."""

    SHAPE_PARAMS = {
        abi.SHAPE_CIRCLE: ("radius",), abi.SHAPE_SPHERE: ("radius",), abi.SHAPE_ELLIPSE: ("radiusa", "radiusb"),
        abi.SHAPE_ELLIPSOID: ("radiusa", "radiusb", "radiusc"), abi.SHAPE_RECTANGLE: ("radiusa", "radiusb"),
        abi.SHAPE_BOX: ("radiusa", "radiusb", "radiusc"), abi.SHAPE_PLANE: (),
        abi.SHAPE_CIRCLE_TAIL: ("radius", "ratio", "thickness"),
        abi.SHAPE_CIRCLE_TWOTAIL: ("radius", "ratio", "thickness"),
    }

    @staticmethod
    def make_shape(type_name, com=(0.0, 0.0, 0.0), **params):
        t = abi.SHAPE_NAMES[type_name] if isinstance(type_name, str) else int(type_name)
        return make_shape(t, [float(params[k]) for k in Lowering.SHAPE_PARAMS[t]], com)

    @staticmethod
    def mask_motion(mask):
        """Motion01Mask from its 'b######' word (motion01mask.h:21-48)."""
        if not (isinstance(mask, str) and len(mask) == 7 and mask[0] == "b" and set(mask[1:]) <= {"0", "1"}):
            raise ValueError("bad mask %r" % (mask,))
        p = np.zeros(8)
        p[:6] = [float(ch) for ch in mask[1:]]
        return abi.MOTION_01MASK, p

    @staticmethod
    def make_solid(sid, shape, rho, pos, euler_deg=(0, 0, 0), vel=(0, 0, 0), omega=(0, 0, 0), motion=None,
                   forcer=None):
        """Solid + IMaterial: Solid::setMaterial (solid.h:95-103), setOrientation from XYZ Euler angles."""
        mt, mp = motion if motion is not None else (abi.MOTION_FREE, np.zeros(8))
        ft, fp = forcer if forcer is not None else (abi.FORCER_NONE, np.zeros(8))
        d = abi.SolidDesc()
        d.id = int(sid)
        d.shape = shape
        d.motion_type, d.forcer_type = int(mt), int(ft)
        for i in range(8):
            d.motion_p[i] = float(mp[i])
            d.forcer_p[i] = float(fp[i])
        d.rho = float(rho)
        d.mass = shape.volume * rho
        d.mass_inv = shape.volume_inv / rho
        for i in range(9):
            d.moi_inv[i] = shape.moi_inv[i] / rho
        e = [float(x) for x in euler_deg] + [0.0] * (3 - len(euler_deg))
        q = np.zeros(4)
        a = np.array([e[0] * np.pi / 180.0, e[1] * np.pi / 180.0, e[2] * np.pi / 180.0])
        lib().oracle_quat_from_euler(_p(a), _p(q))
        for i in range(3):
            d.pos[i] = float(pos[i])
            d.vel[i] = float(vel[i])
            d.omega[i] = float(omega[i])
        for i in range(4):
            d.quat[i] = float(q[i])
        return d
