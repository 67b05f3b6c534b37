"""Host-side construction of solids (the reference's factories and Solid setters), through the C++ lowering in
libsdfibm_cuda.so (include/sdfibm_host.h).  Mirrors the reference's object model:

    make_shape("Sphere", radius=0.01)                ShapeFactory / IShape constructors
    make_solid(i, shape, rho, pos, euler_deg, ...)   Solid + IMaterial (Solid::setMaterial, setOrientation)
    parse_soliddict(text, rho_f)                     SolidCloud::initFromDictionary
    format_state(time, states, twod), StateFile      SolidCloud::saveState (cloud.out, meanfield.out)
    format_mean_field(means)                         SolidCloud::writeMeanField
    write_restart(dict_text, states, twod)           SolidCloud::saveRestart (restart solidDict)
    soliddict_lookup(text, "meta/writeFrequency")    dictionary::lookupOrDefault
"""
import ctypes as C

import numpy as np

from . import abi
from ._lib import load

_SHAPE_PARAMS = {
    abi.SHAPE_CIRCLE: ("radius",), abi.SHAPE_SPHERE: ("radius",), abi.SHAPE_ELLIPSE: ("radiusa", "radiusb"),
    abi.SHAPE_ELLIPSOID: ("radiusa", "radiusb", "radiusc"), abi.SHAPE_RECTANGLE: ("radiusa", "radiusb"),
    abi.SHAPE_BOX: ("radiusa", "radiusb", "radiusc"), abi.SHAPE_PLANE: (),
    abi.SHAPE_CIRCLE_TAIL: ("radius", "ratio", "thickness"), abi.SHAPE_CIRCLE_TWOTAIL: ("radius", "ratio", "thickness"),
}
MOTION_NAMES = {
    "free": abi.MOTION_FREE, "Motion000002": abi.MOTION_000002, "Motion110002": abi.MOTION_110002,
    "Motion222000": abi.MOTION_222000, "MotionSineDirectional": abi.MOTION_SINEDIRECTIONAL,
    "Motion01Mask": abi.MOTION_01MASK, "MotionRotor": abi.MOTION_ROTOR, "MotionOpenClose": abi.MOTION_OPENCLOSE,
}


class HostError(ValueError):
    pass


def _arr(vals, n=8):
    a = np.zeros(n, dtype=np.float64)
    a[:len(vals)] = vals
    return a


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def make_shape(type_name, com=(0.0, 0.0, 0.0), **params):
    t = abi.SHAPE_NAMES[type_name] if isinstance(type_name, str) else int(type_name)
    raw = _arr([float(params[k]) for k in _SHAPE_PARAMS[t]])
    c = _arr(com, 3)
    s = abi.ShapeDesc()
    if load().sdfibm_host_make_shape(t, _p(raw), _p(c), C.byref(s)) != abi.OK:
        raise HostError("cannot create shape %s with %s" % (type_name, params))
    return s


def make_motion(type_name, *raw):
    t = MOTION_NAMES[type_name]
    r = _arr(raw)
    p = np.zeros(8)
    if load().sdfibm_host_make_motion(t, _p(r), _p(p)) != abi.OK:
        raise HostError("bad motion %s" % type_name)
    return t, p


def mask_motion(mask):
    """Motion01Mask from its 'b######' word (motion01mask.h:21-48)."""
    if not (isinstance(mask, str) and len(mask) == 7 and mask[0] == "b" and set(mask[1:]) <= {"0", "1"}):
        raise HostError("bad mask %r" % (mask,))
    return make_motion("Motion01Mask", *[float(ch) for ch in mask[1:]])


def make_forcer(type_name, *raw):
    t = {"Constant": abi.FORCER_CONSTANT, "Spring": abi.FORCER_SPRING, "Magnetic": abi.FORCER_MAGNETIC}[type_name]
    r = _arr(raw)
    p = np.zeros(8)
    if load().sdfibm_host_make_forcer(t, _p(r), _p(p)) != abi.OK:
        raise HostError("bad forcer %s" % type_name)
    return t, p


def quat_from_euler_deg(euler):
    e = _arr(euler, 3)
    q = np.zeros(4)
    load().sdfibm_host_quat_from_euler_deg(_p(e), _p(q))
    return q


def make_solid(sid, shape, rho, pos, euler_deg=(0, 0, 0), vel=(0, 0, 0), omega=(0, 0, 0), motion=None,
               forcer=None):
    mt, mp = motion if motion is not None else (abi.MOTION_FREE, np.zeros(8))
    ft, fp = forcer if forcer is not None else (abi.FORCER_NONE, np.zeros(8))
    d = abi.SolidDesc()
    pos, eu, v, om = _arr(pos, 3), _arr(euler_deg, 3), _arr(vel, 3), _arr(omega, 3)
    mp, fp = np.ascontiguousarray(mp, np.float64), np.ascontiguousarray(fp, np.float64)
    rc = load().sdfibm_host_make_solid(int(sid), C.byref(shape), float(rho), int(mt), _p(mp), int(ft), _p(fp),
                                       _p(pos), _p(eu), _p(v), _p(om), C.byref(d))
    if rc != abi.OK:
        raise HostError("cannot create solid %d" % sid)
    return d


def parse_soliddict(text, rho_f=1.0, capacity=1 << 20):
    """SolidCloud::initFromDictionary: returns (solids, options, on_twod)."""
    L = load()
    n = C.c_int32(0)
    tw = C.c_int32(0)
    opt = abi.Options()
    msg = C.create_string_buffer(512)
    rc = L.sdfibm_host_parse_soliddict(text.encode(), float(rho_f), None, 0, C.byref(n), C.byref(opt), C.byref(tw),
                                       msg, 512)
    if rc != abi.OK and n.value == 0:
        raise HostError(msg.value.decode())
    arr = (abi.SolidDesc * max(1, n.value))()
    rc = L.sdfibm_host_parse_soliddict(text.encode(), float(rho_f), arr, n.value, C.byref(n), C.byref(opt),
                                       C.byref(tw), msg, 512)
    if rc != abi.OK:
        raise HostError(msg.value.decode())
    return list(arr)[:n.value], opt, tw.value


def euler_from_quat(quat_wxyz):
    """quaternion::eulerAngles(quaternion::XYZ): radians (a, b, c) with q = qx(a) qy(b) qz(c)."""
    q = np.ascontiguousarray(quat_wxyz, dtype=np.float64)
    e = np.zeros(3)
    load().sdfibm_host_euler_from_quat(_p(q), _p(e))
    return e


def _state_array(states):
    return (abi.SolidState * max(1, len(states)))(*states)


def _text(call):
    """Runs a text-producing entry point twice: once to measure, once into a buffer of that size."""
    n = C.c_int64(0)
    rc = call(None, 0, C.byref(n))
    if rc != abi.OK:
        return rc, None
    buf = C.create_string_buffer(n.value + 1)
    rc = call(buf, n.value + 1, C.byref(n))
    return rc, buf.raw[:n.value].decode()


def format_state(time, states, twod):
    """The cloud.out records of one SolidCloud::saveState (src/solidcloud.cpp:595-614): a line per solid."""
    arr = _state_array(states)
    rc, text = _text(lambda b, cap, n: load().sdfibm_host_format_state(float(time), int(bool(twod)), arr,
                                                                         len(states), b, cap, n))
    if rc != abi.OK:
        raise HostError("format_state failed (status %d)" % rc)
    return text


def format_mean_field(means):
    """The meanfield.out line of one SolidCloud::writeMeanField (src/solidcloud.cpp:303-313)."""
    m = np.ascontiguousarray(means, dtype=np.float64).reshape(-1, 3)
    rc, text = _text(lambda b, cap, n: load().sdfibm_host_format_mean_field(_p(m), len(m), b, cap, n))
    if rc != abi.OK:
        raise HostError("format_mean_field failed (status %d)" % rc)
    return text


def write_restart(dict_text, states, twod, precision=6, stamp=None):
    """SolidCloud::saveRestart (src/solidcloud.cpp:616-665): the solidDict text updated to the solids' states."""
    arr = _state_array(states)
    msg = C.create_string_buffer(512)
    st = stamp.encode() if stamp is not None else None
    rc, text = _text(lambda b, cap, n: load().sdfibm_host_write_restart(
        dict_text.encode(), arr, len(states), int(bool(twod)), int(precision), st, b, cap, n, msg, 512))
    if rc != abi.OK:
        raise HostError(msg.value.decode() or "write_restart failed (status %d)" % rc)
    return text


def soliddict_lookup(text, path, default=None):
    """The value of one solidDict entry ("meta/writeFrequency"), as text; default when the entry is absent."""
    L = load()
    n = C.c_int64(0)
    if L.sdfibm_host_soliddict_lookup(text.encode(), path.encode(), None, 0, C.byref(n)) != abi.OK:
        raise HostError("cannot look up %s" % path)
    if n.value < 0:
        return default
    buf = C.create_string_buffer(n.value + 1)
    if L.sdfibm_host_soliddict_lookup(text.encode(), path.encode(), buf, n.value + 1, C.byref(n)) != abi.OK:
        raise HostError("cannot look up %s" % path)
    return buf.raw[:n.value].decode()


def soliddict_shape(text, name):
    """The shape named `name` in a solidDict's shapes library (e.g. the meta.sampler shape)."""
    sh = abi.ShapeDesc()
    msg = C.create_string_buffer(512)
    if load().sdfibm_host_soliddict_shape(text.encode(), name.encode(), C.byref(sh), msg, 512) != abi.OK:
        raise HostError(msg.value.decode())
    return sh


class StateFile:
    """cloud.out (and meanfield.out) as SolidCloud keeps them: opened (truncated) at construction
    (src/solidcloud.cpp:29-33, 234-236); every saveState call (src/solidcloud.cpp:578-593) appends one block of records
    when its call counter is a multiple of meta.writeFrequency (default 1), and a mean-field line on every call when
    meta.on_meanfield is present (mean_field_path), then flushes."""

    def __init__(self, path="cloud.out", twod=False, write_frequency=1, mean_field_path=None):
        if int(write_frequency) < 1:
            raise HostError("writeFrequency must be positive")
        self.f = open(path, "w")
        self.mf = open(mean_field_path, "w") if mean_field_path else None
        self.twod = bool(twod)
        self.write_frequency = int(write_frequency)
        self.counter = 0

    @property
    def keeps_mean_field(self):
        return self.mf is not None

    def save(self, time, states, mean_field=None):
        if self.counter % self.write_frequency == 0:
            self.f.write(format_state(time, states, self.twod))
            self.f.flush()
        if self.mf is not None and mean_field is not None:
            self.mf.write(format_mean_field(mean_field))
            self.mf.flush()
        self.counter += 1

    def close(self):
        self.f.close()
        if self.mf is not None:
            self.mf.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
