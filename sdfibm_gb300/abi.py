"""ctypes mirror of include/sdfibm_cuda.h (descriptor structs, enums, status codes).

The layouts here must match the C header field for field; ``tests/test_abi_layout.py`` checks the sizes
against the compiled library's own ``sizeof`` answers.
"""
import ctypes as C

ABI_VERSION = 1

OK, ERR_ARG, ERR_CAPACITY, ERR_CUDA, ERR_TIMEOUT, ERR_STATE = range(6)

SHAPE_CIRCLE, SHAPE_SPHERE, SHAPE_ELLIPSE, SHAPE_ELLIPSOID, SHAPE_RECTANGLE, SHAPE_BOX, SHAPE_PLANE, \
    SHAPE_CIRCLE_TAIL, SHAPE_CIRCLE_TWOTAIL = range(1, 10)
SHAPE_NAMES = {
    "Circle": SHAPE_CIRCLE, "Sphere": SHAPE_SPHERE, "Ellipse": SHAPE_ELLIPSE, "Ellipsoid": SHAPE_ELLIPSOID,
    "Rectangle": SHAPE_RECTANGLE, "Box": SHAPE_BOX, "Plane": SHAPE_PLANE, "Circle_Tail": SHAPE_CIRCLE_TAIL,
    "Circle_TwoTail": SHAPE_CIRCLE_TWOTAIL,
}

MOTION_FREE, MOTION_000002, MOTION_110002, MOTION_222000, MOTION_SINEDIRECTIONAL, MOTION_01MASK, \
    MOTION_ROTOR, MOTION_OPENCLOSE = range(8)
FORCER_NONE, FORCER_CONSTANT, FORCER_SPRING, FORCER_MAGNETIC = range(4)
COLLISION_OFF, COLLISION_REFERENCE, COLLISION_SPHERES = range(3)
FRACTION_REFGEO, FRACTION_SUBSAMPLE, FRACTION_LEARNED = range(3)

# cell types written into Ct / returned by the touched-list query (CellEnumerator::CELL_TYPE)
ALL_INSIDE, CENTER_INSIDE, CENTER_OUTSIDE = 1, 2, 3


class MeshDesc(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("twod", C.c_int32),
                ("origin", C.c_double * 3), ("h", C.c_double * 3)]


class ShapeDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("collision_id", C.c_int32), ("p", C.c_double * 8), ("com", C.c_double * 3),
                ("radiusB", C.c_double), ("volume", C.c_double), ("volume_inv", C.c_double),
                ("moi_inv", C.c_double * 9)]


class SolidDesc(C.Structure):
    _fields_ = [("id", C.c_int32), ("motion_type", C.c_int32), ("forcer_type", C.c_int32), ("pad0", C.c_int32),
                ("shape", ShapeDesc), ("motion_p", C.c_double * 8), ("forcer_p", C.c_double * 8),
                ("rho", C.c_double), ("mass", C.c_double), ("mass_inv", C.c_double), ("moi_inv", C.c_double * 9),
                ("pos", C.c_double * 3), ("quat", C.c_double * 4), ("vel", C.c_double * 3),
                ("omega", C.c_double * 3)]


class SolidState(C.Structure):
    _fields_ = [(n, C.c_double * k) for n, k in [
        ("pos", 3), ("quat", 4), ("vel", 3), ("omega", 3), ("force", 3), ("torque", 3),
        ("fluid_force", 3), ("fluid_torque", 3), ("fluid_force_old", 3), ("fluid_torque_old", 3),
        ("forcer_force", 3), ("forcer_torque", 3), ("forcer_force_old", 3), ("forcer_torque_old", 3)]] + \
        [("first_fluid_step", C.c_int32), ("first_forcer_step", C.c_int32)]


class Options(C.Structure):
    _fields_ = [("rho_f", C.c_double), ("gravity", C.c_double * 3), ("collision_mode", C.c_int32),
                ("n_subiter", C.c_int32), ("fraction_method", C.c_int32), ("subsample_n", C.c_int32),
                ("dense_reset", C.c_int32), ("exact_forcing", C.c_int32), ("tile_cells", C.c_int32),
                ("timing", C.c_int32), ("learned_fallback_n", C.c_int32), ("graphs", C.c_int32),
                ("recheck_cap", C.c_int32), ("reserved", C.c_int32 * 3)]


class MlpDataDesc(C.Structure):
    """sdfibm_mlp_data_desc (include/sdfibm_mlp.h)."""
    _fields_ = [("hr_min", C.c_double), ("hr_max", C.c_double), ("families", C.c_int32), ("n_sub", C.c_int32),
                ("z_axis_frac", C.c_double)]


class MlpTrainDesc(C.Structure):
    """sdfibm_mlp_train_desc (include/sdfibm_mlp.h)."""
    _fields_ = [("epochs", C.c_int32), ("batch", C.c_int32), ("lr", C.c_float), ("lr_final_frac", C.c_float),
                ("warmup_steps", C.c_int32), ("reserved", C.c_int32)]


MLP_NIN = 16
MLP_NFEAT = 17  # rows of a feature buffer: the 16 network inputs, then the prior logit
MLP_NPARAM = 5313
MLP_SPHERE, MLP_ELLIPSOID, MLP_BOX, MLP_PLANE, MLP_CYLINDER, MLP_ELLIPTIC_CYL = 1, 2, 4, 8, 16, 32


def mesh_desc(n, origin, h, twod=0):
    m = MeshDesc()
    m.nx, m.ny, m.nz = (int(v) for v in n)
    m.twod = int(twod)
    for a in range(3):
        m.origin[a] = float(origin[a])
        m.h[a] = float(h[a])
    return m


def options(**kw):
    o = Options()
    o.rho_f = 1.0
    o.collision_mode = COLLISION_OFF
    o.fraction_method = FRACTION_REFGEO
    o.subsample_n = 10
    o.exact_forcing = 1
    for k, v in kw.items():
        if k == "gravity":
            for a in range(3):
                o.gravity[a] = float(v[a])
        else:
            setattr(o, k, v)
    return o


def state_to_dict(st):
    return {f: list(getattr(st, f)) if not f.startswith("first") else int(getattr(st, f))
            for f, _ in SolidState._fields_}
