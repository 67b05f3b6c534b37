"""Host-side construction (shape / motion / forcer / material lowering and the solidDict front end), CPU only."""
import math

import numpy as np
import pytest

from oracle.oracle import make_shape as oracle_shape, quat_from_euler_deg as oracle_quat
from sdfibm_gb300 import abi
from sdfibm_gb300.host import HostError, make_shape, make_solid, mask_motion, parse_soliddict, quat_from_euler_deg

SHAPES = [("Circle", dict(radius=0.3)), ("Sphere", dict(radius=0.01)), ("Ellipse", dict(radiusa=0.3, radiusb=0.15)),
          ("Ellipsoid", dict(radiusa=0.1, radiusb=0.2, radiusc=0.3)), ("Box", dict(radiusa=0.1, radiusb=0.2, radiusc=0.3)),
          ("Rectangle", dict(radiusa=0.1, radiusb=0.2)), ("Plane", {}),
          ("Circle_Tail", dict(radius=0.2, ratio=2, thickness=0.05)),
          ("Circle_TwoTail", dict(radius=0.2, ratio=2, thickness=0.05))]


@pytest.mark.parametrize("name,kw", SHAPES)
def test_shape_lowering_matches_oracle_bitwise(cuda_lib, name, kw):
    a = make_shape(name, com=(0.01, 0.02, 0.03), **kw)
    b = oracle_shape(abi.SHAPE_NAMES[name], list(kw.values()), (0.01, 0.02, 0.03))
    assert bytes(a) == bytes(b)


def test_reference_shape_quirks(cuda_lib):
    assert list(make_shape("Ellipsoid", com=(1, 2, 3), radiusa=1, radiusb=1, radiusc=1).com) == [0, 0, 0]
    assert make_shape("Box", radiusa=1, radiusb=2, radiusc=3).radiusB == 3  # not a bound of the box
    assert [make_shape(n, **kw).collision_id for n, kw in SHAPES] == [1, 2, 0, 0, 0, 0, 0, 0, 0]
    tt = make_shape("Circle_TwoTail", radius=0.2, ratio=2, thickness=0.05)
    assert tt.p[2] == 0.025 and tt.radiusB == 2 * (3 * 0.5 * 0.2)


@pytest.mark.parametrize("e", [(0, 0, 0), (0, 0, -45), (10, 20, 30), (90, -90, 180)])
def test_euler_quaternion(cuda_lib, e):
    q = quat_from_euler_deg(e)
    assert np.array_equal(q, oracle_quat(e))
    assert abs(np.linalg.norm(q) - 1) < 1e-15
    # quaternion(XYZ): rotation about x, then y, then z composed as qx*qy*qz; check the rotation of e_x
    ax, ay, az = np.radians(e)
    Rx = np.array([[1, 0, 0], [0, math.cos(ax), -math.sin(ax)], [0, math.sin(ax), math.cos(ax)]])
    Ry = np.array([[math.cos(ay), 0, math.sin(ay)], [0, 1, 0], [-math.sin(ay), 0, math.cos(ay)]])
    Rz = np.array([[math.cos(az), -math.sin(az), 0], [math.sin(az), math.cos(az), 0], [0, 0, 1]])
    w, x, y, z = q
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    assert np.allclose(R, Rx @ Ry @ Rz, atol=1e-14)


def test_material_lowering(cuda_lib):
    sh = make_shape("Sphere", radius=0.5)
    d = make_solid(3, sh, 2.0, (1, 2, 3), (0, 0, 90), vel=(1, 0, 0), omega=(0, 0, 2), motion=mask_motion("b110001"))
    assert d.id == 3 and d.mass == sh.volume * 2.0 and d.mass_inv == sh.volume_inv / 2.0
    assert list(d.moi_inv) == [v / 2.0 for v in sh.moi_inv]
    assert list(d.motion_p)[:6] == [1, 1, 0, 0, 0, 1] and d.motion_type == abi.MOTION_01MASK


DICT = """
FoamFile { version 2.0; format ascii; class dictionary; object solidDict; }
// comment
meta { on_fluid 1; on_twod 1; gravity (0.0 -10.0 0.0); }
shapes
{
    shape1 { name circle1; type Circle; radius 0.15; }
    shape2 { name plane1; type Plane; }
    shape3 { name tail; type Circle_Tail; radius 0.1; ratio 2; thickness 0.02; com (0.01 0 0); }
}
forces { f1 { name spring1; type Spring; pivot (0 1 0); k 10; l 0.5; } }
materials { material1 { name mat1; type General; rho 3.0; } }
motions
{
    motion1 { name free1; type Motion01Mask; mask b111111; }
    motion2 { name rot; type Motion000002; period 2; }
}
solids
{
    solid1 { shp_name circle1; mot_name free1; mat_name mat1; pos (-1.8 4.2 0.0); vel (0.5 0.0 0.0); euler (0 0 30); }
    solid2 { shp_name tail; mot_name rot; mat_name mat1; pos (1 2 0); for_name spring1; }
    solid3 { shp_name plane1; mot_name free; mat_name mat1; pos (0 0 0); }
}
planes {}
"""


def test_soliddict_front_end(cuda_lib):
    solids, opt, twod = parse_soliddict(DICT, rho_f=1.5)
    assert twod == 1 and len(solids) == 3
    assert opt.rho_f == 1.5 and list(opt.gravity) == [0.0, -10.0, 0.0]
    s0, s1, s2 = solids
    assert s0.shape.type == abi.SHAPE_CIRCLE and s0.rho == 3.0 and list(s0.vel) == [0.5, 0, 0]
    assert np.array_equal(np.array(s0.quat), quat_from_euler_deg((0, 0, 30)))
    assert s1.motion_type == abi.MOTION_000002 and s1.motion_p[1] == 2 * math.pi / 2
    assert s1.forcer_type == abi.FORCER_SPRING and list(s1.forcer_p)[:5] == [0, 1, 0, 10, 0.5]
    assert list(s1.shape.com) == [0.01, 0, 0]
    assert s2.shape.type == abi.SHAPE_PLANE and s2.motion_type == abi.MOTION_FREE
    _, opt0, _ = parse_soliddict(DICT.replace("on_fluid 1", "on_fluid 0"), rho_f=1.5)
    assert opt0.rho_f == 0.0


@pytest.mark.parametrize("bad,msg", [
    ("mask b111111;", "mask b11111;"), ("pos (1 2 0);", "pos (1 2 0.5);"), ("type Circle;", "type Hexagon;"),
    ("for_name spring1;", "for_name nope;"), ("type General;", "type Steel;")])
def test_soliddict_errors(cuda_lib, bad, msg):
    with pytest.raises(HostError):
        parse_soliddict(DICT.replace(bad, msg), rho_f=1.0)


def test_unknown_motion_name_is_free(cuda_lib):
    # m_libmotion[name] of an unknown name yields a null motion (solidcloud.cpp:185-186)
    solids, _, _ = parse_soliddict(DICT.replace("mot_name rot;", "mot_name nothing;"), rho_f=1.0)
    assert solids[1].motion_type == abi.MOTION_FREE


def test_repeated_names(cuda_lib):
    """Shapes and forcers come from EntityLibrary (emplace: the first of a repeated name stays,
    src/entitylibrary.h:22); motions and materials are assigned into a map (the last stays, solidcloud.cpp:116, 137)."""
    text = DICT.replace("shape3 {", "shape4 { name circle1; type Circle; radius 0.9; }\n    shape3 {").replace(
        "material1 { name mat1; type General; rho 3.0; }",
        "material1 { name mat1; type General; rho 3.0; } material2 { name mat1; type General; rho 5.0; }")
    solids, _, _ = parse_soliddict(text, rho_f=1.0)
    assert solids[0].shape.radiusB == 0.15   # first circle1
    assert solids[0].rho == 5.0              # last mat1
