"""The reference's two output formats, on CPU: the cloud.out records of SolidCloud::saveState and the restart
solidDict of SolidCloud::saveRestart, and the quaternion -> XYZ Euler angle conversion both use."""
import ctypes as C
import re

import numpy as np
import pytest

from sdfibm_gb300 import abi
from sdfibm_gb300.host import (HostError, StateFile, euler_from_quat, format_state, make_shape, make_solid,
                               parse_soliddict, quat_from_euler_deg, write_restart)

DICT_3D = """/* a solidDict in the layout of the reference's examples */
FoamFile
{
    version     2.0;
    format      ascii;
    class       dictionary;
    object      solids;
}
meta
{
    on_fluid 1;
    on_twod  0;
    gravity  (0.0 -9.81 0.0);
    writeFrequency 2;
}
shapes
{
    s1 { name ball; type Sphere; radius 0.05; }
    s2 { name brick; type Box; radiusa 0.1; radiusb 0.05; radiusc 0.02; com (0 0 0.01); }
}
materials
{
    m1 { name heavy; type General; rho 2.5; }
}
motions
{
    f1 { name pinned; type Motion01Mask; mask b000111; }
}
solids
{
    a { shp_name ball;  mot_name free;   mat_name heavy; pos (0.1 0.2 0.3); vel (1 0 0); }
    b { shp_name brick; mot_name pinned; mat_name heavy; pos (0.5 0.5 0.5); euler (10 20 30); omega (0 0 1);
        note "kept as written"; }
}
"""

DICT_2D = DICT_3D.replace("on_twod  0", "on_twod  1").replace("(0.1 0.2 0.3)", "(0.1 0.2 0)").replace(
    "(0.5 0.5 0.5)", "(0.5 0.5 0)").replace("Sphere", "Circle").replace(
    "type Box; radiusa 0.1; radiusb 0.05; radiusc 0.02; com (0 0 0.01);", "type Ellipse; radiusa 0.1; radiusb 0.05;")


def _states(n, seed, twod=False):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        s = abi.SolidState()
        for f, vals in (("pos", rng.uniform(-1, 1, 3)), ("vel", rng.normal(0, 1, 3)), ("omega", rng.normal(0, 3, 3)),
                        ("force", rng.normal(0, 1e-3, 3)), ("torque", rng.normal(0, 1e-5, 3))):
            for a in range(3):
                getattr(s, f)[a] = float(vals[a])
        e = (rng.uniform(-170, 170), rng.uniform(-85, 85), rng.uniform(-170, 170))
        if twod:
            e = (0.0, 0.0, e[2])
        q = quat_from_euler_deg(e)
        for a in range(4):
            s.quat[a] = float(q[a])
        out.append(s)
    return out


def _rot(axis, t):
    c, s = np.cos(t), np.sin(t)
    i, j = [(1, 2), (2, 0), (0, 1)][axis]
    R = np.eye(3)
    R[i, i] = R[j, j] = c
    R[i, j], R[j, i] = -s, s
    return R


def _quat_matrix(q):
    w, v = q[0], np.asarray(q[1:])
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return (w * w - v @ v) * np.eye(3) + 2 * np.outer(v, v) + 2 * w * K


@pytest.mark.parametrize("seed", range(4))
def test_euler_inverts_quat_from_euler(cuda_lib, seed):
    rng = np.random.default_rng(seed)
    for _ in range(200):
        e = np.array([rng.uniform(-179, 179), rng.uniform(-89, 89), rng.uniform(-179, 179)])
        back = euler_from_quat(quat_from_euler_deg(e)) * 180.0 / np.pi
        assert np.abs(back - e).max() < 1e-9
        # the convention, independently: q = qx(a) qy(b) qz(c) rotates as Rx(a) Ry(b) Rz(c)
        a, b, c = np.radians(e)
        R = _rot(0, a) @ _rot(1, b) @ _rot(2, c)
        assert np.abs(_quat_matrix(quat_from_euler_deg(e)) - R).max() < 1e-14


def test_euler_known_values(cuda_lib):
    assert np.allclose(euler_from_quat([1, 0, 0, 0]), 0)
    assert np.allclose(euler_from_quat(quat_from_euler_deg((0, 0, -45))), (0, 0, -np.pi / 4))
    # -q is the same rotation
    q = quat_from_euler_deg((30, -40, 50))
    assert np.allclose(euler_from_quat(-q), euler_from_quat(q), atol=1e-14)


@pytest.mark.parametrize("twod", [False, True])
def test_state_records(cuda_lib, twod):
    st = _states(5, 3, twod)
    t = 0.0123456789
    text = format_state(t, st, twod)
    lines = text.split("\n")
    assert lines[-1] == "" and len(lines) == 6
    for s, line in zip(st, lines):
        e = euler_from_quat(list(s.quat))
        if twod:
            vals = [t, s.pos[0], s.pos[1], s.vel[0], s.vel[1], s.force[0], s.force[1], e[2], s.omega[2], s.torque[2]]
        else:
            vals = [t] + [g[a] for g in (s.pos, s.vel, s.force, e, s.omega, s.torque) for a in range(3)]
        # std::scientific with the stream's default precision 6
        assert line == " ".join("%.6e" % v for v in vals)
        assert len(line.split(" ")) == (10 if twod else 19)


def test_state_file_frequency(cuda_lib, tmp_path):
    st = _states(3, 4)
    with StateFile(str(tmp_path / "cloud.out"), twod=False, write_frequency=2) as f:
        for k in range(5):
            f.save(0.1 * k, st)
    assert f.f.closed
    rows = [l.split() for l in open(tmp_path / "cloud.out").read().splitlines()]
    # calls 0, 2 and 4 write: three blocks of three solids
    assert len(rows) == 9
    assert [r[0] for r in rows[::3]] == ["%.6e" % v for v in (0.0, 0.2, 0.4)]
    with pytest.raises(HostError):
        StateFile(str(tmp_path / "x"), write_frequency=0)


def test_empty_state_block(cuda_lib):
    assert format_state(1.0, [], False) == ""


@pytest.mark.parametrize("twod", [False, True])
def test_restart_round_trip(cuda_lib, twod):
    src = DICT_2D if twod else DICT_3D
    solids, opt, tw = parse_soliddict(src, 1.0)
    assert tw == int(twod) and len(solids) == 2
    st = _states(2, 7, twod)
    text = write_restart(src, st, twod, precision=17, stamp="26/01/02 03:04:05")
    again, opt2, tw2 = parse_soliddict(text, 1.0)
    assert tw2 == tw and list(opt2.gravity) == list(opt.gravity)
    for d0, d, s in zip(solids, again, st):
        pos, vel, om = list(s.pos), list(s.vel), list(s.omega)
        if twod:
            pos[2] = vel[2] = om[0] = om[1] = 0.0
        assert list(d.pos) == pos and list(d.vel) == vel and list(d.omega) == om
        q0, q1 = np.array(list(s.quat)), np.array(list(d.quat))
        assert min(np.abs(q1 - q0).max(), np.abs(q1 + q0).max()) < 1e-14
        # shape, material and motion carry over unchanged
        assert bytes(d.shape) == bytes(d0.shape) and d.motion_type == d0.motion_type and d.mass == d0.mass


def test_restart_layout(cuda_lib):
    st = _states(2, 8)
    text = write_restart(DICT_3D, st, False, precision=6, stamp="26/01/02 03:04:05")
    lines = text.split("\n")
    # the solidDict header, the input's own FoamFile entry dropped, entries written right after the banner line
    assert lines[0].startswith("/*---") and "object      solidDict;" in text and "object      solids;" not in text
    body = text[text.index("// * *"):].split("\n", 1)[1]
    assert body.startswith("meta\n{\n    on_fluid        1;\n")
    # keywords padded to 16 columns, tokens re-written with 6 significant digits, one empty line between the top-level
    # entries, none inside
    assert "    gravity         ( 0 -9.81 0 );\n    writeFrequency  2;\n}\n\nshapes\n{\n    s1\n    {\n" in body
    assert "        com             ( 0 0 0.01 );\n" in body
    assert '        note            "kept as written";\n' in body
    # pos/vel/euler replaced in place, omega appended to the solid that had none
    a = body[body.index("    a\n"):body.index("    b\n")]
    keys = re.findall(r"^        (\w+) ", a, flags=re.M)
    assert keys == ["shp_name", "mot_name", "mat_name", "pos", "vel", "euler", "omega"]
    e = euler_from_quat(list(st[0].quat)) * 180.0 / np.pi
    assert "        euler           ( %s );\n" % " ".join("%.6g" % v for v in e) in a
    assert "        pos             ( %s );\n" % " ".join("%.6g" % v for v in st[0].pos) in a
    assert text.endswith("}\n\n// 26/01/02 03:04:05\n")


def test_restart_default_stamp(cuda_lib):
    text = write_restart(DICT_3D, _states(2, 9), False)
    assert re.search(r"\n// \d\d/\d\d/\d\d \d\d:\d\d:\d\d\n$", text)


def test_restart_errors(cuda_lib):
    with pytest.raises(HostError, match="2 entries, 1 states"):
        write_restart(DICT_3D, _states(1, 1), False)
    with pytest.raises(HostError, match="solids"):
        write_restart("meta { on_fluid 1; }", [], False)
    with pytest.raises(HostError, match="bad argument"):
        write_restart(DICT_3D, _states(2, 1), False, precision=40)
    # a buffer one byte short of the text and its NUL
    arr = (abi.SolidState * 2)(*_states(2, 1))
    n = C.c_int64(0)
    assert cuda_lib.sdfibm_host_format_state(0.0, 0, arr, 2, None, 0, C.byref(n)) == abi.OK
    buf = C.create_string_buffer(n.value)
    assert cuda_lib.sdfibm_host_format_state(0.0, 0, arr, 2, buf, n.value, C.byref(n)) == 2


def test_restart_of_a_real_cloud_description(cuda_lib):
    """Solids built by the host factories round-trip through the restart writer at full precision."""
    sh = make_shape("Ellipsoid", radiusa=0.2, radiusb=0.1, radiusc=0.05)
    d = make_solid(0, sh, 2.0, (0.25, -0.5, 0.125), euler_deg=(15, -30, 45), vel=(0.5, 0, -0.25), omega=(1, 2, 3))
    st = abi.SolidState()
    for f in ("pos", "vel", "omega", "quat"):
        for a in range(len(getattr(st, f))):
            getattr(st, f)[a] = getattr(d, f)[a]
    src = DICT_3D.replace("    b { shp_name brick;", "    //").replace("        note \"kept as written\"; }", "")
    text = write_restart(src, [st], False, precision=17)
    e = re.search(r"euler +\( ([^)]*) \)", text).group(1).split()
    assert np.allclose([float(v) for v in e], (15, -30, 45), atol=1e-12)


def test_soliddict_lookup(cuda_lib):
    from sdfibm_gb300.host import soliddict_lookup
    assert soliddict_lookup(DICT_3D, "meta/writeFrequency") == "2"
    assert soliddict_lookup(DICT_3D, "meta/gravity") == "( 0.0 -9.81 0.0 )"
    assert soliddict_lookup(DICT_3D, "solids/b/note") == "kept as written"
    assert soliddict_lookup(DICT_3D, "meta/sampler", "none") == "none"
    assert soliddict_lookup(DICT_3D, "nothing/here") is None
    with pytest.raises(HostError):
        soliddict_lookup(DICT_3D, "meta")
    with pytest.raises(HostError):
        soliddict_lookup("meta { on_fluid 1;", "meta/on_fluid")


def test_cloud_writers_host_logic(cuda_lib, tmp_path):
    """SolidCloud.save_state / save_restart with the device state read answered on the host."""
    from sdfibm_gb300.cloud import SolidCloud
    st = _states(2, 11)
    cloud = SolidCloud.__new__(SolidCloud)
    cloud.time = 0.25
    cloud.mesh = abi.mesh_desc((4, 4, 4), (0, 0, 0), (0.25, 0.25, 0.25), twod=0)
    cloud._sampler = None
    cloud._sampler_fields = None
    cloud.states = lambda: st
    f = StateFile(str(tmp_path / "cloud.out"), twod=False, mean_field_path=str(tmp_path / "meanfield.out"))
    cloud.save_state(f)           # no sampler: no mean-field line
    f.close()
    assert open(tmp_path / "cloud.out").read() == format_state(0.25, st, False)
    assert open(tmp_path / "meanfield.out").read() == ""
    cloud.save_restart(DICT_3D, str(tmp_path / "solidDict"), precision=17, stamp="s")
    again, _, _ = parse_soliddict(open(tmp_path / "solidDict").read(), 1.0)
    assert [list(d.pos) for d in again] == [list(s.pos) for s in st]


def test_cloud_info_host_logic(cuda_lib):
    """SolidCloud's info methods on host tensors (totalSolidVolume, isOnTwoD, operator[])."""
    torch = pytest.importorskip("torch")
    from sdfibm_gb300.cloud import SolidCloud
    cloud = SolidCloud.__new__(SolidCloud)
    cloud.mesh = abi.mesh_desc((4, 2, 1), (0, 0, -0.5), (0.5, 0.25, 1.0), twod=1)
    cloud.opt = abi.options(rho_f=0.0)
    cloud.nsolids = 2
    st = _states(2, 12)
    cloud.states = lambda: st
    As = torch.tensor([0.0, 1.0, 0.5, 0.25, 1.0, 0.0, 0.0, 1.0])
    assert cloud.total_solid_volume({"As": As}) == 3.75 * 0.125
    assert cloud.is_on_twod() and not cloud.is_on_fluid() and len(cloud) == 2
    assert list(cloud[1].pos) == list(st[1].pos)
    with pytest.raises(IndexError):
        cloud[2]


def test_soliddict_shape(cuda_lib):
    from sdfibm_gb300.host import soliddict_shape
    sh = soliddict_shape(DICT_3D, "brick")
    assert bytes(sh) == bytes(make_shape("Box", radiusa=0.1, radiusb=0.05, radiusc=0.02, com=(0, 0, 0.01)))
    with pytest.raises(HostError, match="unknown shape name"):
        soliddict_shape(DICT_3D, "nothing")
