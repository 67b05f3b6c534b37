"""The VOF initializer (tool_vof): its solidDict front end, the uniform block of a blockMeshDict, the OpenFOAM
field writer, and the phase field itself against the one the reference's tool wrote for its example case
(tool_vof/example/0/alpha.water, 200 x 200 cells on [0,4]^2: three circle-tails, three rectangles, three ellipses and
three circles in rotated poses, and two planes)."""
import os
import re

import numpy as np
import pytest

from conftest import golden
from oracle.oracle import OracleCloud
from sdfibm_gb300 import abi
from sdfibm_gb300.host import HostError, make_shape, make_solid

# the example's configuration: (shape, x, y, euler z in degrees)
EXAMPLE = [("circle_tail1", 0.5, 1.5, -45), ("circle_tail1", 0.5, 2.5, 0), ("circle_tail1", 0.5, 3.5, 45),
           ("rectangle1", 1.5, 1.5, 0), ("rectangle1", 1.5, 2.5, 30), ("rectangle1", 1.5, 3.5, 60),
           ("ellipse1", 2.5, 1.5, 0), ("ellipse1", 2.5, 2.5, 60), ("ellipse1", 2.5, 3.5, 120),
           ("circle1", 3.5, 1.0, 0), ("circle1", 3.5, 2.5, 0), ("circle1", 3.5, 3.5, 0)]
PLANES = [("plane1", 0.0, 0.0, 15), ("plane1", 0.0, 0.0, -90)]
SHAPES = {"circle1": ("Circle", dict(radius=0.3)),
          "circle_tail1": ("Circle_Tail", dict(radius=0.3, ratio=1.0, thickness=0.1)),
          "ellipse1": ("Ellipse", dict(radiusa=0.3, radiusb=0.2)),
          "rectangle1": ("Rectangle", dict(radiusa=0.3, radiusb=0.2)),
          "plane1": ("Plane", {})}


def vof_dict_text(entries=EXAMPLE, planes=PLANES, twod=1):
    out = ["FoamFile\n{\n    format ascii;\n    class dictionary;\n    object solidDict;\n}\n",
           "meta\n{\n    on_twod %d;\n}\n" % twod, "shapes\n{\n"]
    for i, (name, (typ, kw)) in enumerate(sorted(SHAPES.items())):
        body = "".join("        %s %r;\n" % (k, v) for k, v in kw.items())
        out.append("    shape%d\n    {\n        name %s;\n        type %s;\n%s    }\n" % (i, name, typ, body))
    out.append("}\n")
    for sec, lst in (("solids", entries), ("planes", planes)):
        out.append("%s\n{\n" % sec)
        for i, (name, x, y, ez) in enumerate(lst):
            out.append("    s%d\n    {\n        shp_name %s;\n        pos ( %r %r 0 );\n        euler ( 0 0 %r );\n"
                       "    }\n" % (i, name, x, y, ez))
        out.append("}\n")
    return "".join(out)


BLOCKMESH = """FoamFile { version 2.0; format ascii; class dictionary; object blockMeshDict; }
convertToMeters 1;
vertices
(
    (0 0 -0.5) (4 0 -0.5) (4 4 -0.5) (0 4 -0.5)
    (0 0 0.5) (4 0 0.5) (4 4 0.5) (0 4 0.5)
);
blocks ( hex (0 1 2 3 4 5 6 7) (200 200 1) simpleGrading (1 1 1) );
edges ( );
boundary
(
    left { type wall; faces ((0 4 7 3)); }
    right { type wall; faces ((2 6 5 1)); }
    frontAndBack { type empty; faces ((0 3 2 1) (4 5 6 7)); }
);
"""

FIELD = """/* phase field template */
FoamFile
{
    version     2.0;
    format      ascii;
    class       volScalarField;
    object      alpha.water;
}
dimensions      [0 0 0 0 0 0 0];

internalField   uniform 0;

boundaryField
{
    left { type zeroGradient; }
    right { type zeroGradient; }
    frontAndBack { type empty; }
}
"""


def example_solids():
    out = []
    for i, (name, x, y, ez) in enumerate(EXAMPLE + PLANES):
        typ, kw = SHAPES[name]
        out.append(make_solid(i, make_shape(typ, **kw), 1.0, (x, y, 0.0), (0, 0, ez)))
    return out


def read_field(data):
    """The internalField of an OpenFOAM scalar field file (ascii or binary)."""
    binary = re.search(rb"format\s+binary", data) is not None
    m = re.search(rb"internalField\s+nonuniform\s+List<scalar>\s*\n(\d+)\n\(", data)
    n = int(m.group(1))
    if binary:
        assert data[m.end() + 8 * n:m.end() + 8 * n + 1] == b")"
        return np.frombuffer(data[m.end():m.end() + 8 * n], dtype="<f8"), data[m.end() + 8 * n + 1:]
    body = data[m.end():data.index(b")", m.end())]
    return np.array([float(v) for v in body.split()]), data[data.index(b")", m.end()) + 1:]


def test_vofdict_front_end(cuda_lib):
    from sdfibm_gb300.vof import parse_vofdict
    solids, twod = parse_vofdict(vof_dict_text())
    assert twod and len(solids) == 14
    for got, want in zip(solids, example_solids()):
        assert bytes(got) == bytes(want)
    assert len(parse_vofdict(vof_dict_text(), with_planes=False)[0]) == 12
    with pytest.raises(HostError, match="z=0"):
        parse_vofdict(vof_dict_text().replace("pos ( 0.5 1.5 0 )", "pos ( 0.5 1.5 0.1 )"))
    with pytest.raises(HostError, match="unknown shape name"):
        parse_vofdict(vof_dict_text(entries=[("nothing", 1.0, 1.0, 0)]))
    # a repeated shape name keeps the last definition (map assignment), unlike the coupling's library
    text = vof_dict_text().replace("shapes\n{\n", "shapes\n{\n    first\n    {\n        name circle1;\n"
                                   "        type Circle;\n        radius 0.1;\n    }\n", 1)
    s2, _ = parse_vofdict(text)
    assert s2[9].shape.radiusB == pytest.approx(0.3)


def test_blockmesh(cuda_lib):
    from sdfibm_gb300.vof import parse_blockmesh
    m = parse_blockmesh(BLOCKMESH)
    assert (m.nx, m.ny, m.nz, m.twod) == (200, 200, 1, 1)
    assert list(m.origin) == [0.0, 0.0, -0.5] and list(m.h) == [0.02, 0.02, 1.0]
    m = parse_blockmesh(BLOCKMESH.replace("convertToMeters 1;", "convertToMeters 0.5;"))
    assert list(m.origin) == [0.0, 0.0, -0.25] and list(m.h) == [0.01, 0.01, 0.5]
    with pytest.raises(HostError, match="uniform grading"):
        parse_blockmesh(BLOCKMESH.replace("simpleGrading (1 1 1)", "simpleGrading (2 1 1)"))
    with pytest.raises(HostError, match="not a box"):
        parse_blockmesh(BLOCKMESH.replace("(4 4 0.5)", "(4.1 4 0.5)"))


@pytest.mark.parametrize("fmt", [None, "ascii", "binary"])
def test_field_writer(cuda_lib, fmt):
    from sdfibm_gb300.vof import write_scalar_field
    v = np.random.default_rng(1).uniform(0, 1, 1000)
    v[:10] = (0.0, 1.0, 0.5, 1e-9, 0.25, 0.125, 1.0, 0.0, 0.999999, 3.383163316996635e-05)
    data = write_scalar_field(FIELD.encode(), v, fmt, precision=17)
    got, rest = read_field(data)
    assert np.array_equal(got, v)
    assert (b"binary" in data.split(b"}")[0]) == (fmt == "binary")
    # everything after the list is the template's
    assert rest.lstrip(b"\n").startswith(b";\n\nboundaryField\n{\n    left { type zeroGradient; }")
    # the written file is itself a template: a second write replaces the first list
    again = write_scalar_field(data, v[::-1], None, precision=17)
    assert np.array_equal(read_field(again)[0], v[::-1])
    assert len(again) == len(data)


def test_field_writer_precision(cuda_lib):
    from sdfibm_gb300.vof import write_scalar_field
    data = write_scalar_field(FIELD.encode(), [0.123456789, 1.0, 0.0], "ascii", precision=6)
    assert b"\n3\n(\n0.123457\n1\n0\n)\n;" in data


def test_oracle_matches_the_tools_field():
    """The oracle's REF-GEO fractions summed over the example's solids and planes reproduce the shipped field: all
    but the cells with a vertex exactly on a rectangle's edge (blockMesh's point coordinates decide those, 3.4e-5)."""
    g = golden("tool_vof_alpha.npz")
    mesh = abi.mesh_desc((200, 200, 1), g["origin"], g["h"], twod=1)
    oc = OracleCloud(mesh, example_solids(), abi.options(rho_f=1.0), faithful=True)
    f = oc.new_fields()
    oc.interact(0.0, 1.0, np.zeros(3 * oc.N), f)
    d = np.abs(f["As"] - g["alpha"])
    assert (d <= 1e-12).sum() >= 40000 - 64 and d.max() < 3.5e-5
    assert abs(f["As"].sum() - g["alpha"].sum()) * 4e-4 < 1e-6 * 5.2
    # without the planes, the field differs in the half plane below the first one
    oc2 = OracleCloud(mesh, example_solids()[:12], abi.options(rho_f=1.0), faithful=False)
    f2 = oc2.new_fields()
    oc2.interact(0.0, 1.0, np.zeros(3 * oc2.N), f2)
    assert (np.abs(f2["As"] - g["alpha"]) > 0.5).sum() > 4000


def _write_case(case):
    for d in ("system", "0"):
        (case / d).mkdir(parents=True)
    (case / "solidDict").write_text(vof_dict_text())
    (case / "system" / "blockMeshDict").write_text(BLOCKMESH)
    (case / "system" / "controlDict").write_text("application interFoam;\nwriteFormat binary;\nwritePrecision 6;\n")
    (case / "0" / "alpha.water").write_text(FIELD)


def test_run_case_host_logic(cuda_lib, tmp_path, monkeypatch):
    """run_case's host logic (dictionaries, mesh, template, writer) with the coupling pass answered by the oracle."""
    from sdfibm_gb300 import vof

    def oracle_vof(mesh, solids, device="cuda"):
        oc = OracleCloud(mesh, solids, abi.options(rho_f=1.0), faithful=False)
        f = oc.new_fields()
        oc.interact(0.0, 1.0, np.zeros(3 * oc.N), f)
        return f["As"]

    monkeypatch.setattr(vof, "smooth_vof", oracle_vof)
    case = tmp_path / "case"
    _write_case(case)
    logs = []
    alpha = vof.run_case(str(case), log=logs.append)
    data = (case / "0" / "alpha.water").read_bytes()
    assert b"format      binary;" in data
    got, _ = read_field(data)
    assert np.array_equal(got, alpha)
    g = golden("tool_vof_alpha.npz")["alpha"]
    assert np.abs(got - g).max() < 3.5e-5
    assert re.match(r"\* Write smooth phase field \[alpha.water\] to \./0, total volume = 5\.2017", logs[-1])


@pytest.mark.gpu
def test_run_case_gpu(cuda_lib, torch_cuda, tmp_path):
    from sdfibm_gb300.vof import run_case
    case = tmp_path / "case"
    _write_case(case)
    logs = []
    alpha = run_case(str(case), log=logs.append)
    got, _ = read_field((case / "0" / "alpha.water").read_bytes())
    assert np.array_equal(got, alpha)
    g = golden("tool_vof_alpha.npz")["alpha"]
    # FP32 fractions within 1e-5 relative of the FP64 evaluation, plus the 64 cells on rectangle edges
    assert np.abs(got - g).max() < 4e-5
    assert abs(got.sum() - g.sum()) < 1e-5 * g.sum()
    assert logs[-1].startswith("* Write smooth phase field [alpha.water]")
