"""Regenerates the golden fixtures of tests/golden from the reference checkout (run in a container that has it).

  re200_As.npz          the As field the reference ships for examples/flow_past_cylinder/re200 (0/As, written by
                        SolidCloud::initialCorrect: a static circle r=1 at the origin, 78400-cell multi-block mesh).
                        Kept: the 14400 cells of the uniform centre block (h=0.1 on [-6,6]^2, cell offset 20800).
  falling_ellipse.npz   the oracle run on the reference's own OpenFOAM polyMesh of examples/falling_ellipse
                        (100x200x1 cells, ellipse 0.3x0.15 at (0.5,3.5), euler z=-45 deg): touched cells, As, forcing.
                        It pins the uniform-mesh ordering conventions against a real OpenFOAM mesh.
  re200_blocks.npz      the block structure of examples/flow_past_cylinder/re200/system/blockMeshDict (32 vertices,
                        9 hex blocks with their cell counts and simpleGrading): the tests rebuild the graded
                        multi-block mesh from it (tests/polymesh_gen.py) for the unstructured-mesh path.
  tool_vof_alpha.npz    the smooth phase field the reference's VOF initializer wrote for tool_vof/example
                        (0/alpha.water: 200x200x1 cells on [0,4]^2, twelve shapes and two planes of its solidDict).
It also checks that the host front ends read every solidDict the reference ships, and that the library's OpenFOAM
readers agree with this script's on the reference's binary mesh and field files (no fixture is written for those).
Usage: python tests/golden/make_golden.py /path/to/reference
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))


def read_foam_list(path, dtype, ncomp=1):
    b = open(path, "rb").read()
    i = b.index(b"}")
    m = re.compile(rb"\n(\d+)\n\(").search(b, i)
    n = int(m.group(1))
    s = m.end()
    a = np.frombuffer(b[s:s + n * ncomp * np.dtype(dtype).itemsize], dtype=dtype)
    return (a.reshape(n, ncomp) if ncomp > 1 else a), b[s + n * ncomp * np.dtype(dtype).itemsize:]


def read_faces(path):
    b = open(path, "rb").read()
    i = b.index(b"}")
    m = re.compile(rb"\n(\d+)\n\(").search(b, i)
    n = int(m.group(1))
    s = m.end()
    off = np.frombuffer(b[s:s + n * 4], dtype="<i4")
    rest = b[s + n * 4:]
    m2 = re.compile(rb"\n(\d+)\n\(").search(rest)
    n2 = int(m2.group(1))
    lab = np.frombuffer(rest[m2.end():m2.end() + n2 * 4], dtype="<i4")
    return off, lab


def read_block_mesh_dict(path):
    """vertices [V, 3], hex labels [B, 8], cell counts [B, 3] and simpleGrading [B, 3] of a blockMeshDict (straight
    edges, uniform expansion per direction), comments removed."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    vblock = text[text.index("vertices"):text.index("blocks")]
    verts = np.array([[float(v) for v in m.split()] for m in re.findall(r"\(([^()]*)\)", vblock)])
    bblock = text[text.index("blocks"):text.index("edges")]
    hexes, counts, grades = [], [], []
    for m in re.finditer(r"hex\s*\(([^)]*)\)\s*\(([^)]*)\)\s*simpleGrading\s*\(([^)]*)\)", bblock):
        hexes.append([int(v) for v in m.group(1).split()])
        counts.append([int(v) for v in m.group(2).split()])
        grades.append([float(v) for v in m.group(3).split()])
    return verts, np.array(hexes), np.array(counts), np.array(grades)


def check_example_dicts(ref):
    """The host front ends read every solidDict the reference ships: the solid count, and the positions in order
    against a plain-text extraction of the pos entries of the solids block."""
    import glob
    from sdfibm_gb300.host import parse_soliddict
    from sdfibm_gb300.vof import parse_vofdict
    for path in sorted(glob.glob(os.path.join(ref, "examples", "**", "solidDict"), recursive=True)):
        text = open(path).read()
        solids, _, _ = parse_soliddict(text, 1.0)
        block = text[text.index("solids"):]
        pos = [tuple(float(v) for v in m.split()) for m in re.findall(r"\bpos\s*\(([^)]*)\)", block)]
        assert [tuple(d.pos) for d in solids] == pos, path
        print("%s: %d solids" % (os.path.relpath(path, ref), len(solids)))
    solids, _ = parse_vofdict(open(os.path.join(ref, "tool_vof", "example", "solidDict")).read())
    assert len(solids) == 14
    print("tool_vof/example/solidDict: %d solids and planes" % len(solids))


def check_foam_readers(ref):
    """The library's OpenFOAM readers (sdfibm_gb300.foam_io) give the arrays this script's readers give on the
    reference's binary files, and the falling_ellipse polyMesh is the uniform 100 x 200 x 1 mesh the tests use."""
    from sdfibm_gb300 import foam_io
    pm = os.path.join(ref, "examples/falling_ellipse/constant/polyMesh")
    assert np.array_equal(foam_io.read_list(os.path.join(pm, "points"), "vector")[0],
                          read_foam_list(os.path.join(pm, "points"), "<f8", 3)[0])
    for name in ("owner", "neighbour"):
        assert np.array_equal(foam_io.read_list(os.path.join(pm, name), "label")[0],
                              read_foam_list(os.path.join(pm, name), "<i4")[0])
    off, lab = foam_io.read_faces(os.path.join(pm, "faces"))
    off2, lab2 = read_faces(os.path.join(pm, "faces"))
    assert np.array_equal(off, off2) and np.array_equal(lab, lab2)
    m = foam_io.uniform_mesh_from_polymesh(pm)
    assert (m.nx, m.ny, m.nz) == (100, 200, 1) and list(m.origin) == [0.0, 0.0, -0.5] and list(m.h) == [0.02, 0.02, 1.0]
    for f in ("examples/flow_past_cylinder/re200/0/As", "tool_vof/example/0/alpha.water"):
        assert np.array_equal(foam_io.read_list(os.path.join(ref, f), "scalar")[0],
                              read_foam_list(os.path.join(ref, f), "<f8")[0])
    print("OpenFOAM readers agree on the falling_ellipse polyMesh, re200 As and tool_vof alpha.water")


def main(ref):
    from oracle.oracle import OracleCloud
    from sdfibm_gb300 import abi
    from sdfibm_gb300.host import make_shape, make_solid, mask_motion
    As, _ = read_foam_list(os.path.join(ref, "examples/flow_past_cylinder/re200/0/As"), "<f8")
    assert len(As) == 78400
    centre = np.ascontiguousarray(As[20800:20800 + 14400])
    np.savez_compressed(os.path.join(HERE, "re200_As.npz"), As=centre, nx=120, ny=120,
                        origin=np.array([-6.0, -6.0, -0.5]), h=np.array([0.1, 0.1, 1.0]))
    pm = os.path.join(ref, "examples/falling_ellipse/constant/polyMesh")
    pts, _ = read_foam_list(os.path.join(pm, "points"), "<f8", 3)
    own, _ = read_foam_list(os.path.join(pm, "owner"), "<i4")
    nei, _ = read_foam_list(os.path.join(pm, "neighbour"), "<i4")
    off, lab = read_faces(os.path.join(pm, "faces"))
    shape = make_shape("Ellipse", radiusa=0.3, radiusb=0.15)
    solid = make_solid(0, shape, 2.0, (0.5, 3.5, 0.0), (0.0, 0.0, -45.0), motion=mask_motion("b111111"))
    mesh = abi.mesh_desc((100, 200, 1), (0.0, 0.0, -0.5), (0.02, 0.02, 1.0), twod=1)
    opt = abi.options(rho_f=1.0)
    oc = OracleCloud(mesh, [solid], opt, polymesh=(pts, off, lab, own, nei))
    N = oc.N
    rng = np.random.default_rng(7)
    U = (rng.standard_normal((3, N), dtype=np.float32) * np.float32(0.1)).astype(np.float64)
    f = oc.new_fields()
    FT = oc.interact(0.0, 0.01, U, f)
    cells, types = oc.touched(0)
    np.savez_compressed(os.path.join(HERE, "falling_ellipse.npz"), cells=cells, types=types, As=f["As"][cells],
                        Fs=f["Fs"].reshape(3, N)[:, cells], FT=FT, U_seed=7, U_std=0.1, dt=0.01)
    verts, hexes, counts, grades = read_block_mesh_dict(
        os.path.join(ref, "examples/flow_past_cylinder/re200/system/blockMeshDict"))
    assert verts.shape == (32, 3) and hexes.shape == (9, 8) and counts.prod(1).sum() == 78400
    np.savez_compressed(os.path.join(HERE, "re200_blocks.npz"), vertices=verts, hexes=hexes, counts=counts,
                        grading=grades)
    vof, _ = read_foam_list(os.path.join(ref, "tool_vof/example/0/alpha.water"), "<f8")
    assert len(vof) == 40000
    np.savez_compressed(os.path.join(HERE, "tool_vof_alpha.npz"), alpha=np.ascontiguousarray(vof), nx=200, ny=200,
                        origin=np.array([0.0, 0.0, -0.5]), h=np.array([0.02, 0.02, 1.0]))
    print("re200: %d nonzero; falling_ellipse: %d touched cells, FT=%s; tool_vof: %d nonzero"
          % ((centre > 0).sum(), len(cells), FT, (vof > 0).sum()))
    check_example_dicts(ref)
    check_foam_readers(ref)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SDFIBM_REFERENCE")
    if not src:
        sys.exit("usage: make_golden.py REFERENCE_CHECKOUT  (or set SDFIBM_REFERENCE)")
    main(src)
