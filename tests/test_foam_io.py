"""OpenFOAM file input (sdfibm_gb300.foam_io over the host half of the library), on CPU: polyMesh lists and field
internalFields in ascii and binary, faces as faceCompactList and faceList, and the uniform mesh of a single-block
point lattice.  The files are written here in OpenFOAM's layout; the fixture script checks the same readers on the
reference's own binary mesh and field files."""
import numpy as np
import pytest

from sdfibm_gb300.host import HostError


def _header(fmt, cls, obj):
    return ("FoamFile\n{\n    version     2.0;\n    format      %s;\n    class       %s;\n    note        \"n: 1\";\n"
            "    object      %s;\n}\n// * * * * //\n\n" % (fmt, cls, obj)).encode()


def _list(arr, fmt, kind):
    arr = np.asarray(arr)
    if fmt == "binary":
        dt = "<i4" if kind == "label" else "<f8"
        return b"%d\n(" % len(arr) + np.ascontiguousarray(arr, dtype=dt).tobytes() + b")\n"
    if kind == "vector":
        items = ["(%r %r %r)" % tuple(float(v) for v in row) for row in arr]
    else:
        items = [repr(int(v)) if kind == "label" else repr(float(v)) for v in arr]
    return ("%d\n(\n%s\n)\n" % (len(arr), "\n".join(items))).encode()


def lattice(n, o=(0.0, 0.0, -0.5), h=(0.25, 0.5, 1.0), jitter=0.0, seed=0):
    i, j, k = np.meshgrid(np.arange(n[0] + 1), np.arange(n[1] + 1), np.arange(n[2] + 1), indexing="ij")
    pts = np.stack([o[0] + i * h[0], o[1] + j * h[1], o[2] + k * h[2]], -1).transpose(2, 1, 0, 3).reshape(-1, 3)
    if jitter:
        pts = pts + np.random.default_rng(seed).uniform(-jitter, jitter, pts.shape)
    return pts


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_lists(cuda_lib, fmt):
    from sdfibm_gb300.foam_io import read_list
    pts = lattice((4, 3, 2))
    got, uniform = read_list(_header(fmt, "vectorField", "points") + _list(pts, fmt, "vector"), "vector")
    assert not uniform and np.array_equal(got, pts)
    own = np.arange(17, dtype=np.int32) * 3 - 5
    got, _ = read_list(_header(fmt, "labelList", "owner") + _list(own, fmt, "label"), "label")
    assert np.array_equal(got, own)
    assert read_list(_header(fmt, "labelList", "neighbour") + _list([], fmt, "label"), "label")[0].size == 0
    with pytest.raises(HostError):
        read_list(_header(fmt, "labelList", "owner") + _list(own, fmt, "label")[:-12], "label")


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_faces(cuda_lib, fmt):
    from sdfibm_gb300.foam_io import read_faces
    faces = [[0, 1, 5, 4], [1, 2, 6, 5, 9], [3, 7, 8]]
    off = np.cumsum([0] + [len(f) for f in faces]).astype(np.int32)
    lab = np.concatenate(faces).astype(np.int32)
    data = _header(fmt, "faceCompactList", "faces") + _list(off, fmt, "label") + b"\n" + _list(lab, fmt, "label")
    o, l = read_faces(data)
    assert np.array_equal(o, off) and np.array_equal(l, lab)
    if fmt == "ascii":
        text = "%d\n(\n%s\n)\n" % (len(faces), "\n".join("%d(%s)" % (len(f), " ".join(map(str, f))) for f in faces))
        o, l = read_faces(_header(fmt, "faceList", "faces") + text.encode())
        assert np.array_equal(o, off) and np.array_equal(l, lab)
    bad = _header(fmt, "faceCompactList", "faces") + _list(off[::-1], fmt, "label") + _list(lab, fmt, "label")
    with pytest.raises(HostError):
        read_faces(bad)


def test_uniform_mesh(cuda_lib):
    from sdfibm_gb300.foam_io import uniform_mesh
    m = uniform_mesh(lattice((4, 3, 2)), 24)
    assert (m.nx, m.ny, m.nz, m.twod) == (4, 3, 2, 0)
    assert list(m.origin) == [0.0, 0.0, -0.5] and list(m.h) == [0.25, 0.5, 1.0]
    # blockMesh's points sit within rounding of the lattice (y = 0.019999999999999997 and the like)
    m = uniform_mesh(lattice((5, 4, 1), jitter=1e-14), 20)
    assert (m.nx, m.ny, m.nz, m.twod) == (5, 4, 1, 1)
    pts = lattice((4, 3, 2))
    pts[7, 1] += 1e-6
    with pytest.raises(HostError, match="off the uniform lattice"):
        uniform_mesh(pts, 24)
    with pytest.raises(HostError, match="cell count"):
        uniform_mesh(lattice((4, 3, 2)), 25)
    graded = lattice((4, 3, 2))
    graded[:, 0] = graded[:, 0] ** 2
    with pytest.raises(HostError):
        uniform_mesh(graded, 24)


def test_field_internal(cuda_lib):
    from sdfibm_gb300.foam_io import read_list
    from sdfibm_gb300.vof import write_scalar_field
    from test_vof import FIELD
    v = np.random.default_rng(4).uniform(0, 1, 333)
    for fmt in ("ascii", "binary"):
        got, uniform = read_list(write_scalar_field(FIELD.encode(), v, fmt, precision=17), "scalar")
        assert not uniform and np.array_equal(got, v)
    got, uniform = read_list(FIELD.encode(), "scalar")
    assert uniform and got.tolist() == [0.0]
    U = np.random.default_rng(5).normal(size=(6, 3))
    text = FIELD.replace("volScalarField", "volVectorField").replace(
        "internalField   uniform 0;",
        "internalField   nonuniform List<vector> %s;" % _list(U, "ascii", "vector").decode())
    got, uniform = read_list(text.encode(), "vector")
    assert not uniform and np.array_equal(got, U)
    got, uniform = read_list(FIELD.replace("volScalarField", "volVectorField").replace(
        "uniform 0;", "uniform (1 -2 3.5);").encode(), "vector")
    assert uniform and got.tolist() == [[1.0, -2.0, 3.5]]
    with pytest.raises(HostError, match="List<vector>"):
        read_list(text.encode(), "scalar")


def test_vof_case_from_polymesh(cuda_lib, tmp_path, monkeypatch):
    """run_case on a case that has only its polyMesh: the uniform block is recovered from the points."""
    import test_vof
    from sdfibm_gb300 import abi, vof
    from oracle.oracle import OracleCloud

    def oracle_vof(mesh, solids, device="cuda"):
        oc = OracleCloud(mesh, solids, abi.options(rho_f=1.0), faithful=False)
        f = oc.new_fields()
        oc.interact(0.0, 1.0, np.zeros(3 * oc.N), f)
        return f["As"]

    monkeypatch.setattr(vof, "smooth_vof", oracle_vof)
    case = tmp_path / "case"
    test_vof._write_case(case)
    (case / "system" / "blockMeshDict").unlink()
    pm = case / "constant" / "polyMesh"
    pm.mkdir(parents=True)
    pts = lattice((200, 200, 1), o=(0.0, 0.0, -0.5), h=(0.02, 0.02, 1.0))
    (pm / "points").write_bytes(_header("binary", "vectorField", "points") + _list(pts, "binary", "vector"))
    (pm / "owner").write_bytes(_header("binary", "labelList", "owner") +
                               _list(np.arange(40000, dtype=np.int32), "binary", "label"))
    alpha = vof.run_case(str(case), log=lambda s: None)
    g = test_vof.golden("tool_vof_alpha.npz")["alpha"]
    assert np.abs(alpha - g).max() < 3.5e-5


def test_nul_bytes_in_the_header(cuda_lib):
    """Binary files can hold NUL bytes where text is expected: the dictionary lexer takes them as word characters
    (a NUL once matched strchr's terminator and the lexer stopped advancing)."""
    from sdfibm_gb300.foam_io import read_faces, read_list
    from sdfibm_gb300.vof import write_scalar_field
    pts = _header("binary", "vectorField", "points").replace(b"{", b"{\x00", 1) + _list(lattice((2, 2, 1)), "binary",
                                                                                       "vector")
    got, _ = read_list(pts, "vector")
    assert got.shape == (18, 3)
    bad = _header("binary", "face\x00List", "faces") + b"1\n(\x00)\n"
    with pytest.raises(HostError):
        read_faces(bad)
    from test_vof import FIELD
    data = FIELD.replace("version     2.0;", "version \x00 2.0;").encode()
    assert b"\n3\n(" in write_scalar_field(data, [0.5, 0.25, 1.0], "ascii")


@pytest.mark.parametrize("fmt", ["ascii", "binary"])
def test_vector_field_writer(cuda_lib, fmt):
    from sdfibm_gb300.foam_io import read_list, write_field
    from test_vof import FIELD
    template = FIELD.replace("volScalarField", "volVectorField").replace("uniform 0;", "uniform (0 0 0);").encode()
    Fs = np.random.default_rng(6).normal(size=(3, 40))          # cell-major planes, as the coupling returns them
    data = write_field(template, Fs, fmt, precision=17)
    got, uniform = read_list(data, "vector")
    assert not uniform and np.array_equal(got, Fs.T)
    again = write_field(data, Fs.T[::-1], None, precision=17)   # the written file as the next template
    assert np.array_equal(read_list(again, "vector")[0], Fs.T[::-1])
    assert again.endswith(b"boundaryField\n{\n    left { type zeroGradient; }\n    right { type zeroGradient; }\n"
                          b"    frontAndBack { type empty; }\n}\n")


def test_ascii_rewrite_of_short_entries(cuda_lib):
    """A VOF field written at 6 digits is mostly "0" and "1": rewriting it must not take its size as too large."""
    from sdfibm_gb300.foam_io import read_list, write_field
    from test_vof import FIELD
    v = np.zeros(5000)
    v[::7] = 1.0
    data = write_field(FIELD.encode(), v, "ascii")
    again = write_field(data, v[::-1], "ascii")
    assert np.array_equal(read_list(again, "scalar")[0], v[::-1])
