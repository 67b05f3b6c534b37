"""The C++ SolidCloud of include/sdfibm_cloud.hpp (the reference's interface over the C ABI, host fields).

CPU: the header and the time-loop client of tests/cpp_client/cloud_client.cpp compile with -Wall -Wextra -Werror
and link against libsdfibm_cuda.so; linked instead against a stand-in library that the oracle answers, the client
writes what the same loop written with the oracle directly writes, and the Python SolidCloud loaded on that
stand-in writes the same files.  GPU: the client's cloud.out, meanfield.out and
restart dictionary agree with what the Python SolidCloud writes for the same loop on device fields."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from sdfibm_gb300.build import HOST_SOURCES

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DICT = """meta { on_fluid 1; on_twod 1; gravity (0 -9.81 0); writeFrequency 2; sampler probe; on_meanfield 1; }
shapes
{
    disc { name disc; type Circle; radius 0.05; }
    probe { name probe; type Circle; radius 0.1; }
    wall { name wall; type Plane; }
}
materials { m { name heavy; type General; rho 1.5; } }
motions { f { name fixed; type Motion01Mask; mask b000000; } }
solids
{
    a { shp_name disc; mot_name free; mat_name heavy; pos (0.3 0.5 0); vel (0.1 0 0); omega (0 0 1); }
    b { shp_name disc; mot_name free; mat_name heavy; pos (0.62 0.45 0); vel (-0.1 0.05 0); }
    c { shp_name disc; mot_name free; mat_name heavy; pos (0.5 0.8 0); euler (0 0 30); }
    w { shp_name wall; mot_name fixed; mat_name heavy; pos (0 0.1 0); }
}
"""
MESH = (128, 128, 1, 0.0, 0.0, -0.5, 0.0078125, 0.0078125, 1.0)
STEPS, DT = 3, 0.002


def _client(tmp_path):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    from sdfibm_gb300._lib import LIB_PATH
    libdir = os.path.dirname(LIB_PATH)
    exe = str(tmp_path / "cloud_client")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp_client", "cloud_client.cpp"), "-o", exe, "-L", libdir,
                        "-l:libsdfibm_cuda.so", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_cpp_cloud_compiles(cuda_lib, tmp_path):
    _client(tmp_path)


def _case_files(tmp_path):
    N = MESH[0] * MESH[1] * MESH[2]
    rng = np.random.default_rng(3)
    U = (rng.standard_normal((3, N)) * 0.05).astype(np.float32)
    U[0] += np.float32(0.2)
    (tmp_path / "solidDict").write_text(DICT)
    (tmp_path / "mesh.txt").write_text(" ".join(repr(v) for v in MESH))
    U.tofile(str(tmp_path / "U.bin"))
    return U


def _run(exe, tmp_path, out):
    out.mkdir()
    r = subprocess.run([exe, str(tmp_path / "solidDict"), str(tmp_path / "mesh.txt"), str(tmp_path / "U.bin"),
                        str(STEPS), repr(DT), str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    return r.stdout


def _shim_client(tmp_path):
    """The stand-in library (the oracle behind the entry points) and the time-loop client linked against it."""
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    shim = tmp_path / "shim"
    shim.mkdir()
    inc = ["-I", os.path.join(ROOT, "include")]
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off"] + inc +
                       [os.path.join(ROOT, f) for f in ["tests/cpp_client/oracle_abi_shim.cpp", "oracle/oracle.cpp"] +
                        HOST_SOURCES] +
                       ["-o", str(shim / "libsdfibm_cuda.so"), "-pthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = str(shim / "client")
    r = subprocess.run([cxx, "-std=c++17", "-Wall", "-Wextra", "-Werror"] + inc +
                       [os.path.join(ROOT, "tests", "cpp_client", "cloud_client.cpp"), "-o", exe, "-L", str(shim),
                        "-l:libsdfibm_cuda.so", "-Wl,-rpath," + str(shim)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _python_loop(torch, U, out, device):
    """The client's loop through the Python SolidCloud: initialCorrect, saveState (with the mean field), then per
    step interact, evolve, saveState; a restart dictionary at the end."""
    from sdfibm_gb300 import abi
    from sdfibm_gb300.cloud import SolidCloud
    from sdfibm_gb300.host import StateFile, parse_soliddict, soliddict_shape
    solids, opt, twod = parse_soliddict(DICT, 1.0)
    mesh = abi.mesh_desc(MESH[:3], MESH[3:6], MESH[6:], twod=twod)
    cloud = SolidCloud(mesh, solids, opt)
    cloud.set_sampler(soliddict_shape(DICT, "probe"))
    Ud = torch.from_numpy(U).to(device)
    f = cloud.new_fields(device=device)
    out.mkdir()
    with StateFile(str(out / "cloud.out"), twod, 2, mean_field_path=str(out / "meanfield.out")) as sf:
        cloud.initial_correct(Ud, f)
        cloud.save_state(sf, Ud, f["Ct"])
        for s in range(1, STEPS + 1):
            t = s * DT
            cloud.interact(t, DT, Ud, f)
            cloud.evolve(t, DT)
            cloud.save_state(sf, Ud, f["Ct"])
    cloud.save_restart(DICT, str(out / "solidDict.restart"), precision=17)
    cloud.close()


def test_python_cloud_on_the_oracle(cuda_lib, tmp_path, monkeypatch):
    """The Python SolidCloud's orchestration (initial_correct, save_state with the mean field and its Ct writes,
    save_restart) on CPU tensors, with the stand-in library loaded in place of libsdfibm_cuda.so: its files equal the
    C++ client's on the same stand-in, byte for byte (the same FP64 arithmetic behind both)."""
    torch = pytest.importorskip("torch")
    from sdfibm_gb300 import _lib
    exe = _shim_client(tmp_path)
    U = _case_files(tmp_path)
    _run(exe, tmp_path, tmp_path / "cpp")
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "shim" / "libsdfibm_cuda.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    assert b"oracle" in _lib.load().sdfibm_cuda_version()
    _python_loop(torch, U, tmp_path / "py", "cpu")
    for name in ("cloud.out", "meanfield.out"):
        assert (tmp_path / "py" / name).read_text() == (tmp_path / "cpp" / name).read_text(), name
    a = (tmp_path / "py" / "solidDict.restart").read_text().splitlines()[:-1]
    assert a == (tmp_path / "cpp" / "solidDict.restart").read_text().splitlines()[:-1]


def test_cpp_cloud_on_the_oracle(cuda_lib, tmp_path):
    """The C++ SolidCloud's own logic (construction with initialCorrect, saveState every writeFrequency calls, the
    mean field from two passes of a sampler context with its Ct writes, the host fixInternal, saveRestart) on CPU:
    the time-loop client linked against a stand-in library whose entry points the oracle answers
    (tests/cpp_client/oracle_abi_shim.cpp), against the same loop written with the oracle directly."""
    from oracle.oracle import OracleCloud
    from sdfibm_gb300 import abi
    from sdfibm_gb300.host import format_mean_field, format_state, parse_soliddict, soliddict_shape, write_restart
    exe = _shim_client(tmp_path)
    U = _case_files(tmp_path)
    stdout = _run(exe, tmp_path, tmp_path / "cpp")
    assert "solids 4" in stdout

    # the same loop on the oracle, written out directly
    solids, opt, twod = parse_soliddict(DICT, 1.0)
    mesh = abi.mesh_desc(MESH[:3], MESH[3:6], MESH[6:], twod=twod)
    oc = OracleCloud(mesh, solids, opt, faithful=False)
    f = oc.new_fields()
    Uo = U.astype(np.float64).reshape(-1)
    oc.interact(0.0, 1.0, Uo, f)                                  # initialCorrect
    st = oc.get_state()
    for x in st:
        for a in range(3):
            x.force[a] = x.torque[a] = 0.0
    oc.set_state(st)
    sampler = soliddict_shape(DICT, "probe")
    state, means = [], []
    for call in range(STEPS + 1):
        t = call * DT
        if call:
            oc.interact(t, DT, Uo, f)
            oc.evolve(t, DT)
        if call % 2 == 0:                                         # writeFrequency 2
            state.append(format_state(t, list(oc.get_state()), True))
        means.append(oc.mean_field(sampler, Uo))
    assert (tmp_path / "cpp" / "cloud.out").read_text() == "".join(state)
    got = np.array([[float(v) for v in l.split()] for l in (tmp_path / "cpp" / "meanfield.out").read_text().splitlines()])
    want = np.array([[float(v) for v in format_mean_field(m).split()] for m in means])
    assert got.shape == want.shape and np.allclose(got, want, rtol=2e-6, atol=1e-12)
    restart = write_restart(DICT, list(oc.get_state()), True, precision=17, stamp="x").splitlines()[:-1]
    assert (tmp_path / "cpp" / "solidDict.restart").read_text().splitlines()[:-1] == restart


@pytest.mark.gpu
def test_cpp_cloud_matches_python(cuda_lib, torch_cuda, tmp_path):
    torch = torch_cuda
    exe = _client(tmp_path)
    U = _case_files(tmp_path)
    out = tmp_path / "cpp"
    _run(exe, tmp_path, out)

    # the same loop through the Python binding, device fields
    py = tmp_path / "py"
    _python_loop(torch, U, py, "cuda")

    # the per-solid force sums are FP64 atomics whose order varies from run to run, so the two runs agree to the last
    # bits of the force and what follows from it: the 7-digit records within one unit of their last digit, the
    # 17-digit restart within 1e-12
    def numbers(text):
        return np.array([[float(v) for v in line.split()] for line in text.splitlines()])

    def close(a, b):  # per column: one unit of the 7th digit, or 1e-9 of the column's scale (sums that cancel)
        scale = np.maximum(np.abs(a).max(axis=0), np.abs(b).max(axis=0))
        return np.all(np.abs(a - b) <= 2e-6 * np.abs(b) + 1e-9 * scale)
    a, b = numbers((out / "cloud.out").read_text()), numbers((py / "cloud.out").read_text())
    assert a.shape == b.shape == (2 * 4, 10)                 # calls 0 and 2 of 4, four solids, 2-D columns
    assert close(a, b)
    a, b = numbers((out / "meanfield.out").read_text()), numbers((py / "meanfield.out").read_text())
    assert a.shape == b.shape == (STEPS + 1, 3 * 4)
    assert close(a, b)
    ra = (out / "solidDict.restart").read_text().splitlines()[:-1]   # all but the time stamp
    rb = (py / "solidDict.restart").read_text().splitlines()[:-1]
    assert len(ra) == len(rb)
    for x, y in zip(ra, rb):
        if "(" in x:
            vx = [float(v) for v in x[x.index("(") + 1:x.index(")")].split()]
            vy = [float(v) for v in y[y.index("(") + 1:y.index(")")].split()]
            assert x[:x.index("(")] == y[:y.index("(")] and np.allclose(vx, vy, rtol=1e-12, atol=1e-15), (x, y)
        else:
            assert x == y
