"""Address and undefined-behaviour sanitizer builds of the host code, on CPU.

Three drivers are compiled with g++ -fsanitize=address,undefined and run; a sanitizer report aborts them:
  - tests/sanitize/host_driver.cpp drives the host half of the library (sdfibm_gb300/csrc/host*.cpp). Inputs are
    the solidDict, VOF-dict, blockMesh, OpenFOAM list and field-file front ends and writers: every prefix of each input,
    byte-mutated copies, and output buffers of every capacity below what is needed;
  - tests/sanitize/oracle_driver.cpp drives the oracle: both modes, 2-D and 3-D, every shape, interact, evolve with
    collisions (solids that coincide, leave the mesh or go non-finite), fixInternal and the mean field;
  - tests/cpp_client/cloud_client.cpp drives the C++ SolidCloud (include/sdfibm_cloud.hpp) through the reference's
    time loop, the device entry points answered by the oracle.
The device half has no sanitizer run here."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from sdfibm_gb300.build import HOST_SOURCES

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN = ["-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-ffp-contract=off",
       "-I", os.path.join(ROOT, "include")]
ENV = dict(os.environ, UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", ASAN_OPTIONS="detect_leaks=1")


def _compile(out, sources, extra=()):
    cxx = shutil.which(os.environ.get("CXX", "g++"))
    if cxx is None:
        pytest.skip("no C++ compiler")
    r = subprocess.run([cxx] + SAN + [os.path.join(ROOT, s) for s in sources] + ["-o", out] + list(extra),
                       capture_output=True, text=True)
    if r.returncode != 0 and "sanitize" in r.stderr:
        pytest.skip("the compiler has no sanitizer runtime")
    assert r.returncode == 0, r.stderr[-2000:]


def test_host_code_under_sanitizers(cuda_lib, tmp_path):
    from test_host import DICT
    from test_vof import BLOCKMESH, FIELD, vof_dict_text
    from sdfibm_gb300.vof import write_scalar_field
    d = tmp_path / "in"
    d.mkdir()
    (d / "soliddict.txt").write_text(DICT)
    (d / "vofdict.txt").write_text(vof_dict_text())
    (d / "blockmesh.txt").write_text(BLOCKMESH)
    (d / "field_ascii").write_text(FIELD)
    (d / "field_binary").write_bytes(write_scalar_field(FIELD.encode(), np.linspace(0, 1, 50), "binary"))
    from test_foam_io import _header, _list, lattice
    (d / "points_binary").write_bytes(_header("binary", "vectorField", "points") +
                                      _list(lattice((3, 2, 2)), "binary", "vector"))
    off, lab = np.array([0, 4, 8, 11], np.int32), np.array([0, 1, 5, 4, 1, 2, 6, 5, 3, 7, 8], np.int32)
    (d / "faces_binary").write_bytes(_header("binary", "faceCompactList", "faces") + _list(off, "binary", "label") +
                                     _list(lab, "binary", "label"))
    (d / "faces_ascii").write_bytes(_header("ascii", "faceList", "faces") +
                                    b"3\n(\n4(0 1 5 4)\n4(1 2 6 5)\n3(3 7 8)\n)\n")
    exe = str(tmp_path / "host_driver")
    _compile(exe, ["tests/sanitize/host_driver.cpp"] + HOST_SOURCES)
    r = subprocess.run([exe, str(d)], capture_output=True, text=True, env=ENV, timeout=600)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "calls clean" in r.stdout


def test_oracle_under_sanitizers(tmp_path):
    exe = str(tmp_path / "oracle_driver")
    _compile(exe, ["tests/sanitize/oracle_driver.cpp", "oracle/oracle.cpp"] + HOST_SOURCES, ["-pthread"])
    r = subprocess.run([exe], capture_output=True, text=True, env=ENV, timeout=600)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "calls clean" in r.stdout


def test_cpp_solidcloud_under_sanitizers(tmp_path):
    """The C++ SolidCloud of include/sdfibm_cloud.hpp through its time-loop client, with the device entry points
    answered by the oracle (tests/cpp_client/oracle_abi_shim.cpp), everything built with the sanitizers."""
    from test_solidcloud_cpp import STEPS, DT, _case_files
    exe = str(tmp_path / "client")
    _compile(exe, ["tests/cpp_client/cloud_client.cpp", "tests/cpp_client/oracle_abi_shim.cpp", "oracle/oracle.cpp"] +
             HOST_SOURCES, ["-pthread"])
    _case_files(tmp_path)
    (tmp_path / "out").mkdir()
    r = subprocess.run([exe, str(tmp_path / "solidDict"), str(tmp_path / "mesh.txt"), str(tmp_path / "U.bin"),
                        str(STEPS), repr(DT), str(tmp_path / "out")], capture_output=True, text=True, env=ENV,
                       timeout=600)
    assert r.returncode == 0, (r.stdout + r.stderr)[-4000:]
    assert "solids 4" in r.stdout and (tmp_path / "out" / "meanfield.out").exists()
