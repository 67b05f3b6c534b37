"""The library's C ABI from a plain C99 program (tests/c_client/client.c), on CPU: the headers compile as C with
-Wall -Wextra -pedantic -Werror, every entry point links against libsdfibm_cuda.so, and the host-side functions give
the same records as the Python binding."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
DICT = """meta { on_fluid 1; on_twod 0; gravity (0 0 -9.81); }
shapes { a { name ball; type Sphere; radius 0.1; } b { name brick; type Box; radiusa 0.1; radiusb 0.2; radiusc 0.05; } }
materials { m { name steel; type General; rho 7.8; } }
motions { f { name fixed; type Motion01Mask; mask b000000; } }
solids { s1 { shp_name ball; mot_name free; mat_name steel; pos (0.5 0.5 0.5); vel (0 0 -1); }
         s2 { shp_name brick; mot_name fixed; mat_name steel; pos (0.2 0.3 0.4); euler (10 20 30); } }
"""


def test_c_client(cuda_lib, tmp_path):
    cc = shutil.which(os.environ.get("CC", "gcc"))
    if cc is None:
        pytest.skip("no C compiler")
    from sdfibm_gb300 import abi
    from sdfibm_gb300._lib import LIB_PATH
    from sdfibm_gb300.host import format_state, parse_soliddict
    exe = str(tmp_path / "client")
    libdir = os.path.dirname(LIB_PATH)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "c_client", "client.c"), "-o", exe, "-L", libdir,
                        "-l:libsdfibm_cuda.so", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    (tmp_path / "solidDict").write_text(DICT)
    r = subprocess.run([exe, str(tmp_path / "solidDict")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.split("\n")
    assert lines[0] == "linked 15" and lines[1] == "solids 2 twod 0 rho_f 1000"
    assert int(lines[2].split()[1]) > 500
    # the same records through the Python binding
    solids, _, _ = parse_soliddict(DICT, 1000.0)
    states = []
    for d in solids:
        s = abi.SolidState()
        for f in ("pos", "quat", "vel", "omega"):
            for a in range(len(getattr(s, f))):
                getattr(s, f)[a] = getattr(d, f)[a]
        states.append(s)
    assert "\n".join(lines[3:]) == format_state(0.5, states, False)
