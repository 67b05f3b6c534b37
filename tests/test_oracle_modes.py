"""The oracle's fast mode (the reference side of every GPU parity test) against its faithful mode (the reference's own data
structures: per-solid cell-type arrays, std::set, the phi cache, the full-mesh nearest-cell search), on CPU.
Both must give the same bits for interact, evolve and fixInternal."""
import numpy as np
import pytest

from oracle.oracle import OracleCloud
from sdfibm_gb300 import workloads as W

CASES = {
    "poly3d_256_s0.25": lambda: W.poly3d_256(scale=0.25),
    "poly3d_512_s0.125": lambda: W.poly3d_512(scale=0.125),
    "sedimentation2d_s0.5": lambda: W.sedimentation2d(scale=0.5),
    "cylinder2d_s0.5": lambda: W.cylinder2d(scale=0.5),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fast_equals_faithful(name):
    w = CASES[name]()
    U = w.U_numpy().astype(np.float64).reshape(-1)
    runs = []
    for faithful in (True, False):
        oc = OracleCloud(w.mesh, w.solids, w.opt, faithful=faithful)
        f = oc.new_fields()
        out = []
        for k in range(2):
            FT = oc.interact(k * w.dt, w.dt, U, f)
            out.append((FT.copy(), {key: v.copy() for key, v in f.items()},
                        [oc.touched(s) for s in range(len(w.solids))]))
            oc.evolve(k * w.dt, w.dt)
            out.append(bytes(oc.get_state()))
        out.append(oc.fix_internal(f["Ct"], U))
        runs.append(out)
    a, b = runs
    for x, y in zip(a, b):
        if isinstance(x, bytes):
            assert x == y                                    # solid states after evolve, bit for bit
        elif isinstance(x, np.ndarray):
            assert np.array_equal(x, y)                      # U after fixInternal
        else:
            assert np.array_equal(x[0], y[0])                # force and torque per solid
            for key in x[1]:
                assert np.array_equal(x[1][key], y[1][key]), key
            for (c0, t0), (c1, t1) in zip(x[2], y[2]):       # touched sets and types
                assert np.array_equal(c0, c1) and np.array_equal(t0, t1)
    assert sum(len(c) for c, _ in a[0][2]) > 20
