"""Host-side pieces of bench.py, on CPU: the clock record taken during the timed region (median SM clock and the
throttle reasons that reject a run), the roofline denominators, and the workload set-up of each method."""
import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def test_clock_record():
    import bench
    c = bench.ClockSampler(0)
    c.proc = _Proc()
    # index, clocks.sm, clocks.max.sm, power, active mask, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    c.lines = ["0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
               "0, 1980, 2070, 950.0, 0x4, Not Active, Not Active, Not Active, Active",
               "0, 2010, 2070, 990.3, 0x0, Not Active, Not Active, Not Active, Not Active",
               "garbage line", "0, [N/A], 2070, 1.0, 0x0, a, b, c, d"]
    r = c.stop()
    assert r["sm_mhz"] == 1980.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]
    c.lines.append("0, 1500, 2070, 700.0, 0x8, Active, Not Active, Not Active, Not Active")
    assert "hw_slowdown" in c.stop()["reasons"]
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


def test_peaks():
    import bench
    peaks, kind = bench.load_peaks()
    assert kind in ("measured", "fallback") and peaks["hbm_gbs"] > 1000 and peaks["bf16_tflops"] > 100


def test_workload_setup():
    import bench
    from sdfibm_gb300 import abi
    for method, fm in (("refgeo", abi.FRACTION_REFGEO), ("subsample", abi.FRACTION_SUBSAMPLE),
                       ("learned", abi.FRACTION_LEARNED)):
        a = argparse.Namespace(config="poly3d_512", scale=0.125, method=method, subsample_n=12, exact_forcing=False)
        w = bench.make_workload(a)
        assert w.opt.fraction_method == fm and w.opt.exact_forcing == 0
        if method == "subsample":
            assert w.opt.subsample_n == 12
        if method == "learned":
            assert w.opt.learned_fallback_n == 16
        assert w.mesh.nx == 64 and len(w.solids) > 10
