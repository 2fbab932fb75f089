"""Host logic of bench.py (no GPU): the equal-time interpolation, the
nvidia-smi clock and throttle parser, and the traffic figures read from the
committed k_extend capture."""
import math

import pytest

import bench


def test_interp_time_is_exact_on_a_power_law():
    # relMSE = 10 / t: straight in log-log, so the interpolation is exact
    curve = [(t, 10.0 / t) for t in (30.0, 60.0, 120.0, 240.0, 480.0)]
    assert bench.interp_time(curve, 0.05) == pytest.approx(200.0)
    assert bench.interp_time(list(reversed(curve)), 0.05) == pytest.approx(200.0)


def test_interp_time_edges():
    curve = [(10.0, 0.5), (20.0, 0.2)]
    assert bench.interp_time(curve, 0.01) is None          # never reached
    assert bench.interp_time(curve, 0.9) == 10.0            # reached at the first point
    assert bench.interp_time([], 0.1) is None
    # the first crossing counts when the curve rises again after it
    bumpy = [(10.0, 0.5), (20.0, 0.05), (40.0, 0.2), (80.0, 0.01)]
    t = bench.interp_time(bumpy, 0.1)
    assert 10.0 < t < 20.0 and t == pytest.approx(math.exp(math.log(10) + math.log(5) / math.log(10) * math.log(2)))


class _Proc:
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


class _Thread:
    def join(self, timeout=None):
        pass


def test_clock_sampler_parses_reasons_and_median():
    cs = bench.ClockSampler(0)
    cs.proc, cs.t = _Proc(), _Thread()
    cs.lines = [
        "0, 2070, 2070, 812.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1390.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1201.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    r = cs.stop()
    assert r["sm_mhz"] == 2070.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 3
    assert r["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi():
    r = bench.ClockSampler(0).stop()
    assert r["sm_mhz"] is None and r["reasons"] == ["nvidia-smi unavailable"]


def test_traffic_figures_come_from_the_committed_capture():
    tr = bench.extend_traffic()
    assert tr is not None
    for part in ("camera", "bounce"):
        d = tr[part]
        assert d["dram_bytes_per_ray"] == pytest.approx(d["dram_bytes"] / d["rays"])
        assert d["l2_bytes_per_ray"] == pytest.approx(d["l2_bytes"] / d["rays"])
        assert 0 < d["dram_bytes_per_ray"] < d["l2_bytes_per_ray"]
    # a whole frame: one camera launch and eleven bounce launches per wavefront
    assert tr["camera"]["rays"] == 1024 * 1024 * 64
    assert tr["bounce"]["launches"] == 11 * tr["camera"]["launches"]
