"""The benchmark's own measurement logic, on synthetic inputs: the clock
record keeps only the samples taken inside the timed region and reports the
throttle reasons seen there; the roofline turns a profiled run's phase times
and unit counts into fractions of each roof and names the closest."""
import importlib.util
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def row(sm, active="Not Active", thermal="Not Active", power="Not Active"):
    # index, clocks.sm, clocks.max.sm, power.draw, active reasons, hw_slowdown,
    # hw_thermal_slowdown, sw_thermal_slowdown, sw_power_cap
    return ["0", str(sm), "2070", "900.0", "0x0", active, thermal, "Not Active", power]


class FakeProc:
    """stands in for the nvidia-smi process the sampler stops"""
    def terminate(self):
        pass

    def wait(self, timeout=None):
        return 0


def sampler(bench):
    c = bench.ClockSampler(0)
    c.proc = FakeProc()
    return c


def test_clocks_inside_the_timed_region_only(bench):
    c = sampler(bench)
    c.t0, c.t1 = 10.0, 11.0
    c.rows = [(9.5, row(345)), (10.1, row(2070)), (10.5, row(2055)), (10.9, row(2070, power="Active")),
              (11.5, row(600, thermal="Active"))]
    out = c.stop()
    assert out["samples"] == 3 and out["sm_mhz"] == 2070.0 and out["sm_max_mhz"] == 2070.0
    assert out["reasons"] == ["sw_power_cap"]        # the thermal sample came after the region


def test_clocks_of_a_region_shorter_than_a_period(bench):
    c = sampler(bench)
    c.t0, c.t1 = 10.0, 10.01
    c.rows = [(9.95, row(2070)), (10.06, row(2040, active="Active"))]
    out = c.stop()
    assert out["samples"] == 2 and out["reasons"] == ["hw_slowdown"]


def test_clocks_without_nvidia_smi(bench):
    assert bench.ClockSampler(0).stop()["reasons"] == ["nvidia-smi unavailable"]


class FakeDpm:
    @staticmethod
    def atomic_roof():
        return 200e9


def test_roofline_names_the_closest_roof(bench):
    pr = {"electron_ms": 16.0, "photon_ms": 6.0, "electron_launches": 32.0, "photon_launches": 32.0,
          "electron_steps": 4.0e8, "photon_steps": 9.0e7, "total_ms": 22.0}
    r = bench.roofline_of(FakeDpm, pr, True, True, {"sm_mhz": 2070.0})
    c = r["roofs"]
    assert r["kernel"] == "ElectronPhaseB" and r["bound"] == max(c, key=lambda k: c[k]["frac"])
    import json
    with open(os.path.join(ROOT, "profiles", "counters.json")) as f:
        k = json.load(f)["ElectronPhaseB"]
    issue = k["warp_inst_per_unit"] * 4.0e8 / 16e-3 / 1e9
    assert c["issue"]["achieved"] == pytest.approx(issue)
    assert c["issue"]["peak"] == pytest.approx(152 * 4 * 2070e6 / 1e9)
    assert c["l2_atomic"]["frac"] == pytest.approx(4.0e8 / 16e-3 / 200e9)
    assert r["traffic"] == pytest.approx(k["dram_bytes_per_unit"] * 4.0e8 / 32.0)
    assert r["avg_launch_ms"] == pytest.approx(0.5) and r["units_per_launch"] == pytest.approx(1.25e7)
