"""bench.py's clock record on CPU: the summary of nvidia-smi lines counts only the samples taken
after the sampler's first line (the timed region starts once that line exists), reports the
median SM clock under load and every throttle reason seen active, and says so when nvidia-smi
could not be started."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _sampler(tmp_path, lines, skip):
    import bench
    c = bench.ClockSampler(0)
    c.path = str(tmp_path / "clocks.csv")
    with open(c.path, "w") as f:
        f.write("\n".join(lines) + "\n")
    c.proc = object()   # stands for a started nvidia-smi
    c.skip = skip
    return c


def test_summary_skips_the_first_sample_and_takes_the_median(tmp_path):
    idle = "345, 2070, 150.0, Not Active, Not Active, Not Active, Not Active"
    load = ["2070, 2070, 900.0, Not Active, Not Active, Not Active, Not Active",
            "2055, 2070, 950.0, Not Active, Not Active, Not Active, Active",
            "2070, 2070, 960.0, Not Active, Not Active, Not Active, Not Active"]
    s = _sampler(tmp_path, [idle] + load, skip=1).summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]


def test_summary_reports_thermal_slowdown_and_ignores_malformed_lines(tmp_path):
    lines = ["1500, 2070, 1200.0, Not Active, Active, Not Active, Not Active",
             "[N/A], 2070, 1200.0, Not Active, Not Active, Not Active, Not Active",
             "garbage"]
    s = _sampler(tmp_path, lines, skip=0).summary()
    assert s["samples"] == 1 and s["sm_mhz"] == 1500.0
    assert s["reasons"] == ["hw_thermal_slowdown"]


def test_summary_without_nvidia_smi():
    import bench
    c = bench.ClockSampler(0)
    c.proc = None
    s = c.summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["nvidia-smi unavailable"]


class _FakeNvml:
    """Stands for NvmlApi: a scripted sequence of SM clocks and clock-event reason words."""

    def __init__(self, clocks, reasons):
        self.clocks, self.reasons_seq, self.k = list(clocks), list(reasons), 0

    def sm_max_mhz(self):
        return 2070

    def sm_mhz(self):
        return self.clocks[min(self.k, len(self.clocks) - 1)]

    def reasons(self):
        r = self.reasons_seq[min(self.k, len(self.reasons_seq) - 1)]
        self.k += 1
        return r


def test_nvml_sampler_records_clocks_and_reasons_inside_the_region():
    import time
    import bench
    api = _FakeNvml([2070, 2055, 2070, 2070], [0, 0x4, 0, 0])   # one sample under the power cap
    with bench.NvmlClocks(api, period=0.001) as c:
        time.sleep(0.02)
    s = c.summary()
    assert s["samples"] >= 4 and s["sm_max_mhz"] == 2070
    assert s["sm_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"]


def test_nvml_sampler_names_slowdowns():
    import bench
    api = _FakeNvml([1200], [0x8 | 0x40 | 0x20])
    with bench.NvmlClocks(api, period=0.001) as c:
        pass
    assert c.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_sampler_falls_back_to_nvidia_smi_without_nvml():
    import bench

    class NoDevice:
        class cuda:
            @staticmethod
            def get_device_properties(i):
                raise RuntimeError("no CUDA device")
    assert isinstance(bench.clock_sampler(NoDevice, 0), bench.ClockSampler)
