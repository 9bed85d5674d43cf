"""The bench's clock record: SM clocks and throttle reasons sampled through
read-only NVML queries during the timed region, checked here against a
stand-in NVML library (no GPU, no driver)."""
import time

import numpy as np

import bench


class FakeNvml:
    """Answers the five NVML queries the sampler makes; `reasons` is the
    clock-event bit mask returned from the `switch_after`-th read on."""

    def __init__(self, sm=(1980, 2070), reasons=0x0, switch_after=None):
        self.sm = list(sm)
        self.reads = 0
        self.reasons = reasons
        self.switch_after = switch_after
        self.shutdowns = 0

    def nvmlInit_v2(self):
        return 0

    def nvmlShutdown(self):
        self.shutdowns += 1
        return 0

    def nvmlDeviceGetHandleByIndex_v2(self, idx, handle):
        handle._obj.value = 1234
        return 0

    def nvmlDeviceGetMaxClockInfo(self, handle, kind, out):
        assert kind == bench.NvmlClocks.NVML_CLOCK_SM
        out._obj.value = 2070
        return 0

    def nvmlDeviceGetClockInfo(self, handle, kind, out):
        out._obj.value = self.sm[self.reads % len(self.sm)]
        self.reads += 1
        return 0

    def nvmlDeviceGetCurrentClocksEventReasons(self, handle, out):
        on = self.switch_after is None or self.reads > self.switch_after
        out._obj.value = self.reasons if on else 0
        return 0


def test_nvml_sampler_counts_samples_inside_the_region():
    lib = FakeNvml(sm=(2070,))
    nv = bench.NvmlClocks(lib, 0)
    with bench.ClockSampler(0, nvml=nv) as clk:
        time.sleep(0.03)
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == []
    # a 30 ms region polled every millisecond holds many samples, and the
    # region is bracketed by samples on both sides
    assert s["samples_in_region"] >= 5
    assert s["samples"] >= s["samples_in_region"] + 1
    assert clk.samples[0][0] <= clk.t0 and clk.samples[-1][0] >= clk.t1
    assert s["sampling"].startswith("NVML")
    assert lib.shutdowns == 1


def test_nvml_sampler_reports_throttle_reasons_by_name():
    # power cap and hardware slowdown bits
    lib = FakeNvml(reasons=0x4 | 0x8)
    with bench.ClockSampler(0, nvml=bench.NvmlClocks(lib, 0)) as clk:
        time.sleep(0.01)
    assert clk.summary()["reasons"] == ["hw_slowdown", "sw_power_cap"]
    # thermal bits; other bits (idle 0x1, application clocks 0x2) are not reasons
    lib = FakeNvml(reasons=0x20 | 0x40 | 0x1 | 0x2)
    with bench.ClockSampler(0, nvml=bench.NvmlClocks(lib, 0)) as clk:
        time.sleep(0.01)
    assert clk.summary()["reasons"] == ["hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_nvml_sampler_median_is_taken_inside_the_region():
    lib = FakeNvml(sm=(1000, 2070, 2070))
    with bench.ClockSampler(0, nvml=bench.NvmlClocks(lib, 0)) as clk:
        time.sleep(0.03)
    s = clk.summary()
    inside = [x[1] for x in clk.samples if clk.t0 <= x[0] <= clk.t1]
    assert len(inside) >= 5
    assert s["sm_mhz"] == float(np.median(inside))


def test_sampler_without_nvml_or_nvidia_smi_reports_nothing(monkeypatch):
    def no_smi(*a, **k):
        raise FileNotFoundError("nvidia-smi")
    monkeypatch.setattr(bench.subprocess, "Popen", no_smi)
    with bench.ClockSampler(0, nvml=None) as clk:
        pass
    assert clk.summary() is None


def test_lj_roofline_bytes_model():
    """The algorithmic bytes behind the headline roofline: the fused mixed
    step kernel moves 488 B per atom at K = 78 list entries (list count 4,
    FP32 shadow 16, home cell 4, the entries 4K, force written 24, velocity
    read and written 48, FP64 position read 32, next position written 32,
    next shadow written 16), of which 356 B are the force's own; the
    measured DRAM traffic of one 4M-atom launch is within 1% of it."""
    per_atom, force_only = bench.lj_kernel_bytes(78, True, 0)
    assert (per_atom, force_only) == (488, 356)
    assert bench.lj_kernel_bytes(78, True, 1) == (380, 380)
    assert bench.lj_kernel_bytes(78, False, 0)[0] == 4 + 32 + 4 + 4 * 78 + 24 + 24 + 24 + 32
    traffic = bench.profile_traffic("lj_step_mixed_full", 4_000_000) / 4_000_000
    assert abs(traffic - per_atom) / per_atom < 0.01
