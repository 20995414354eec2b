"""CPU tests of bench.py's host logic: the roofline inputs read from the
committed profile summary and their staleness check against the kernel
sources, the clock summaries (nvidia-smi lines and NVML samples, with the
throttle reasons that reject a run), the CUDA-to-NVML device mapping, and the
algorithmic bytes per sweep.
"""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_profile_inputs_are_current_and_detect_changes(monkeypatch):
    prof = bench.profile_inputs()
    assert prof["stale"] is False, "profiles/ no longer matches the kernel sources"
    assert 40e6 < prof["dram_bytes_per_launch"] < 50e6
    assert 40 < prof["thread_inst_per_update"] < 80
    # sources that changed since the capture make the figures stale
    monkeypatch.setattr(bench, "kernel_sources_hash", lambda: "0123456789abcdef")
    assert bench.profile_inputs()["stale"] is True


def test_clock_summary_from_nvidia_smi_lines():
    c = bench.Clocks(0)
    c.lines = ["2070, 2070, 900.1, Not Active, Not Active, Not Active, Not Active",
               "2055, 2070, 950.0, Not Active, Not Active, Not Active, Active",
               "garbage", "1980, 2070, 1000, Not Active, Active, Not Active, Not Active"]
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2055 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_summary_from_nvml_samples():
    class FakeNvml:
        max_mhz = 2070.0

    c = bench.Clocks(0)
    c.nvml = FakeNvml()
    c.samples = [(2070.0, set()), (2070.0, {"sw_power_cap"}), (2040.0, set())]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3,
                 "reasons": ["sw_power_cap"], "source": "NVML, 1 ms"}
    assert bench._Nvml.BITS[0x8] == "hw_slowdown" and bench._Nvml.BITS[0x40] == \
        "hw_thermal_slowdown" and bench._Nvml.BITS[0x20] == "sw_thermal_slowdown"


@pytest.mark.parametrize("env,index,want", [(None, 0, "0"), ("3", 0, "3"), ("5,2", 1, "2"),
                                            ("GPU-aa,GPU-bb", 1, "GPU-bb")])
def test_clock_device_follows_cuda_visible_devices(monkeypatch, env, index, want):
    if env is None:
        monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    else:
        monkeypatch.setenv("CUDA_VISIBLE_DEVICES", env)
    assert bench.Clocks(index).index == want


def test_sweep_bytes_brain_study():
    # outcome bits + beta read/write + Omega pass + FP64 sums + lattice
    N, V, P, S = 1000, 230261, 5, 1
    b = bench.sweep_bytes(N, V, P, S)
    assert b == N * V // 8 + 8 * P * V + 4 * P * V + 5 * V + 2 * 8 * (2 * P + S) * V
    assert 80e6 < b < 90e6
