"""CPU tests of bench.py's host-side measurement logic: the clocks record,
the algorithmic bytes of the roofline, and the traffic read from the
committed ncu summaries."""
from __future__ import annotations

import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def test_clock_summary_median_max_and_reasons():
    out = "\n".join([
        "0, 2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1380.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ])
    c = bench.ClockSampler.summarize(out)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_summary_flags_slowdowns():
    out = ("0, 1200, 2070, 700.0, 0x0000000000000008, Active, Not Active, Not Active, Not Active\n"
           "0, 1100, 2070, 650.0, 0x0000000000000040, Not Active, Active, Active, Not Active\n")
    c = bench.ClockSampler.summarize(out)
    assert c["sm_mhz"] == 1150.0
    assert c["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert bench.ClockSampler.summarize("") is None


def test_algorithmic_bytes_per_pass():
    # 1M particles, c = cells / particle = 0.5: lambda 20 + 8c, delta_p 36 + 8c bytes per particle
    a = bench.algorithmic_bytes(1 << 20, 1 << 19)
    assert a == {"lambda": (1 << 20) * 24.0, "delta_p": (1 << 20) * 40.0}


def test_traffic_from_committed_summary():
    t = bench.ncu_traffic("delta_p")
    assert t is not None and 1e6 < t < 1e9
    assert bench.ncu_traffic("no_such_kernel") is None


def test_fp32_roofline():
    # 1M particles, 4 iterations: 27 (240 + 15) = 6,885 flops per particle-step
    r = bench.fp32_roofline(1 << 20, 240, 240 * 2.5, 152, 2070.0, 4)
    assert r["algorithmic_flops_per_step"] == 6885 * (1 << 20)
    assert abs(r["achieved"] - 6885 * (1 << 20) / 2.5e-3 / 1e12) < 1e-9
    assert abs(r["peak"] - 152 * 256 * 2070e6 / 1e12) < 1e-9 and 0 < r["frac"] < 1
    assert bench.fp32_roofline(1000, 10, 5.0, None, None)["frac"] is None


def test_reference_arm_loads_no_product_library():
    """bench.py --impl reference runs the CPU port only: after a small run the
    process has not mapped libpbf.so (the product's CUDA library)."""
    import subprocess

    code = ("import sys; sys.argv = ['bench.py']; import bench; "
            "bench.main(['--impl', 'reference', '--scene', 'dam_break', '--steps', '2', '--warmup', '3', "
            "'--cpu-budget', '1']); "
            "maps = open('/proc/self/maps').read(); "
            "assert 'libpbf' not in maps, 'libpbf mapped'; print('NO_LIBPBF')")
    r = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "NO_LIBPBF" in r.stdout
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][0]
    import json

    d = json.loads(line)
    assert d["impl"] == "reference" and d["steps"] >= 1 and d["warmup"] == 3
    assert d["steps_timed"][0] == 4
