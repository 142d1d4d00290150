"""Host-side pieces of bench.py on the CPU: the clock record taken from
nvidia-smi during the timed region (median SM clock, maximum clock, throttle
reasons seen, this GPU's rows only) and the peak bandwidth it divides by."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

NA = "Not Active"


def _row(idx, sm, reasons=()):
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    return [str(idx), sm, "2070", "900.5", "0x0"] + ["Active" if n in reasons else NA for n in names]


def test_clock_summary_takes_this_gpus_rows():
    cs = bench.ClockSampler(gpu_index=1)
    cs.rows = [_row(0, "1200", ("hw_slowdown",)), _row(1, "2070"), _row(1, "2050", ("sw_power_cap",)),
               _row(1, "2060"), ["1", "2070"]]  # a cut-off line is left out
    s = cs.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2060.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]  # GPU 0's slowdown is another GPU's


def test_clock_summary_of_one_gpu_and_unreadable_clocks():
    cs = bench.ClockSampler(gpu_index=0)
    cs.rows = [_row(3, "[N/A]", ("hw_thermal_slowdown",)), _row(3, "1995")]
    s = cs.summary()  # one GPU visible: its rows are taken whatever its index
    assert s["samples"] == 2 and s["sm_mhz"] == 1995.0 and s["reasons"] == ["hw_thermal_slowdown"]


def test_clock_summary_without_nvidia_smi():
    s = bench.ClockSampler().summary()
    assert s["samples"] == 0 and s["sm_mhz"] is None and s["reasons"] == ["nvidia-smi unavailable"]


def test_peak_bandwidth_source():
    v, src = bench.measured_peaks()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        assert src == "measured" and 1000.0 < v < 20000.0
    else:
        assert (v, src) == (6800.0, "fallback")
