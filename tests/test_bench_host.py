"""Host-side parts of bench.py that need no GPU: the summary of the clock
samples taken during the timed region."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))

import bench  # noqa: E402


def _row(sm, smax, hw="Not Active", hwt="Not Active", swt="Not Active", pcap="Not Active"):
    return f"0, {sm}, {smax}, 950.12, 0x0000000000000000, {hw}, {hwt}, {swt}, {pcap}"


def test_clock_summary_median_max_and_reasons():
    text = "\n".join([_row(2070, 2070), _row(2055, 2070, pcap="Active"), _row(1980, 2070),
                      _row(2070, 2070, hwt="Active")])
    c = bench.ClockSampler.summarize(text)
    assert c["sm_mhz"] == 2062.5 and c["sm_max_mhz"] == 2070.0 and c["samples"] == 4
    assert c["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_summary_skips_malformed_rows():
    text = "\n".join(["[N/A]", _row("[N/A]", 2070), _row(2070, 2070), ""])
    c = bench.ClockSampler.summarize(text)
    assert c["samples"] == 1 and c["sm_mhz"] == 2070.0 and c["reasons"] == []
    assert bench.ClockSampler.summarize("")["reasons"] == ["no samples"]


def test_clock_sampler_without_nvidia_smi_leaves_no_file(monkeypatch):
    monkeypatch.delenv("SL_CLOCKS_DIR", raising=False)
    s = bench.ClockSampler(0)
    s.proc = None  # as when nvidia-smi cannot be started
    assert s.stop()["reasons"] == ["nvidia-smi unavailable"]
    assert not s.path.exists()
