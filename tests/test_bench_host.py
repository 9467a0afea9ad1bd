"""bench.py's host-side logic on the CPU: the summary of the nvidia-smi clock
samples that decides whether a run's clocks are acceptable, and the lookups
of the roofline's denominators and DRAM traffic."""
import json

import bench
from glemur_gb300 import configs

ROW = "0, {sm}, 2070, 850.10, 0x0000000000000000, {hw}, Not Active, Not Active, {cap}"


def _clocks(text, sampled=True):
    c = bench.Clocks.__new__(bench.Clocks)
    c.proc = object() if sampled else None
    c.text = text
    return c


def test_clock_summary_median_and_reasons():
    rows = [ROW.format(sm=s, hw="Not Active", cap="Not Active") for s in (2070, 2055, 2070, 1980, 2070)]
    s = _clocks("\n".join(rows)).summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 5}
    rows.append(ROW.format(sm=1800, hw="Active", cap="Active"))
    s = _clocks("\n".join(rows)).summary()
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"] and s["samples"] == 6


def test_clock_summary_without_samples():
    assert _clocks("", sampled=False).summary()["reasons"] == ["unsampled"]
    assert _clocks("garbage\n[N/A]\n").summary()["reasons"] == ["unsampled"]
    # unreadable clock values are left out of the median, the row still counts
    s = _clocks(ROW.format(sm="[N/A]", hw="Not Active", cap="Not Active")).summary()
    assert s["sm_mhz"] is None and s["samples"] == 1


def test_peak_and_traffic_lookups():
    peak, kind = bench.peaks()
    f = bench.ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        assert kind == "measured" and peak == float(json.loads(f.read_text())["hbm_gbs"])
    else:
        assert (peak, kind) == (6800.0, "fallback")
    # the bench workload has a measured per-launch figure
    t, src = bench.traffic_per_launch(configs.braid6(128, 128, 256, precision=32))
    assert t == 338378880.0 and "k_stage_tma_braid6_128x128x256" in src
    # a larger pressure grid scales the per-point figure with the inner points
    p = configs.braid6_large(256, 256, 512, precision=32)
    t, src = bench.traffic_per_launch(p)
    assert abs(t - 80.211 * 256 * 256 * 512) < 1e3
