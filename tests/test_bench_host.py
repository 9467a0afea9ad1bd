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


def test_nvml_sampler_summary_and_fallback():
    """The NVML sampler's summary (median SM clock, clock-event reason bits
    decoded), and its behaviour without NVML: no thread, no summary, so the
    bench line falls back to the nvidia-smi record."""
    c = bench.NvmlClocks.__new__(bench.NvmlClocks)
    c.lib, c.max_mhz = None, 2070.0
    c.samples = [(2070.0, 0), (2055.0, 0x4), (2070.0, 0)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"] and s["sampler"].startswith("nvml")
    c.samples.append((1500.0, 0x8 | 0x40))
    assert c.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap"]
    c.samples = []
    assert c.summary() is None
    # a library that is not there: the context manager starts nothing
    n = bench.NvmlClocks.__new__(bench.NvmlClocks)
    n.lib, n.samples = None, []
    with n as ck:
        pass
    assert ck.thread is None and ck.summary() is None


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


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (the reference's arithmetic on the host
    cores) prints one JSON line with the keys the benchmark contract names,
    on the same metric, unit and workload as the GPU arm."""
    import subprocess
    import sys
    r = subprocess.run([sys.executable, str(bench.ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=bench.ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["grid"] == [128, 128, 256]


def test_reference_arm_loads_no_product_library():
    """The reference arm builds its parameters and initial state with the
    oracle: the product library is never loaded in that process."""
    import subprocess
    import sys
    code = ("import sys, runpy; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3'];\n"
            "try:\n    runpy.run_path('bench.py', run_name='__main__')\nexcept SystemExit:\n    pass\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('LOADED_LIBGLEMUR' if 'libglemur.so' in maps else 'CLEAN')\n"
            "print('IMPORTED_PACKAGE' if any(m.startswith('glemur_gb300') for m in sys.modules) else 'NO_PACKAGE')")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=bench.ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "CLEAN" in r.stdout and "NO_PACKAGE" in r.stdout, r.stdout[-500:]
