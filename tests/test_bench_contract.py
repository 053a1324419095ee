"""The benchmark's reference arm on the host (no GPU): `bench.py --impl
reference` times complete solves by the reference algorithm (the oracle port)
of a body small enough to finish in seconds, nothing scaled, and prints one
JSON line with the fields the benchmark contract names."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--cpu-seconds", "2"], capture_output=True, text=True, timeout=600,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["unit"] == "solves/s" and d["higher_is_better"] is True
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "workload" in d["config"] and "complete solves" in d["config"]["workload"]
    assert "nothing scaled" in cb["sample"]
    # the reference's serial path beside it: the same solve with the integration on one thread
    st = d["single_thread"]
    assert st["cores"] == 1 and 0 < st["solves_per_s"] <= d["value"] * 1.2
    # the timed region is the run's own: steps x ms_per_step within the host time
    assert d["steps"] * d["ms_per_step"] / 1000.0 <= d["host_s"] * 1.001


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_record_summary():
    """The clocks object of the JSON line from nvidia-smi's CSV samples: median SM
    clock under load, the maximum, and every throttle reason seen active."""
    B = _bench_module()
    cs = B.ClockSampler(0)
    cs.out = ("2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
              "2055, 2070, 1350.2, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
              "1980, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
              "[N/A], 2070, 10, 0x0, Not Active, Not Active, Not Active, Not Active\n")
    s = cs.summary()
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]
    cs.out = "2070, 2070, 900, 0x0, Active, Not Active, Active, Not Active\n"
    assert cs.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]
    cs.out = None
    assert cs.summary()["sm_mhz"] is None


def test_measured_peaks_source():
    B = _bench_module()
    peak, kind = B.measured_peaks()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            assert peak == float(json.load(f)["hbm_gbs"]) and kind == "measured"
    else:
        assert (peak, kind) == (6800.0, "fallback")


def test_measured_bf16_peak_source():
    B = _bench_module()
    peak, kind = B.measured_peaks("bf16_tflops")
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            assert peak == float(json.load(f)["bf16_tflops"]) and kind == "measured"
    else:
        assert (peak, kind) == (1900.0, "fallback")


def test_profile_traffic_figures_present():
    """The DRAM traffic that the headline and batch lines report comes from the
    committed ncu summaries: both files carry their machine-readable line."""
    B = _bench_module()
    with open(B.PROFILE_TRAFFIC) as f:
        t = [float(l.split(":")[1]) for l in f if l.startswith("traffic_bytes_per_launch_k_avp_c2:")]
    assert len(t) == 1 and 1.0e10 < t[0] < 1.1e10  # 10.38 GB of packed matrix per launch, read once
    with open(B.PROFILE_BATCH) as f:
        r = [float(l.split(":")[1]) for l in f if l.startswith("traffic_ratio_gb_avp_b16:")]
    assert len(r) == 1 and 1.0 <= r[0] < 1.1
