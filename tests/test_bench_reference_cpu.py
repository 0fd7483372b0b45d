"""bench.py's reference arm (the reference algorithm's CPU restatement on the
host cores) runs without a GPU and prints the one JSON line the benchmark
contract asks for: impl, metric, unit, value, cpu_baseline and e2e with zero
copy bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_json_line():
    env = dict(os.environ)
    env.pop("RANK", None)
    env.pop("WORLD_SIZE", None)
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                        "--ref-seconds", "1"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "perms/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]


def test_clock_sampler_keeps_the_timed_window():
    # samples outside the marked region are dropped; throttle reasons from the
    # region are reported; unparsable timestamps fall back to all samples
    import datetime
    sys.path.insert(0, ROOT)
    import bench
    t0 = datetime.datetime(2026, 1, 2, 3, 4, 5, 0)
    def line(dt_ms, sm, reason):
        ts = (t0 + datetime.timedelta(milliseconds=dt_ms)).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
        return "%s, 0, %d, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, %s" % (ts, sm, reason)
    lines = [line(0, 1000, "Not Active"), line(500, 2070, "Active"), line(550, 2060, "Not Active"),
             line(600, 2070, "Not Active"), line(2000, 1200, "Not Active")]
    b = t0 + datetime.timedelta(milliseconds=480)
    e = t0 + datetime.timedelta(milliseconds=620)
    c = bench.ClockSampler.summarize(lines, b, e)
    assert c["samples"] == 3 and c["window"] == "timed region"
    assert c["sm_mhz"] == 2070 and c["sm_max_mhz"] == 2070 and c["reasons"] == ["sw_power_cap"]
    bad = ["garbage, 0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    c = bench.ClockSampler.summarize(bad, b, e)
    assert c["samples"] == 1 and c["window"] == "all samples"
