"""bench.py's JSON contract where it can run without a GPU: the reference arm
(the CPU implementation) prints one line with the required keys, and the
clock sampler keeps the nvidia-smi samples taken inside the timed region plus
the first one after it."""
import datetime
import importlib.util
import json
import os
import subprocess
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reference_arm_prints_the_contract_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "it/s"
    assert d["steps"] == 1 and d["warmup"] == 0 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "it/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def _line(t, sm, cap="Not Active", slow="Not Active"):
    ts = t.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return f"{ts}, 0, {sm}, 2070, 900.0, 0x0, {slow}, Not Active, Not Active, {cap}"


def test_clock_samples_are_chosen_by_timestamp():
    b = _bench()
    cs = b.ClockSampler(0)
    t = datetime.datetime(2026, 1, 1, 12, 0, 0)
    ms = datetime.timedelta(milliseconds=1)
    cs.lines = [_line(t + 200 * i * ms, 1900 + i, cap="Active" if i == 3 else "Not Active")
                for i in range(8)]
    cs.lines.insert(2, "garbage line")
    cs.t0, cs.t1 = t + 300 * ms, t + 700 * ms  # samples 2 and 3 inside, 4 right after
    cs.proc = types.SimpleNamespace(terminate=lambda: None, wait=lambda timeout=None: None,
                                    kill=lambda: None)
    r = cs.stop()
    assert r["samples_inside"] == 2 and r["samples"] == 3
    assert r["sm_mhz"] == 1903.0 and r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]


def test_clock_sampler_without_nvidia_smi():
    b = _bench()
    cs = b.ClockSampler(0)
    cs.proc = None
    r = cs.stop()
    assert r["sm_mhz"] is None and r["reasons"] == ["nvidia-smi unavailable"]
