"""bench.py's host-side pieces without a GPU: the CPU baseline (the oracle
on the host cores) reports a well-formed object on a small workload."""
import importlib
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_baseline_object(wl, oracle):
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    spec = wl.config0(out=32, ex=16)
    cb, parity = bench.measure_cpu_baseline(spec, min_seconds=0.05, max_runs=3)
    assert parity == "not checked"
    assert cb["kind"] == "port" and cb["unit"] == "Mpx/s"
    assert cb["value"] > 0 and cb["cores"] >= 1
    assert "full runs" in cb["sample"]


def test_tuning_dict_keys():
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")

    class T:
        team_max_items, team_full_max_items, walk_window_max_items, trials, gpu_ms, default_gpu_ms = 1, 2, 3, 4, 5.0, 6.0

    d = bench._tuning_dict(T())
    assert d == {"team_max_items": 1, "team_full_max_items": 2, "walk_window_max_items": 3, "trials": 4,
                 "tuned_ms": 5.0, "default_ms": 6.0}


def test_reference_arm_line():
    """bench.py --impl reference prints one JSON line with the contract's
    keys (the oracle port on the host cores; no GPU needed)."""
    import json
    import subprocess

    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_parity_check_in_cpu_baseline(wl, oracle):
    """The CPU-baseline leg compares a run's outputs with the oracle's: an
    identical copy reads bit-exact, a planted change to the copy is named."""
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    spec = wl.config0(out=24, ex=16)
    ref = oracle.run(spec, nthreads=2)
    _, parity = bench.measure_cpu_baseline(spec, min_seconds=0.0, max_runs=1, check=ref)
    assert parity == "bit-exact"
    bad = dict(ref)
    bad["image"] = ref["image"].copy()
    bad["image"][3, 5, 1] ^= 1
    _, parity = bench.measure_cpu_baseline(spec, min_seconds=0.0, max_runs=1, check=bad)
    assert parity.startswith("MISMATCH") and "image (1 places)" in parity


def test_config_same_in_both_arms(wl):
    sys.path.insert(0, ROOT)
    bench = importlib.import_module("bench")
    spec = bench.workload()
    assert bench.bench_config(spec) == bench.bench_config(wl.config1())
    assert bench.bench_config(spec)["workload"] == "multi_example_tiling_512"
