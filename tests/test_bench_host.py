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
    cb = bench.measure_cpu_baseline(spec, min_seconds=0.05, max_runs=3)
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
