"""Benchmark of the synthesis hot loop on one GB300.

Workload: multi-example remix with tiling (4 x 300^2 RGBA8 examples from
seeds 1-4, random_init 10, seed 211, k = m = 50, 512^2 output) -- the
configuration the headline metric is quoted on.  A step is one
Session::run() over one session.

  value  output Mpx/s with the inputs already on the device when the timed
         region starts (sessions built beforehand); device time measured
         with CUDA events on the launching stream inside run()
  e2e    the same metric through the C ABI with host buffers: build (input
         upload, pyramids) + run + reading the image back, per step
  roofline  the resolve kernel (dominant) measured with per-launch CUDA
         events in a separate profiled pass
  cpu_baseline  the CPU oracle (a C port of the reference's algorithm) on
         the host cores, one full run of the same workload

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PKG = "texture-synthesis_gb300"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0


def _peaks():
    try:
        with open(PEAKS) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                for line in out.stdout.strip().splitlines():
                    self.rows.append([c.strip() for c in line.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for i, n in enumerate(names):
                    if r[5 + i].lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def workload():
    wl = importlib.import_module(PKG + ".workloads")
    return wl.config1()


def run_reference_arm(args):
    """The reference's algorithm on the host CPU cores: the oracle port (the
    Rust reference cannot be built on this machine), all host threads."""
    from oracle import oracle

    spec = workload()
    threads = os.cpu_count() or 1
    oracle.run(spec, nthreads=threads)  # warm-up of the library and caches
    times = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        r = oracle.run(spec, nthreads=threads)
        times.append(time.perf_counter() - t0)
    px = spec["out_w"] * spec["out_h"]
    sec = sum(times) / len(times)
    value = px / sec / 1e6
    line = {
        "impl": "reference", "metric": "output Mpx/s", "value": value, "unit": "Mpx/s", "n_gpus": args.gpus,
        "steps": len(times), "warmup": 1, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": spec["name"], "out": [spec["out_w"], spec["out_h"]], "examples": 4,
                   "k": 50, "m": 50, "batch_divisor": 8},
        "cpu_baseline": {"value": value, "unit": "Mpx/s", "cores": threads, "kind": "port",
                         "sample": "full runs of the workload, batch-snapshot schedule, %d threads" % threads},
        "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cost_evals_per_s": r["evals"] / sec,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--once", action="store_true", help="build and run one session, print its stats (for profilers)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args)
        return

    importlib.import_module(PKG + ".build").build()
    ts = importlib.import_module(PKG)
    import numpy as np

    spec = workload()
    px = spec["out_w"] * spec["out_h"]
    if args.once:
        g = ts.builder_from_spec(spec).build().run()
        print(json.dumps(g.stats()))
        return
    # --- device-resident throughput: sessions built before the timed region
    for _ in range(args.warmup):
        ts.builder_from_spec(spec).build().run()
    sessions = [ts.builder_from_spec(spec).build() for _ in range(args.steps)]
    gpu_ms, evals, launches = [], [], []
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for s in sessions:
            g = s.run()
            st = g.stats()
            gpu_ms.append(st["gpu_ms"])
            evals.append(st["cost_evals"])
            launches.append(st["kernel_launches"])
        wall = time.perf_counter() - t0
    ms = sum(gpu_ms) / len(gpu_ms)
    value = px * len(gpu_ms) / (sum(gpu_ms) / 1e3) / 1e6
    # --- end to end through the C ABI with host buffers
    e2e_t = []
    h2d = sum(e["image"].nbytes for e in spec["examples"])
    d2h = px * 4
    for _ in range(max(1, min(args.steps, 5))):
        t1 = time.perf_counter()
        g = ts.builder_from_spec(spec).build().run()
        img = g.into_image()
        e2e_t.append(time.perf_counter() - t1)
    e2e = px / (sum(e2e_t) / len(e2e_t)) / 1e6
    peak, peak_kind = _peaks()
    # --- roofline of the dominant kernel: a separate pass with CUDA events
    # around every launch on the launching stream
    prof = ts.builder_from_spec(spec, profile=True).build().run().stats()
    kern = prof["kernels"]
    top = max(kern, key=lambda n: kern[n]["ms"])
    res = kern["resolve"]
    k = spec["params"]["nearest_neighbors"]
    per_eval = 4 * k * (2 if spec.get("target_guide") is not None else 1)
    alg_bytes = prof["cost_evals"] * per_eval  # example texels every candidate-cost evaluation reads
    achieved = alg_bytes / (res["ms"] / 1e3) / 1e9
    roofline = {"kernel": "k_resolve", "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": None,
                "alg_bytes_per_launch": alg_bytes / max(1, res["launches"]),
                "avg_launch_ms": res["ms"] / max(1, res["launches"]), "launches": res["launches"],
                "kernel_share": {n: kern[n]["ms"] / max(1e-9, sum(v["ms"] for v in kern.values())) for n in kern},
                "top_kernel": top}
    line = {
        "metric": "output Mpx/s", "value": value, "unit": "Mpx/s", "n_gpus": world, "steps": len(gpu_ms),
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": {"workload": spec["name"], "out": [spec["out_w"], spec["out_h"]], "examples": 4, "k": 50,
                   "m": 50, "batch_divisor": 8, "l2": "working set (examples 1.4 MB) L2-resident by design"},
        "cost_evals_per_s": sum(evals) / (sum(gpu_ms) / 1e3),
        "gpu_launches": int(sum(launches) / len(launches)),
        "wall_ms_per_step": wall / len(gpu_ms) * 1e3,
        "clocks": clk.summary(),
        "e2e": {"value": e2e, "unit": "Mpx/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "roofline": roofline,
        "cpu_baseline": None,
    }
    if not args.no_cpu_baseline and rank == 0:
        from oracle import oracle

        threads = os.cpu_count() or 1
        t2 = time.perf_counter()
        oracle.run(spec, nthreads=threads)
        sec = time.perf_counter() - t2
        line["cpu_baseline"] = {"value": px / sec / 1e6, "unit": "Mpx/s", "cores": threads, "kind": "port",
                                "sample": "one full run of the workload"}
    print(json.dumps(line))


if __name__ == "__main__":
    main()
