"""Benchmark of the synthesis hot loop on one GB300.

Workload: multi-example remix with tiling (4 x 300^2 RGBA8 examples from
seeds 1-4, random_init 10, seed 211, k = m = 50, 512^2 output) -- the
configuration the headline metric is quoted on.  A step is one
Session::run() over one session.

  value  output Mpx/s with the inputs already on the device when the timed
         region starts (sessions built beforehand); device time measured
         with CUDA events on the launching stream inside run(); L2 is
         flushed (a 256 MB device write) between timed steps
  e2e    the same metric through the C ABI with host buffers: build (input
         upload, pyramids) + run + reading the image back, per step
  roofline  the resolve kernels (dominant) measured with per-launch CUDA
         events in a separate profiled pass, against the measured gather
         ceiling (ts_measure_gather_peak: patch-shaped 32-bit gathers from a
         table the size of the workload's example level), with the HBM copy
         bandwidth beside it
  parity the last timed run's outputs against the oracle's, bit for bit,
         inside the CPU-baseline leg (outside every timed region)
  config0, config2  the single-example 256^2 and guided 512^2 workloads,
         measured the same way (value, e2e, roofline)
  cpu_baseline  the CPU oracle (a C port of the reference's algorithm) on
         the host cores: whole runs of the same workload, repeated for
         about 10 s
  batched  64 sessions of the batched mix (uneven sizes, k and m from
         {8, 20, 50}, a quarter guided), one after another on the plain
         path and together through the batched form: aggregate Mpx/s
  tuning   the launch-shape thresholds the autotuner picked on the workload
         before any timing (ts_autotune_session); the batched and served
         forms use those ts_autotune_batch picked on the batched mix
  served   a Poisson request stream from the batched mix (70%) and 512^2
         inpainting requests (30%), 256 requests at each of 10, 25, 50, 100
         and 200 req/s, through the served form and, for comparison,
         through the plain path one request at a time: p50/p99 latency from
         arrival to result and aggregate Mpx/s; then all 256 submitted at
         once (saturation: the served form's aggregate throughput)

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--workload remix|single|guided|batched|served]
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
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# resolve family (k_resolve_lean, k_resolve_team) on this workload: 993.2 MB
# over the 131 resolve launches of one run (profiles/resolve_dram_multi_example_512.md),
# from
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum
#       --clock-control none -k regex:"k_resolve" --csv python bench.py --once
# (one pass; ncu flushes the caches before each launch, so this is a
# cold-cache upper bound of the live traffic).
RESOLVE_DRAM_BYTES_PER_LAUNCH = 993.2e6 / 131
# The load path, measured in the unit both kernels share: 32-byte L1 sectors
# requested per second by global loads (l1tex__t_sectors_pipe_lsu_mem_global_op_ld.sum
# / gpu__time_duration.sum).  k_resolve_lean on a 26,248-item step of this
# workload against ts_measure_gather_peak's patch kernel on this workload's
# table (profiles/k_resolve_lean_multi_example_512.md and
# profiles/gather_peak_probe_multi_example_512.md, ncu, one launch each).
LOAD_PATH_SECTORS_PER_S = {"k_resolve_lean": 137.0e9, "gather_probe": 405.4e9}


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

    def __init__(self, index=0, period_ms=50):
        self.index = index
        self.period_ms = period_ms
        self.rows = []
        self._p = None

    def __enter__(self):
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                        "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.3)  # first sample before the timed region
        except Exception:
            self._p = None
        return self

    def __exit__(self, *a):
        if self._p is None:
            return
        self._p.terminate()
        try:
            out, _ = self._p.communicate(timeout=10)
        except Exception:
            self._p.kill()
            out, _ = self._p.communicate()
        for line in (out or "").strip().splitlines():
            self.rows.append([c.strip() for c in line.split(",")])

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


class L2Flush:
    """Writes a 256 MB device buffer (L2 is 129 MB) between timed steps."""

    def __init__(self):
        self.buf = None
        try:
            import torch

            if torch.cuda.is_available():
                self.torch = torch
                self.buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda:0")
        except Exception:
            self.buf = None

    def __call__(self):
        if self.buf is not None:
            self.buf.fill_(1.0)
            self.torch.cuda.synchronize()


def _tuning_dict(t):
    return {"team_max_items": t.team_max_items, "team_full_max_items": t.team_full_max_items,
            "walk_window_max_items": t.walk_window_max_items, "trials": t.trials,
            "tuned_ms": t.gpu_ms, "default_ms": t.default_gpu_ms}


_T0 = time.perf_counter()


def _progress(msg):
    """One line on stderr per finished part of the run (stdout keeps the
    JSON line alone)."""
    print("[bench %7.1f s] %s" % (time.perf_counter() - _T0, msg), file=sys.stderr, flush=True)


def _pct(v, q):
    import numpy as np

    return float(np.percentile(np.asarray(v, dtype=np.float64), q))


def measure_batched(ts, wl, n=64):
    """Config 3: the plain path one session after another vs the batched
    form, on the same 64 sessions (built before timing)."""
    specs = wl.config3_sessions(n)
    for s in specs[:2]:
        ts.builder_from_spec(s).build().run()
    px = sum(s["out_w"] * s["out_h"] for s in specs)
    sess = [ts.builder_from_spec(s).build() for s in specs]
    t0 = time.perf_counter()
    gpu = 0.0
    for s in sess:
        gpu += s.run().stats()["gpu_ms"]
    plain_wall = time.perf_counter() - t0
    del sess
    # the batched form's team thresholds, tuned on this mix after the plain
    # runs (which keep the defaults) and before the timed batched runs
    tuning = ts.autotune_batch(lambda: [ts.builder_from_spec(s).build() for s in specs], repeats=2)
    best = None
    for _ in range(2):
        b = ts.Batch(tuning=tuning)
        for s in specs:
            b.add(ts.builder_from_spec(s).build())
        t1 = time.perf_counter()
        b.run()
        wall = time.perf_counter() - t1
        st = b.stats()
        if best is None or st["gpu_ms"] < best[0]["gpu_ms"]:
            best = (st, wall)
    st, wall = best
    return {"workload": "batched_mix_64", "sessions": n, "output_mpx": px / 1e6,
            "plain": {"mpx_s": px / (gpu / 1e3) / 1e6, "wall_mpx_s": px / plain_wall / 1e6, "gpu_ms": gpu},
            "batched": {"mpx_s": px / (st["gpu_ms"] / 1e3) / 1e6, "wall_mpx_s": px / wall / 1e6,
                        "gpu_ms": st["gpu_ms"], "steps": st["steps"], "launches": st["launches"],
                        "plan_ms": st["plan_ms"]},
            "cost_evals_per_s": st["cost_evals"] / (st["gpu_ms"] / 1e3), "tuning": _tuning_dict(tuning)}, tuning


def serve_stream(ts, reqs, served=True, max_active=64, tuning=None):
    """A request stream [(arrival_s, spec)]: sessions are built at arrival on
    a client thread; latency runs from the arrival to the result on the
    host.  served=False: the plain path, one request at a time, FIFO."""
    n = len(reqs)
    lat = [0.0] * n
    px = [0] * n
    t_start = time.perf_counter() + 0.05
    if served:
        srv = ts.Server(max_active=max_active, tuning=tuning)
        tickets = [None] * n
        ready = [threading.Event() for _ in range(n)]
        sub_py = [0.0] * n

        def client():
            for i, (t, spec) in enumerate(reqs):
                d = t_start + t - time.perf_counter()
                if d > 0:
                    time.sleep(d)
                s = ts.builder_from_spec(spec).build()
                sub_py[i] = time.perf_counter()
                tickets[i] = srv.submit(s)
                ready[i].set()

        th = threading.Thread(target=client)
        th.start()
        for i in range(n):
            ready[i].wait()
            g, times = srv.wait(tickets[i])
            done = sub_py[i] + (times["done_ms"] - times["submit_ms"]) / 1e3
            lat[i] = done - (t_start + reqs[i][0])
            px[i] = g.width * g.height
        th.join()
        st = srv.stats()
        srv.close()
    else:
        st = None
        for i, (t, spec) in enumerate(reqs):
            d = t_start + t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            g = ts.builder_from_spec(spec).build().run()
            lat[i] = time.perf_counter() - (t_start + t)
            px[i] = g.width * g.height
    span = max(reqs[i][0] + lat[i] for i in range(n)) - reqs[0][0]
    out = {"requests": n, "p50_ms": _pct(lat, 50) * 1e3, "p99_ms": _pct(lat, 99) * 1e3,
           "mean_ms": sum(lat) / n * 1e3, "mpx_s": sum(px) / span / 1e6}
    if st is not None:
        out["peak_active"] = st["peak_active"]
        out["ticks"] = st["ticks"]
    return out


def serve_saturated(ts, reqs, max_active=64, tuning=None):
    """Every request of the stream submitted at once to the served form, its
    sessions built beforehand: the server's aggregate throughput with work
    always waiting (beside it, the batched form's on the 64-session mix)."""
    sessions = [ts.builder_from_spec(spec).build() for _, spec in reqs]
    px = sum(spec["out_w"] * spec["out_h"] for _, spec in reqs)
    srv = ts.Server(max_active=max_active, tuning=tuning)
    t0 = time.perf_counter()
    tickets = [srv.submit(s) for s in sessions]
    lat = []
    for t in tickets:
        srv.wait(t)
        lat.append(time.perf_counter() - t0)
    span = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return {"requests": len(reqs), "mpx_s": px / span / 1e6, "span_ms": span * 1e3,
            "p50_ms": _pct(lat, 50) * 1e3, "p99_ms": _pct(lat, 99) * 1e3,
            "peak_active": st["peak_active"], "ticks": st["ticks"],
            "driver_ms": {"ticks": st["driver_tick_us"] / 1e3, "ring_wait": st["driver_ring_wait_us"] / 1e3,
                          "pick_wait": st["driver_pick_wait_us"] / 1e3, "launch_calls": st["driver_launch_us"] / 1e3}}


def measure_served(ts, wl, lams=(10, 25, 50, 100, 200), n=256, tuning=None):
    """Config 4: the Poisson stream through the served form and through the
    plain path at each arrival rate (n requests each), then the whole
    stream at once (saturation)."""
    warm = wl.config4_requests(6, 1000.0, seed=99)
    serve_stream(ts, warm, True, tuning=tuning)
    rows = []
    for lam in lams:
        reqs = wl.config4_requests(n, float(lam))
        rows.append({"lambda_req_s": lam, "served": serve_stream(ts, reqs, True, tuning=tuning)})
        _progress("served stream at %g req/s" % lam)
        rows[-1]["plain"] = serve_stream(ts, reqs, False)
        _progress("plain stream at %g req/s" % lam)
    sat = serve_saturated(ts, wl.config4_requests(n, 1e6), tuning=tuning)
    _progress("served saturation")
    return {"workload": "served_mix", "mix": "70% batched mix, 30% 512^2 inpainting",
            "requests_per_rate": n, "rates": rows, "saturated": sat}


def measure_cpu_baseline(spec, min_seconds=10.0, max_runs=20, check=None):
    """The oracle (the C port of the reference's algorithm) on every host
    core: whole runs of the workload, repeated until min_seconds of CPU
    work (at most max_runs runs).  With `check` (a GPU run's outputs), the
    first oracle run's outputs are also compared with it bit for bit; the
    second value returned says how that went."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    px = spec["out_w"] * spec["out_h"]
    runs, sec = 0, 0.0
    parity = "not checked"
    while runs < max(1, max_runs) and (runs == 0 or sec < min_seconds):
        t0 = time.perf_counter()
        r = oracle.run(spec, nthreads=threads)
        sec += time.perf_counter() - t0
        if runs == 0 and check is not None:
            parity = compare_outputs(check, r)
        runs += 1
    return ({"value": px * runs / sec / 1e6, "unit": "Mpx/s", "cores": threads, "kind": "port",
             "sample": "%d full runs of the workload (%.1f s), %d threads" % (runs, sec, threads)}, parity)


def compare_outputs(got, ref):
    """'bit-exact' when image, coordinate map, id map, resolved list, every
    f32 score (NaN-ness only for NaNs) and the eval count agree; else what
    differs."""
    import numpy as np

    bad = []
    for key in ("image", "coord", "id", "resolved", "scores"):
        a, b = np.asarray(got[key]), np.asarray(ref[key])
        if a.shape != b.shape:
            bad.append("%s shape" % key)
            continue
        if key == "scores":
            same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
        else:
            same = a == b
        if not same.all():
            bad.append("%s (%d places)" % (key, int((~same).sum())))
    if got["evals"] != ref["evals"]:
        bad.append("evals")
    return "bit-exact" if not bad else "MISMATCH: " + ", ".join(bad)


def bench_config(spec):
    """The `config` object of a bench line; the same in both arms."""
    p = spec["params"]
    return {"workload": spec["name"], "out": [spec["out_w"], spec["out_h"]], "examples": len(spec["examples"]),
            "k": p["nearest_neighbors"], "m": p["random_sample_locations"], "batch_divisor": 8,
            "guided": spec.get("target_guide") is not None,
            "l2": "GPU arm: L2 flushed between timed steps (256 MB device write)"}


def padded_level_shape(spec):
    """Width and height of one pyramid level of every example, padded as the
    cost kernel reads them (a 32-texel border, one row pitch), stacked: the
    table the gather ceiling is measured on."""
    exs = spec["examples"]
    pw = max(e["image"].shape[1] for e in exs) + 64
    ph = sum(e["image"].shape[0] + 64 for e in exs)
    return pw, ph


def gather_roofline(ts, spec, prof, peak_cache={}):
    """Roofline of the resolve family against the measured gather ceiling
    (ts_measure_gather_peak on a table the size of this workload's example
    level), with the HBM copy bandwidth beside it."""
    kern = {n: v for n, v in prof["kernels"].items() if n != "knn_wait"}  # kernels only
    res = kern["resolve"]
    k = spec["params"]["nearest_neighbors"]
    guided = spec.get("target_guide") is not None
    per_eval = 4 * k * (2 if guided else 1)
    alg_bytes = prof["cost_evals"] * per_eval  # example (+ guide) texels of every candidate-cost evaluation
    achieved = alg_bytes / (res["ms"] / 1e3) / 1e9
    shape = padded_level_shape(spec) + (k,)
    if shape not in peak_cache:
        peak_cache[shape] = ts.gather_peak(*shape, reps=5)
    gp = peak_cache[shape]
    hbm, hbm_kind = _peaks()
    top = max(kern, key=lambda n: kern[n]["ms"])
    out = {"kernel": "k_resolve family", "bound": "gather (L1/L2 load path)", "achieved": achieved,
           "peak": gp["patch_gbs"], "unit": "GB/s", "frac": achieved / gp["patch_gbs"],
           "peak_source": "measured: ts_measure_gather_peak, patch-shaped 32-bit gathers (k=%d) from a %.1f MB "
                          "table, full occupancy" % (k, gp["table_bytes"] / 1e6),
           "random_gather_gbs": gp["random_gbs"],
           "hbm_peak": hbm, "hbm_frac": achieved / hbm, "hbm_peak_source": hbm_kind,
           "alg_bytes_per_eval": per_eval,
           "alg_bytes_per_launch": alg_bytes / max(1, res["launches"]),
           "avg_launch_ms": res["ms"] / max(1, res["launches"]), "launches": res["launches"],
           "kernel_share": {n: kern[n]["ms"] / max(1e-9, sum(v["ms"] for v in kern.values())) for n in kern},
           "top_kernel": top}
    if spec["name"] == "multi_example_tiling_512":
        out["traffic"] = RESOLVE_DRAM_BYTES_PER_LAUNCH
        out["traffic_source"] = "ncu capture of this workload, cold caches, bytes per resolve launch"
        # the bytes above are the reference's; the kernel skips repeated
        # candidates and stops candidates early, so its own load-path use is
        # the fraction of the ceiling's sector rate that its loads reach
        out["load_path_frac"] = LOAD_PATH_SECTORS_PER_S["k_resolve_lean"] / LOAD_PATH_SECTORS_PER_S["gather_probe"]
        out["load_path_source"] = ("ncu: L1 sectors/s of k_resolve_lean over those of the gather probe on this "
                                   "workload's table (profiles/)")
    else:
        out["traffic"] = None
    return out


def measure_workload(ts, spec, steps, warmup, tuning, flush):
    """One workload: `value` (device-timed, sessions built beforehand), `e2e`
    (build + run + image read-back through the C ABI with host buffers), and
    the roofline of the resolve kernels from a separate profiled pass."""
    px = spec["out_w"] * spec["out_h"]
    for _ in range(warmup):
        ts.builder_from_spec(spec, tuning=tuning).build().run()
    sessions = [ts.builder_from_spec(spec, tuning=tuning).build() for _ in range(steps)]
    gpu_ms, evals, launches, walls = [], [], [], []
    last = None
    for s in sessions:
        flush()
        t0 = time.perf_counter()
        g = s.run()
        walls.append(time.perf_counter() - t0)
        st = g.stats()
        gpu_ms.append(st["gpu_ms"])
        evals.append(st["cost_evals"])
        launches.append(st["kernel_launches"])
        last = g
    outputs = ts.generated_outputs(last)  # the last timed run's outputs, read after timing
    value = px * len(gpu_ms) / (sum(gpu_ms) / 1e3) / 1e6
    e2e_t = []
    h2d = sum(e["image"].nbytes for e in spec["examples"])
    h2d += sum(e["guide"].nbytes for e in spec["examples"] if e.get("guide") is not None)
    if spec.get("target_guide") is not None:
        h2d += spec["target_guide"].nbytes
    d2h = px * 4
    parts = []
    for _ in range(max(1, min(steps, 10))):
        t1 = time.perf_counter()
        sess = ts.builder_from_spec(spec, tuning=tuning).build()
        t2 = time.perf_counter()
        g = sess.run()
        t3 = time.perf_counter()
        g.into_image()
        t4 = time.perf_counter()
        e2e_t.append(t4 - t1)
        st = g.stats()
        parts.append({"build_ms": (t2 - t1) * 1e3, "run_ms": (t3 - t2) * 1e3, "image_ms": (t4 - t3) * 1e3,
                      **{k: st[k] for k in ("host_plan_ms", "host_alloc_ms", "host_enqueue_ms", "host_pick_ms",
                                            "host_launch_ms", "host_wait_ms", "host_finish_ms", "upload_ms",
                                            "readback_ms", "gpu_ms")}})
    e2e = px / (sum(e2e_t) / len(e2e_t)) / 1e6
    breakdown = {k: sum(p[k] for p in parts) / len(parts) for k in parts[0]}
    pg = ts.builder_from_spec(spec, profile=True, tuning=tuning).build().run()
    prof = pg.stats()
    waits = [r for r in pg.launches() if r["kernel"] == "knn_wait"]
    by_stage = {}
    for r in waits:
        by_stage[str(r["stage"])] = by_stage.get(str(r["stage"]), 0.0) + r["ms"]
    return {"value": value, "unit": "Mpx/s", "steps": len(gpu_ms), "ms_per_step": sum(gpu_ms) / len(gpu_ms),
            "cost_evals_per_s": sum(evals) / (sum(gpu_ms) / 1e3), "gpu_launches": int(sum(launches) / len(launches)),
            "wall_ms_per_step": sum(walls) / len(walls) * 1e3,
            "e2e": {"value": e2e, "unit": "Mpx/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "breakdown_ms": breakdown},
            "roofline": gather_roofline(ts, spec, prof),
            "knn_ahead_waits": {"waits": len(waits), "ms": sum(r["ms"] for r in waits), "ms_by_stage": by_stage,
                                "source": "profiled run (CUDA events around every launch): the main stream's "
                                          "stalls on chunks of neighbour lists made ahead, per backtrack stage"},
            "outputs": outputs}


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
        "config": bench_config(spec),
        "cpu_baseline": {"value": value, "unit": "Mpx/s", "cores": threads, "kind": "port",
                         "sample": "full runs of the workload, batch-snapshot schedule, %d threads" % threads},
        "e2e": {"value": value, "unit": "Mpx/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cost_evals_per_s": r["evals"] / sec,
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--once", action="store_true", help="build and run one session, print its stats (for profilers)")
    ap.add_argument("--workload", default="remix",
                    choices=["remix", "single", "guided", "batched", "served", "gather_peak"],
                    help="remix: the headline line (config 1, plus configs 0 and 2, batched and served objects); "
                         "single / guided: config 0 / config 2 alone; gather_peak: the gather ceiling alone")
    ap.add_argument("--no-extra", action="store_true", help="skip the batched and served objects of the remix line")
    ap.add_argument("--out", type=int, default=0,
                    help="output side of the remix, single or guided workload instead of its own (sides that are "
                         "not powers of two take the per-step k-NN form; for profilers)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args)
        return

    importlib.import_module(PKG + ".build").build()
    ts = importlib.import_module(PKG)
    wl = importlib.import_module(PKG + ".workloads")
    if args.workload == "gather_peak":
        # the gather ceiling alone, on the remix workload's table (for profilers)
        print(json.dumps(ts.gather_peak(*padded_level_shape(workload()), 50, reps=3)))
        return
    if args.workload == "batched":
        if args.once:  # one batched run of the 64-session mix (for profilers)
            b = ts.Batch()
            for sp in wl.config3_sessions(64):
                b.add(ts.builder_from_spec(sp).build())
            b.run()
            print(json.dumps(b.stats()))
            return
        print(json.dumps({"metric": "aggregate output Mpx/s (batched form)", **measure_batched(ts, wl)[0]}))
        return
    if args.workload == "served":
        print(json.dumps({"metric": "request latency p50/p99 and aggregate Mpx/s (served form)",
                          **measure_served(ts, wl)}))
        return
    spec = {"remix": workload, "single": wl.config0, "guided": wl.config2}[args.workload]()
    if args.out:
        spec["out_w"] = spec["out_h"] = args.out
        if spec.get("target_guide") is not None:
            spec["target_guide"] = wl.target_guide(22, args.out, args.out)
    if args.workload != "remix" or args.out:
        args.no_extra = True
    if args.once:
        g = ts.builder_from_spec(spec).build().run()
        print(json.dumps(g.stats()))
        return
    # --- launch-shape thresholds tuned on this workload (before any timing)
    tuning = ts.autotune_session(lambda: ts.builder_from_spec(spec), repeats=3)
    _progress("tuned (%d trials)" % tuning.trials)
    flush = L2Flush()
    with ClockSampler(0) as clk:
        m = measure_workload(ts, spec, args.steps, args.warmup, tuning, flush)
    _progress("%s measured" % args.workload)
    outputs = m.pop("outputs")
    line = {
        "metric": "output Mpx/s", "value": m["value"], "unit": "Mpx/s", "n_gpus": world, "steps": m["steps"],
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": bench_config(spec),
        "cost_evals_per_s": m["cost_evals_per_s"],
        "gpu_launches": m["gpu_launches"],
        "wall_ms_per_step": m["wall_ms_per_step"],
        "clocks": clk.summary(),
        "e2e": m["e2e"],
        "roofline": m["roofline"],
        "knn_ahead_waits": m["knn_ahead_waits"],
        "tuning": _tuning_dict(tuning),
        "cpu_baseline": None,
        "parity": "not checked (CPU baseline skipped)",
    }
    if not args.no_extra:
        # configs 0 and 2 (single-example 256^2 and guided 512^2), their
        # launch shapes tuned on each the same way; parity tests cover them
        # at full size
        for key, sp in (("config0", wl.config0()), ("config2", wl.config2())):
            tun = ts.autotune_session(lambda sp=sp: ts.builder_from_spec(sp), repeats=3)
            with ClockSampler(0) as c2:
                r = measure_workload(ts, sp, max(3, args.steps // 2), args.warmup, tun, flush)
            r.pop("outputs")
            r["clocks"] = c2.summary()
            r["config"] = bench_config(sp)
            r["tuning"] = _tuning_dict(tun)
            line[key] = r
            _progress("%s measured" % key)
        line["batched"], btun = measure_batched(ts, wl)
        _progress("batched measured")
        line["served"] = measure_served(ts, wl, tuning=btun)
    if not args.no_cpu_baseline and rank == 0:
        line["cpu_baseline"], line["parity"] = measure_cpu_baseline(spec, check=outputs)
        _progress("cpu baseline measured")
    print(json.dumps(line))


if __name__ == "__main__":
    main()
