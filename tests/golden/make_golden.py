"""Regenerates the golden fixtures in this folder from the CPU oracle.

The reference (Rust) cannot be built here, so these fixtures pin the oracle
against itself: each holds a small session's inputs (from the seeded
workload generators) and the oracle's outputs.  tests/test_golden.py checks
that the oracle still reproduces them bit for bit.  Run from the repository
root:  python tests/golden/make_golden.py
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def cases():
    wl = importlib.import_module("texture-synthesis_gb300.workloads")
    c = {}
    c["single_32"] = (wl.config0(out=32, ex=16), 8)
    s = wl.config0(out=16, ex=12)
    s["params"]["nearest_neighbors"] = 10
    s["params"]["random_sample_locations"] = 10
    c["sequential_16"] = (s, 0)
    c["multi_tiling_40"] = (wl.config1(out=40, ex=20), 8)
    c["guided_40"] = (wl.config2(out=40, ex=20), 8)
    c["inpaint_32"] = (wl.inpaint_session(31, side=32), 8)
    s = wl.config0(out=24, ex=16)
    s["params"]["random_init"] = 20
    s["params"]["cauchy_dispersion"] = 0.3
    c["random_init_24"] = (s, 4)
    return c


def pack(spec, divisor, res):
    d = {"divisor": np.int64(divisor), "out_w": np.int64(spec["out_w"]), "out_h": np.int64(spec["out_h"])}
    for k, v in spec["params"].items():
        d["param_" + k] = np.array(-1 if v is None else v)
    for i, e in enumerate(spec["examples"]):
        d["ex%d_image" % i] = e["image"]
        if e.get("guide") is not None:
            d["ex%d_guide" % i] = e["guide"]
    if spec.get("target_guide") is not None:
        d["target_guide"] = spec["target_guide"]
    if spec.get("inpaint_mask") is not None:
        d["inpaint_mask"] = spec["inpaint_mask"]
        d["inpaint_index"] = np.int64(spec["inpaint_index"])
    for k in ("image", "coord", "id", "resolved", "scores"):
        d["out_" + k] = res[k]
    d["out_evals"] = np.int64(res["evals"])
    return d


def unpack(d):
    params = {}
    for k in d.files:
        if k.startswith("param_"):
            v = d[k].item()
            name = k[len("param_"):]
            if name == "random_init" and v == -1:
                v = None
            elif name == "tiling_mode":
                v = bool(v)
            params[name] = v
    exs = []
    i = 0
    while "ex%d_image" % i in d.files:
        e = {"image": d["ex%d_image" % i]}
        if "ex%d_guide" % i in d.files:
            e["guide"] = d["ex%d_guide" % i]
        exs.append(e)
        i += 1
    spec = {"out_w": int(d["out_w"]), "out_h": int(d["out_h"]), "params": params, "examples": exs,
            "target_guide": d["target_guide"] if "target_guide" in d.files else None,
            "inpaint_mask": d["inpaint_mask"] if "inpaint_mask" in d.files else None,
            "inpaint_index": int(d["inpaint_index"]) if "inpaint_index" in d.files else -1}
    return spec, int(d["divisor"])


if __name__ == "__main__":
    from oracle import oracle

    for name, (spec, divisor) in cases().items():
        res = oracle.run(spec, batch_divisor=divisor, nthreads=1)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **pack(spec, divisor, res))
        print(name, res["evals"])
