"""GPU path against the CPU oracle: every output bit-exact.

The oracle (oracle/ms_oracle.c) restates the reference's ms.rs; both sides run
the same batch-snapshot schedule, so the output image, the coordinate map,
the id map, the resolved list and every first-resolve score (f32) must be
identical, not merely close.  Sizes are small enough for the oracle to finish
in seconds; test_gpu_fullsize.py compares the full-size workloads the same
way.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("image", "coord", "id", "resolved", "scores")


def assert_same(got, ref, label=""):
    for key in KEYS:
        a, b = np.asarray(got[key]), np.asarray(ref[key])
        assert a.shape == b.shape, "%s %s shape %s != %s" % (label, key, a.shape, b.shape)
        if key == "scores":
            # bit-exact f32, except that NaN payloads are hardware-specific
            same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
        else:
            same = a == b
        if not same.all():
            bad = np.argwhere(~same)
            raise AssertionError("%s %s differs at %d places, first %s: gpu %s oracle %s" % (
                label, key, len(bad), bad[:3].tolist(), a[tuple(bad[0])], b[tuple(bad[0])]))
    assert got["evals"] == ref["evals"], "%s evals %d != %d" % (label, got["evals"], ref["evals"])


def run_both(ts, oracle, spec, divisor=8, max_batch=0, team=None, full=1024):
    got = ts.run_spec(spec, batch_divisor=divisor, max_batch=max_batch, team_max_batch=team,
                      team_full_max_batch=full)
    ref = oracle.run(spec, batch_divisor=divisor, max_batch=max_batch, nthreads=4)
    return got, ref


@pytest.mark.parametrize("team,full", [(0, 0), (1 << 30, 0), (1 << 30, 1 << 30)])
def test_resolve_forms(ts, oracle, wl, team, full):
    """Resolve kernel forms on every batch: warp per item; CTA per item with
    early exit; CTA per item scoring every candidate."""
    specs = [wl.config0(out=64, ex=32), wl.config1(out=64, ex=32), wl.config2(out=64, ex=32)]
    mixed = wl.config1(out=48, ex=20)  # examples of different sizes: one padded pitch for all
    mixed["examples"][1]["image"] = wl.texture(77, 13, 29)
    mixed["examples"][2]["image"] = wl.texture(78, 31, 9)
    specs.append(mixed)
    for spec in specs:
        got, ref = run_both(ts, oracle, spec, team=team, full=full)
        assert_same(got, ref, "%s team=%d full=%d" % (spec["name"], team, full))


@pytest.mark.parametrize("divisor", [8, 2, 1])
def test_single_example_small(ts, oracle, wl, divisor):
    spec = wl.config0(out=64, ex=32)
    got, ref = run_both(ts, oracle, spec, divisor)
    assert_same(got, ref, "config0 64^2 divisor %d" % divisor)


def test_single_example_sequential(ts, oracle, wl):
    """batch_divisor 0: one item per step, the reference's single-thread run."""
    spec = wl.config0(out=24, ex=16)
    spec["params"]["nearest_neighbors"] = 8
    spec["params"]["random_sample_locations"] = 8
    got, ref = run_both(ts, oracle, spec, 0)
    assert_same(got, ref, "sequential")


def test_single_example_full(ts, oracle, wl):
    """config 0 at its full size (128^2 example -> 256^2, k = m = 50)."""
    spec = wl.config0()
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "config0 full")


def test_multi_example_tiling(ts, oracle, wl):
    spec = wl.config1(out=96, ex=48)
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "config1 small")


def test_guided(ts, oracle, wl):
    spec = wl.config2(out=96, ex=48)
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "config2 small")


@pytest.mark.parametrize("k,m", [(1, 1), (3, 2), (8, 20), (20, 8), (50, 50), (120, 64), (256, 16)])
def test_k_m_grid(ts, oracle, wl, k, m):
    spec = wl.config0(out=40, ex=24)
    spec["params"]["nearest_neighbors"] = k
    spec["params"]["random_sample_locations"] = m
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "k=%d m=%d" % (k, m))


def test_k_zero(ts, oracle, wl):
    """k = 0: every item resolves at random with the stage seed and is
    appended again (ms.rs:1002-1010)."""
    spec = wl.config0(out=20, ex=16)
    spec["params"]["nearest_neighbors"] = 0
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "k=0")


@pytest.mark.parametrize("stages", [0, 1, 2, 7])
def test_backtrack_stages(ts, oracle, wl, stages):
    spec = wl.config0(out=40, ex=32)
    spec["params"]["backtrack_stages"] = stages
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "stages=%d" % stages)


@pytest.mark.parametrize("p", [0.0, 0.3, 1.0])
def test_backtrack_percent(ts, oracle, wl, p):
    spec = wl.config0(out=32, ex=24)
    spec["params"]["backtrack_percent"] = p
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "p=%g" % p)


@pytest.mark.parametrize("sigma", [0.0, 0.05, 0.5])
def test_cauchy_dispersion(ts, oracle, wl, sigma):
    """sigma 0 fills the LUT with NaN/inf: the exact sequential argmin runs."""
    spec = wl.config0(out=28, ex=20)
    spec["params"]["cauchy_dispersion"] = sigma
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "sigma=%g" % sigma)


def test_tiny_output(ts, oracle, wl):
    """Fewer resolved points than k, output sides below the tiling band."""
    spec = wl.config0(out=6, ex=8)
    spec["params"]["tiling_mode"] = True
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "tiny")


def test_rectangular_tiling(ts, oracle, wl):
    spec = wl.config1(out=64, ex=40)
    spec["out_w"], spec["out_h"] = 72, 44
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "rect tiling")


def test_examples_of_different_sizes(ts, oracle, wl):
    spec = wl.config1(out=56, ex=32)
    spec["examples"][1]["image"] = wl.texture(9, 20, 44)
    spec["examples"][2]["image"] = wl.texture(10, 37, 23)
    spec["params"]["tiling_mode"] = False
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "sizes")


def test_sample_masks(ts, oracle, wl):
    spec = wl.config0(out=40, ex=32)
    mask = np.zeros((32, 32, 4), np.uint8)
    mask[4:20, 6:30, 0] = 255
    spec["examples"][0]["sample"] = "image"
    spec["examples"][0]["mask"] = mask
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "sample mask")
    ex = spec["examples"][0]
    c = got["coord"].reshape(-1, 3)
    assert (mask[c[:, 1], c[:, 0], 0] != 0).all(), "a pixel was copied from a masked-out texel"


def test_ignored_example(ts, oracle, wl):
    spec = wl.config1(out=40, ex=24)
    spec["examples"][3]["sample"] = "ignore"
    spec["params"]["random_init"] = None
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "ignore")


def test_inpaint(ts, oracle, wl):
    spec = wl.inpaint_session(77, side=64)
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "inpaint")
    # locked pixels end at the last pyramid level, the example itself
    locked = spec["inpaint_mask"][..., 0] == 255
    assert (got["image"][locked] == spec["examples"][0]["image"][locked]).all()


def test_inpaint_tiling(ts, oracle, wl):
    spec = wl.inpaint_session(78, side=48)
    spec["params"]["tiling_mode"] = True
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "inpaint tiling")


def test_random_init(ts, oracle, wl):
    spec = wl.config0(out=40, ex=24)
    spec["params"]["random_init"] = 37
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "random init")


def test_max_batch(ts, oracle, wl):
    spec = wl.config0(out=48, ex=24)
    got, ref = run_both(ts, oracle, spec, divisor=1, max_batch=37)
    assert_same(got, ref, "max batch")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_seeds(ts, oracle, wl, seed):
    spec = wl.config2(out=48, ex=32)
    spec["params"]["seed"] = seed
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "seed %d" % seed)


def _golden_cases():
    import glob
    import os

    here = os.path.dirname(os.path.abspath(__file__))
    return sorted(glob.glob(os.path.join(here, "golden", "*.npz")))


@pytest.mark.parametrize("path", _golden_cases(), ids=lambda p: p.rsplit("/", 1)[-1])
def test_gpu_matches_golden_fixture(ts, path):
    """The GPU path reproduces the committed oracle fixtures (made on another
    machine) bit for bit."""
    import importlib.util
    import os

    here = os.path.dirname(os.path.abspath(__file__))
    sp = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(sp)
    sp.loader.exec_module(mg)
    d = np.load(path)
    spec, divisor = mg.unpack(d)
    got = ts.run_spec(spec, batch_divisor=divisor)
    ref = {k: d["out_" + k] for k in KEYS}
    ref["evals"] = int(d["out_evals"])
    assert_same(got, ref, os.path.basename(path))


@pytest.mark.parametrize("case", ["translucent", "translucent_guided", "tiny_levels"])
def test_alpha_channel_cost_paths(ts, oracle, wl, case):
    """The cost loops skip the alpha term only when every texel a run can
    compare has alpha 255 (its term is then LUT[0] = 0).  Examples or guides
    with other alpha values, and pyramids with an all-zero level (a
    downscale with a zero side), take the four-channel loop; both must
    match the oracle."""
    rng = np.random.default_rng(17)
    if case == "tiny_levels":
        spec = wl.config0(out=32, ex=12)  # 12 >> 4 == 0: the coarsest level is all zeros
        spec["params"]["backtrack_stages"] = 5
    elif case == "translucent":
        spec = wl.config0(out=40, ex=24)
        spec["examples"][0]["image"][..., 3] = rng.integers(0, 256, (24, 24), dtype=np.uint8)
    else:
        spec = wl.config2(out=48, ex=24)
        g = spec["examples"][0]["guide"]
        g[..., 3] = rng.integers(200, 256, g.shape[:2], dtype=np.uint8)
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, case)
