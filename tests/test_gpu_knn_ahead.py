"""The plain path's k-NN made ahead (power-of-two outputs, k > 0) against the
CPU oracle, every output bit-exact.

With W and H powers of two the plain path computes the neighbour lists of
whole chunks of batches on a side stream before their resolves, from the
pick order alone: each item's tree is checked by list position against its
own batch-start length, and a batch of redo items leaves its commit to the
next batch step's resolve launch.  The cases below are the power-of-two
twins of the parity tests whose sizes take the per-step form, so that every
schedule shape the reference has (stage counts, backtrack fractions, random
init, inpainting, tiling mirrors, tiny and rectangular outputs, sequential
and capped batches, NaN cost tables, sample masks) runs through both.
`knn_chunks` in the run statistics says which form ran.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same, run_both

pytestmark = pytest.mark.gpu


def ahead(got):
    return got["stats"]["knn_chunks"] > 0


def test_form_follows_the_output_size(ts, oracle, wl):
    got, ref = run_both(ts, oracle, wl.config0(out=32, ex=24))
    assert_same(got, ref, "32")
    assert ahead(got)
    got, ref = run_both(ts, oracle, wl.config0(out=40, ex=24))
    assert_same(got, ref, "40")
    assert not ahead(got)


@pytest.mark.parametrize("k,m", [(1, 1), (3, 2), (8, 20), (50, 50), (120, 64), (256, 16)])
def test_k_m_grid(ts, oracle, wl, k, m):
    spec = wl.config0(out=32, ex=24)
    spec["params"]["nearest_neighbors"] = k
    spec["params"]["random_sample_locations"] = m
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "k=%d m=%d" % (k, m))
    assert ahead(got)


@pytest.mark.parametrize("stages", [0, 1, 2, 7])
def test_backtrack_stages(ts, oracle, wl, stages):
    spec = wl.config0(out=64, ex=32)
    spec["params"]["backtrack_stages"] = stages
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "stages=%d" % stages)


@pytest.mark.parametrize("p", [0.0, 1.0])
def test_backtrack_percent(ts, oracle, wl, p):
    spec = wl.config1(out=64, ex=32)
    spec["params"]["backtrack_percent"] = p
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "p=%g" % p)


def test_nan_cost_tables(ts, oracle, wl):
    """sigma 0: the exact sequential argmin, its neighbours made ahead."""
    spec = wl.config0(out=32, ex=20)
    spec["params"]["cauchy_dispersion"] = 0.0
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "sigma=0")
    assert ahead(got)


def test_sample_masks(ts, oracle, wl):
    spec = wl.config0(out=64, ex=32)
    mask = np.zeros((32, 32, 4), np.uint8)
    mask[4:20, 6:30, 0] = 255
    spec["examples"][0]["sample"] = "image"
    spec["examples"][0]["mask"] = mask
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "sample mask")


def test_random_init(ts, oracle, wl):
    spec = wl.config1(out=64, ex=24)
    spec["params"]["random_init"] = 37
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "random init")


@pytest.mark.parametrize("divisor,max_batch", [(1, 37), (0, 0), (8, 5)])
def test_batch_schedules(ts, oracle, wl, divisor, max_batch):
    """Capped and sequential schedules: many small batches per chunk, and
    one item per batch."""
    spec = wl.config0(out=32, ex=24)
    got, ref = run_both(ts, oracle, spec, divisor=divisor, max_batch=max_batch)
    assert_same(got, ref, "divisor %d max %d" % (divisor, max_batch))


def test_ignored_example(ts, oracle, wl):
    spec = wl.config1(out=32, ex=24)
    spec["examples"][3]["sample"] = "ignore"
    spec["params"]["random_init"] = None
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "ignore")


def test_tiny_tiling(ts, oracle, wl):
    """Fewer resolved points than k, sides below the tiling band."""
    spec = wl.config0(out=8, ex=8)
    spec["params"]["tiling_mode"] = True
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "tiny")
    assert ahead(got)


def test_rectangular_tiling(ts, oracle, wl):
    """W != H: the exact distance units scale x and y apart."""
    spec = wl.config1(out=64, ex=40)
    spec["out_w"], spec["out_h"] = 128, 32
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "rect tiling")
    assert ahead(got)


def test_inpaint_tiling(ts, oracle, wl):
    spec = wl.inpaint_session(78, side=64)
    spec["params"]["tiling_mode"] = True
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, "inpaint tiling")
    assert ahead(got)


@pytest.mark.parametrize("team,full", [(0, 0), (1 << 30, 0), (1 << 30, 1 << 30)])
def test_resolve_forms(ts, oracle, wl, team, full):
    """Every resolve form reads deferred commits (shadow records) the same."""
    spec = wl.config2(out=64, ex=32)
    got, ref = run_both(ts, oracle, spec, team=team, full=full)
    assert_same(got, ref, "team %d full %d" % (team, full))


@pytest.mark.parametrize("case", ["guided_tiling", "inpaint_128", "k8_m20_128", "rect_256x64"])
def test_larger_schedules(ts, oracle, wl, case):
    """More batches and chunks per stage than the small twins above."""
    if case == "guided_tiling":
        spec = wl.config2(out=64, ex=48)
        spec["params"]["tiling_mode"] = True
    elif case == "inpaint_128":
        spec = wl.inpaint_session(91, side=128)
    elif case == "k8_m20_128":
        spec = wl.config1(out=128, ex=48)
        spec["params"]["nearest_neighbors"] = 8
        spec["params"]["random_sample_locations"] = 20
    else:
        spec = wl.config0(out=64, ex=40)
        spec["out_w"], spec["out_h"] = 256, 64
    got, ref = run_both(ts, oracle, spec)
    assert_same(got, ref, case)
    assert ahead(got)
