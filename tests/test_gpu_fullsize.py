"""The headline workloads at their full sizes, GPU path against the oracle,
every output bit for bit.

  multi-example remix: 4 x 300^2 examples (seeds 1-4) -> 512^2, tiling,
      random_init 10, seed 211, k = m = 50
  guided synthesis: 256^2 example with a guide -> 512^2 following a 512^2
      target guide, guide_alpha 0.8, seed 7

At 512^2 the steps reach the sizes the reduced tests never do: the warp
resolve over batches of ~13k items, the exhaustive k-NN's cell-grid search
above 4096 points, the 5% tiling bands of a 512-pixel plane.  The remix runs
under several launch-shape settings (the thresholds the autotuner moves),
because results must not depend on them.  Reference path: ms.rs:702-1051.
"""
import os

import pytest

from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _tuning(ts, team, full, window):
    t = ts.Tuning.default()
    t.team_max_items, t.team_full_max_items, t.walk_window_max_items = team, full, window
    return t


@pytest.fixture(scope="module")
def remix(wl, oracle):
    spec = wl.config1()
    return spec, oracle.run(spec, nthreads=THREADS)


@pytest.mark.parametrize("shape", ["default", "warp_only", "team_wide"])
def test_multi_example_tiling_512(ts, remix, shape):
    spec, ref = remix
    tuning = {"default": None,
              "warp_only": _tuning(ts, 0, 0, 0),            # a warp per item everywhere, no bitmap window
              "team_wide": _tuning(ts, 8192, 512, 16384)}[shape]  # CTA forms and windows on larger steps
    got = ts.run_spec(spec, tuning=tuning)
    assert_same(got, ref, "remix 512^2 (%s)" % shape)


def test_guided_512(ts, oracle, wl):
    spec = wl.config2()
    ref = oracle.run(spec, nthreads=THREADS)
    got = ts.run_spec(spec)
    assert_same(got, ref, "guided 512^2")
