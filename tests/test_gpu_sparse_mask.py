"""Sample masks so sparse that random candidates run out of draws.

The reference draws a random candidate's (x, y) until it lies in the sample
mask (ms.rs:549-599) and never gives up.  Here the GPU path and the oracle
both stop after TS_MAX_SAMPLE_DRAWS pairs (include/tsgpu.h) and report
TS_ERR_NO_VALID_SAMPLE, so they must agree on every such input: the same
status when the draws run out, identical outputs when they do not.  Only
items with resolved neighbours draw random candidates (ms.rs:1002-1010), so
a session whose single pixel resolves at random succeeds however sparse
the mask is.  Every loop here is bounded: nothing spins.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu

SIDE = 4096  # 16.8 M texels, one valid: 2^22 draws miss it with probability ~0.78


def sparse_spec(wl, out_w, out_h, seed=0, side=SIDE, valid=((1234, 2345),)):
    img = np.zeros((side, side, 4), np.uint8)
    img[..., 3] = 255
    img[..., 0] = (np.arange(side) % 251)[None, :]
    img[..., 1] = (np.arange(side) % 241)[:, None]
    mask = np.zeros((side, side, 4), np.uint8)
    for y, x in valid:
        mask[y, x, 0] = 255
    return wl._spec("sparse_%d" % side, out_w, out_h, [{"image": img, "sample": "image", "mask": mask}],
                    seed=seed, nearest_neighbors=4, random_sample_locations=2, backtrack_stages=1)


def test_draws_run_out_on_both_sides(ts, oracle, wl):
    spec = sparse_spec(wl, 8, 8)
    with pytest.raises(oracle.OracleError) as ref:
        oracle.run(spec)
    assert ref.value.status == oracle.OracleError.NO_VALID_SAMPLE
    with pytest.raises(ts.Error) as got:
        ts.run_spec(spec)
    assert got.value.kind == "NoValidSample", str(got.value)


def test_random_resolve_needs_no_draws(ts, oracle, wl):
    """A 1x1 output: its only item has no neighbours and resolves at random,
    so it never uses the random candidates whose draws ran out."""
    spec = sparse_spec(wl, 1, 1)
    ref = oracle.run(spec)
    got = ts.run_spec(spec)
    assert_same(got, ref, "1x1 sparse mask")


def test_sparse_mask_found(ts, oracle, wl):
    """One valid texel in a 64^2 map: found well within the bound; the GPU
    path and the oracle draw the same pairs and agree bit for bit."""
    spec = sparse_spec(wl, 16, 16, side=64, valid=((17, 40),))
    ref = oracle.run(spec)
    got = ts.run_spec(spec)
    assert_same(got, ref, "one valid texel")
    c = got["coord"].reshape(-1, 3)
    assert ((c[:, 0] == 40) & (c[:, 1] == 17)).sum() > 0
