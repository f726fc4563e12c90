"""Automatic guide maps for style transfer (utils.rs:101-183, lib.rs:575-582)
on the device against the oracle's restatement: the guide itself, and a
style-transfer session (target guide, examples without guides) against the
oracle run with the oracle's guides."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("h,w,th,tw", [(24, 24, 40, 40), (37, 19, 23, 50), (64, 64, 64, 64), (5, 9, 3, 4)])
def test_guide_map_matches_oracle(ts, wl, oracle, h, w, th, tw):
    img = wl.texture(h * 3 + w, h, w)
    tgt = wl.target_guide(h + tw, th, tw)
    got = ts.guide_map(img, tgt)
    ref = oracle.guide_map(img, tgt)
    bad = np.argwhere(got != ref)
    assert len(bad) == 0, "guide differs at %d places, first %s" % (len(bad), bad[:3].tolist())
    assert (got[..., 0] == got[..., 1]).all() and (got[..., 3] == 255).all()


def test_style_transfer_session(ts, wl, oracle):
    spec = wl.config2(out=40, ex=24)
    for e in spec["examples"]:
        e.pop("guide", None)
    got = ts.builder_from_spec(spec).build().run()
    ref_spec = dict(spec)
    ref_spec["examples"] = [dict(e, guide=oracle.guide_map(e["image"], spec["target_guide"]))
                            for e in spec["examples"]]
    ref = oracle.run(ref_spec, batch_divisor=8)
    assert (got.into_image() == ref["image"]).all()
    assert (got.coord_map() == ref["coord"]).all()
