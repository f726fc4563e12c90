"""ImagePyramid on the device (ts_image_pyramid) against the oracle's
restatement of image 0.23.12's Gaussian resize: bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("h,w,levels", [(128, 128, 5), (300, 300, 5), (37, 91, 3), (20, 20, 6), (64, 48, 1), (50, 70, 0)])
def test_pyramid_matches_oracle(ts, oracle, wl, h, w, levels):
    img = wl.texture(h * 7 + w, h, w)
    got = ts.image_pyramid(img, levels)
    ref = oracle.pyramid(img, levels)
    assert got.shape == ref.shape
    bad = np.argwhere(got != ref)
    assert len(bad) == 0, "pyramid differs at %d places, first %s" % (len(bad), bad[:3].tolist())
    assert (got[-1] == img).all()


def test_resize_input_matches_oracle(ts, oracle, wl):
    """Session inputs resized with CatmullRom (resize_input) give the same
    synthesis as the oracle fed the oracle's own resize."""
    spec = wl.config0(out=40, ex=24)
    big = wl.texture(99, 57, 71)
    spec["examples"][0]["image"] = big
    b = ts.builder_from_spec(spec)
    b.resize_input(ts.Dims(33, 29))
    got = b.build().run()
    spec2 = dict(spec)
    spec2["examples"] = [{"image": oracle.resize(big, 33, 29, "catmullrom")}]
    ref = oracle.run(spec2, batch_divisor=8)
    assert (got.into_image() == ref["image"]).all()
    assert (got.coord_map() == ref["coord"]).all()
