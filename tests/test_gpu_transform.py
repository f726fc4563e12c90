"""CoordinateTransform (lib.rs:162-325) and the debug maps (ms.rs:604-653)
of generated images, on the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_transform_reproduces_the_image(ts, wl):
    spec = wl.config1(out=48, ex=24)
    g = ts.builder_from_spec(spec).build().run()
    t = g.coordinate_transform()
    assert (t.width, t.height) == (48, 48)
    assert t.original_maps() == [ts.Dims(24, 24)] * 4
    # the final stage colours every pixel from the full-resolution level
    exs = [e["image"] for e in spec["examples"]]
    assert (t.apply(exs) == g.into_image()).all()
    # the serialised form: header, map sizes, then the coordinate map
    data = t.write()
    words = np.frombuffer(data, "<u4")
    assert list(words[:4]) == [0x12340001, 48, 48, 4]
    assert (words[12:].reshape(48, 48, 3) == g.coord_map()).all()
    assert ts.CoordinateTransform.read(data).write() == data


def test_transform_apply_new_sources(ts, wl):
    spec = wl.config1(out=40, ex=20)
    g = ts.builder_from_spec(spec).build().run()
    t = g.coordinate_transform()
    news = [wl.texture(500 + i, 20, 20) for i in range(4)]
    got = t.apply(news + [wl.texture(9, 8, 8)])  # a fifth source is ignored
    cm = g.coord_map()
    want = np.stack(news)[cm[..., 2], cm[..., 1], cm[..., 0]]
    assert (got == want).all()
    # sources of another size are resized to the original ones first
    big = [wl.texture(600 + i, 31, 27) for i in range(4)]
    got = t.apply(big)
    assert got.shape == (40, 40, 4)
    with pytest.raises(ts.Error) as e:
        t.apply(news[:3])
    assert e.value.kind == "MapsCountMismatch"


def test_debug_maps_match_oracle(ts, wl, oracle):
    for spec in (wl.config0(out=32, ex=20), wl.inpaint_session(7300, scale=0.08)):
        g = ts.builder_from_spec(spec).build().run()
        patch, mapc, unc = g.debug_maps()
        flat, score = g.resolved()
        rp, rm, ru = oracle.debug_maps(g.id_map(), flat, score)
        assert (patch == rp).all() and (mapc == rm).all() and (unc == ru).all()
