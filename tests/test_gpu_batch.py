"""The batched form (ts_batch_*) against the plain path: every session of a
mixed batch -- uneven example and output sizes, k and m from {8, 20, 50},
guided, tiling, inpainting, random init, sample masks -- gives exactly the
result ts_session_run gives it alone (image, coordinate map, id map, resolved
list and scores), with stream launches and with the captured CUDA graph."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _outputs(g):
    flat, score = g.resolved()
    return {"image": g.into_image(), "coord": g.coord_map(), "ids": g.id_map(), "flat": flat,
            "score": score.view(np.uint32)}


def _assert_same(a, b, name):
    for key in a:
        bad = np.argwhere(a[key] != b[key])
        assert len(bad) == 0, "%s: %s differs at %d places, first %s" % (name, key, len(bad), bad[:3].tolist())


def _mixed_specs(wl):
    specs = wl.config3_sessions(12, seed=11, scale=0.12)
    specs.append(wl.inpaint_session(7100, scale=0.1))
    t = wl.config1(out=40, ex=24)
    specs.append(t)  # tiling, 4 examples, random init
    g = wl.config2(out=36, ex=20)
    specs.append(g)  # guided with a target guide
    masked = wl.config0(out=30, ex=18)
    mask = np.zeros((18, 18, 4), np.uint8)
    mask[3:15, 2:16, 0] = 255
    masked["examples"][0]["sample"] = "image"
    masked["examples"][0]["mask"] = mask
    specs.append(masked)
    return specs


@pytest.fixture(scope="module")
def plain_results(ts, wl):
    return [_outputs(ts.builder_from_spec(s).build().run()) for s in _mixed_specs(wl)]


@pytest.mark.parametrize("graph", [False, True])
def test_batch_matches_plain(ts, wl, plain_results, graph):
    specs = _mixed_specs(wl)
    batch = ts.Batch(graph=graph)
    for s in specs:
        batch.add(ts.builder_from_spec(s).build())
    assert len(batch) == len(specs)
    results = batch.run()
    assert len(batch) == 0
    for i, (g, ref) in enumerate(zip(results, plain_results)):
        _assert_same(_outputs(g), ref, "session %d (%s)" % (i, specs[i]["name"]))
    st = batch.stats()
    assert st["sessions"] == len(specs)
    assert st["output_pixels"] == sum(r["image"].shape[0] * r["image"].shape[1] for r in plain_results)
    assert st["launches"] > 0 and st["steps"] > 0


def test_batch_matches_oracle(ts, wl, oracle):
    specs = [wl.config0(out=32, ex=20), wl.config1(out=36, ex=20)]
    batch = ts.Batch()
    for s in specs:
        batch.add(ts.builder_from_spec(s).build())
    for s, g in zip(specs, batch.run()):
        ref = oracle.run(s, batch_divisor=8)
        assert (g.into_image() == ref["image"]).all()
        assert (g.coord_map() == ref["coord"]).all()


def test_batch_reuse_and_single_session(ts, wl, plain_results):
    specs = _mixed_specs(wl)
    batch = ts.Batch()
    for i in (3, 0):
        batch.add(ts.builder_from_spec(specs[i]).build())
        (g,) = batch.run()
        _assert_same(_outputs(g), plain_results[i], "session %d alone" % i)


def test_batch_consumes_session(ts, wl):
    s = ts.builder_from_spec(wl.config0(out=16, ex=12)).build()
    batch = ts.Batch()
    batch.add(s)
    with pytest.raises(ts.Error) as e:
        s.run()
    assert e.value.kind == "State"
    with pytest.raises(ts.Error) as e:
        batch.add(s)
    assert e.value.kind == "State"
    assert len(batch.run()) == 1
