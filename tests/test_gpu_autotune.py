"""The autotuner on the GPU: it returns a setting from its candidate lists
with the device times it measured, and a session, batch or server run under
the tuned setting gives byte for byte what the default setting gives (and,
for the plain path, what the oracle gives)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TEAM = {0, 512, 1024, 2048, 4096, 8192}
FULL = {0, 64, 128, 256, 512}
WINDOW = {0, 1024, 2048, 4096, 8192, 16384}


def _outputs(g):
    flat, score = g.resolved()
    return {"image": g.into_image(), "coord": g.coord_map(), "ids": g.id_map(), "flat": flat,
            "score": score.view(np.uint32)}


def _assert_same(a, b, name):
    for key in a:
        bad = np.argwhere(a[key] != b[key])
        assert len(bad) == 0, "%s: %s differs at %d places, first %s" % (name, key, len(bad), bad[:3].tolist())


def _check_setting(t, repeats, walk):
    assert t.team_max_items in TEAM and t.team_full_max_items in FULL
    assert t.team_full_max_items <= t.team_max_items
    assert t.walk_window_max_items in WINDOW if walk else t.walk_window_max_items == 4096
    assert t.trials >= 1 + repeats
    assert (t.trials - 1) % repeats == 0  # one untimed run, then `repeats` per setting
    assert 0.0 < t.gpu_ms <= t.default_gpu_ms


def test_session_tuning(ts, wl, oracle):
    spec = wl.config1(out=96, ex=48)
    t = ts.autotune_session(lambda: ts.builder_from_spec(spec), repeats=2)
    _check_setting(t, 2, True)
    tuned = _outputs(ts.builder_from_spec(spec, tuning=t).build().run())
    default = _outputs(ts.builder_from_spec(spec).build().run())
    _assert_same(tuned, default, "tuned vs default")
    ref = oracle.run(spec, batch_divisor=8)
    assert (tuned["image"] == ref["image"]).all()
    assert (tuned["coord"] == ref["coord"]).all()


def test_extreme_settings_match(ts, wl):
    spec = wl.config0(out=64, ex=32)
    base = _outputs(ts.builder_from_spec(spec).build().run())
    for team, full, window in [(0, 0, 0), (8192, 512, 16384), (512, 0, 1024)]:
        t = ts.Tuning.default()
        t.team_max_items, t.team_full_max_items, t.walk_window_max_items = team, full, window
        got = _outputs(ts.builder_from_spec(spec, tuning=t).build().run())
        _assert_same(got, base, "setting %s" % ((team, full, window),))


def test_batch_and_server_tuning(ts, wl):
    specs = wl.config3_sessions(6, seed=5, scale=0.12)
    t = ts.autotune_batch(lambda: [ts.builder_from_spec(s).build() for s in specs], repeats=1)
    _check_setting(t, 1, False)
    plain = [_outputs(ts.builder_from_spec(s).build().run()) for s in specs]
    batch = ts.Batch(tuning=t)
    for s in specs:
        batch.add(ts.builder_from_spec(s).build())
    for i, g in enumerate(batch.run()):
        _assert_same(_outputs(g), plain[i], "batched session %d" % i)
    with ts.Server(tuning=t) as srv:
        tickets = [srv.submit(ts.builder_from_spec(s).build()) for s in specs]
        for i, tk in enumerate(tickets):
            g, _ = srv.wait(tk)
            _assert_same(_outputs(g), plain[i], "served session %d" % i)
