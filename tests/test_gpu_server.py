"""The served form (ts_server_*): continuous batching of a request stream.
Requests submitted while others run join them on the device (more than one
request is admitted at once), and every result is byte-identical to the
plain ts_session_run of the same session: alone or in the mix, under a
budget that admits one request at a time, and from concurrent submitters."""
import threading
import time

import numpy as np
import pytest

from test_gpu_batch import _assert_same, _mixed_specs, _outputs

pytestmark = pytest.mark.gpu


def _specs(wl):
    specs = _mixed_specs(wl)
    specs.append(wl.inpaint_session(7200, scale=0.08))
    specs.append(wl.config1(out=72, ex=30))
    return specs


@pytest.fixture(scope="module")
def plain(ts, wl):
    return [_outputs(ts.builder_from_spec(s).build().run()) for s in _specs(wl)]


def test_stream_in_the_mix(ts, wl, plain):
    specs = _specs(wl)
    with ts.Server(max_active=8) as srv:
        tickets = []
        for i, s in enumerate(specs):
            tickets.append(srv.submit(ts.builder_from_spec(s).build()))
            if i % 4 == 3:
                time.sleep(0.003)  # later arrivals join the ones already running
        for i, t in enumerate(tickets):
            g, times = srv.wait(t)
            _assert_same(_outputs(g), plain[i], "request %d (%s)" % (i, specs[i]["name"]))
            assert times["submit_ms"] <= times["admit_ms"] <= times["done_ms"]
        st = srv.stats()
    assert st["completed"] == len(specs) and st["failed"] == 0
    assert st["peak_active"] > 1, st  # requests overlapped on the device
    assert st["output_pixels"] == sum(p["image"].shape[0] * p["image"].shape[1] for p in plain)


def test_alone_equals_mix(ts, wl, plain):
    specs = _specs(wl)
    with ts.Server(max_active=8) as srv:
        for i in (0, 5, len(specs) - 1):
            g, _ = srv.wait(srv.submit(ts.builder_from_spec(specs[i]).build()))
            _assert_same(_outputs(g), plain[i], "request %d alone" % i)
        st = srv.stats()
    assert st["peak_active"] == 1


def test_budget_one_at_a_time(ts, wl, plain):
    specs = _specs(wl)[:6]
    with ts.Server(hbm_budget=1, max_active=8) as srv:
        tickets = [srv.submit(ts.builder_from_spec(s).build()) for s in specs]
        for i, t in enumerate(tickets):
            g, _ = srv.wait(t)
            _assert_same(_outputs(g), plain[i], "request %d under a 1-byte budget" % i)
        st = srv.stats()
    assert st["peak_active"] == 1


def test_concurrent_submitters(ts, wl, plain):
    specs = _specs(wl)
    results = {}
    errors = []
    with ts.Server(max_active=16) as srv:
        def client(idx):
            try:
                for i in idx:
                    g, _ = srv.wait(srv.submit(ts.builder_from_spec(specs[i]).build()))
                    results[i] = _outputs(g)
            except Exception as e:  # reported below
                errors.append(e)
        threads = [threading.Thread(target=client, args=(range(k, len(specs), 4),)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
    assert not errors, errors
    for i in range(len(specs)):
        _assert_same(results[i], plain[i], "request %d from a concurrent client" % i)


def test_errors(ts, wl):
    with ts.Server(max_active=2) as srv:
        s = ts.builder_from_spec(wl.config0(out=16, ex=12)).build()
        t = srv.submit(s)
        with pytest.raises(ts.Error) as e:
            srv.submit(s)
        assert e.value.kind == "State"
        g, _ = srv.wait(t)
        assert g.into_image().shape == (16, 16, 4)
        with pytest.raises(ts.Error) as e:
            srv.wait(t)  # a ticket is waited for once
        assert e.value.kind == "State"
