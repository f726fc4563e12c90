"""The autotuner's host logic without a GPU: the default setting, the
argument checks, and that a failing workload callback ends the tuning with
its status (or its Python exception) before any device work."""
import ctypes as C

import pytest

TS_OK, TS_ERR_STATE, TS_ERR_NULL = 0, 11, 14


def test_default_setting(ts):
    t = ts.Tuning.default()
    assert (t.team_max_items, t.team_full_max_items, t.walk_window_max_items) == (2048, 256, 4096)
    assert t.trials == 0 and t.gpu_ms == 0.0


def test_null_arguments(ts):
    t = ts.Tuning()
    assert ts.lib().ts_autotune_session(ts._BUILDER_FACTORY(), None, 1, C.byref(t)) == TS_ERR_NULL
    assert ts.lib().ts_autotune_batch(0, ts._BATCH_FILLER(), None, 1, C.byref(t)) == TS_ERR_NULL
    assert ts.lib().ts_builder_tuning(None, C.byref(t)) == TS_ERR_NULL
    assert ts.lib().ts_batch_tuning(None, C.byref(t)) == TS_ERR_NULL
    assert ts.lib().ts_server_tuning(None, C.byref(t)) == TS_ERR_NULL


def test_factory_without_builder_stops_the_tuner(ts):
    calls = []

    @ts._BUILDER_FACTORY
    def factory(_user):
        calls.append(1)
        return None

    t = ts.Tuning()
    assert ts.lib().ts_autotune_session(factory, None, 3, C.byref(t)) == TS_ERR_STATE
    assert len(calls) == 1


def test_filler_status_stops_the_tuner(ts):
    @ts._BATCH_FILLER
    def fill(_b, _user):
        return 7

    t = ts.Tuning()
    assert ts.lib().ts_autotune_batch(0, fill, None, 2, C.byref(t)) == 7


def test_empty_batch_stops_the_tuner(ts):
    @ts._BATCH_FILLER
    def fill(_b, _user):
        return TS_OK

    t = ts.Tuning()
    assert ts.lib().ts_autotune_batch(0, fill, None, 2, C.byref(t)) == TS_ERR_STATE


def test_python_exception_is_raised(ts):
    def make():
        raise ValueError("workload broken")

    with pytest.raises(ValueError, match="workload broken"):
        ts.autotune_session(make, repeats=1)
    with pytest.raises(ValueError, match="workload broken"):
        ts.autotune_batch(make, repeats=1)


def test_setting_applies_to_a_builder(ts):
    import numpy as np

    t = ts.Tuning.default()
    t.team_max_items, t.team_full_max_items, t.walk_window_max_items = 0, 0, 0
    b = ts.Session.builder().add_example(ts.Example(np.zeros((8, 8, 4), np.uint8)))
    assert b.tuning(t) is b


def test_build_failure_stops_the_tuner(ts, wl):
    """Without a usable device the first trial's build fails; the tuner
    returns that status after one factory call."""
    import os

    pytest.importorskip("torch")
    import torch

    if torch.cuda.is_available() or os.path.exists("/dev/nvidia0"):
        pytest.skip("a device is present")
    calls = []
    spec = wl.config0(out=16, ex=8)

    def make():
        calls.append(1)
        return ts.builder_from_spec(spec)

    with pytest.raises(ts.Error) as e:
        ts.autotune_session(make, repeats=1)
    assert e.value.status == 10  # TS_ERR_CUDA
    assert len(calls) == 1
