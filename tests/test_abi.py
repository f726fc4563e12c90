"""The C ABI without a GPU: libtsgpu.so loads, exports every function that
include/tsgpu.h declares, and the builder validates parameters and images the
way SessionBuilder::build does (session.rs:450-524) before touching a
device."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tsgpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(ts_[a-z0-9_]+)\s*\(", src)
    return sorted(set(n for n in names if not n.endswith("_fn")))


def test_every_declared_symbol_is_exported(ts):
    lib = C.CDLL(ts.library_path())
    names = declared_functions()
    assert len(names) >= 40, names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python mirror binds each of them with a signature
    unbound = [n for n in names if n not in ts.SIGNATURES]
    assert not unbound, unbound


def test_kernel_kinds_match_the_header(ts):
    """The Python names of the run statistics' record kinds follow the
    header's TS_KERNEL_* values, and fit the stats arrays."""
    src = open(HEADER).read()
    kinds = dict((n, int(v)) for n, v in re.findall(r"\bTS_KERNEL_([A-Z_]+)\s*=\s*(\d+)", src))
    count = kinds.pop("KINDS")
    assert count == len(ts.KERNEL_KINDS) == len(kinds)
    assert count <= len(ts.RunStats().kernel_ms)
    for name, value in kinds.items():
        assert ts.KERNEL_KINDS[value] == name.lower(), name


def test_status_strings(ts):
    assert ts.lib().ts_status_str(0) == b"ok"
    assert ts.lib().ts_status_str(1) == b"invalid range"
    assert ts.lib().ts_status_str(999) == b"unknown"


def test_limits(ts):
    lim = ts.limits()
    assert lim["max_nearest_neighbors"] == 256
    assert lim["max_random_sample_locations"] == 1024


def _img(h=8, w=8):
    return np.zeros((h, w, 4), np.uint8)


@pytest.mark.parametrize("setter,value,name", [
    ("cauchy_dispersion", 1.5, "cauchy-dispersion"),
    ("cauchy_dispersion", -0.1, "cauchy-dispersion"),
    ("backtrack_percent", 2.0, "backtrack-percent"),
    ("guide_alpha", -1.0, "guide-alpha"),
])
def test_invalid_range(ts, setter, value, name):
    b = ts.Session.builder().add_example(_img())
    getattr(b, setter)(value)
    with pytest.raises(ts.Error) as e:
        b.build()
    assert e.value.kind == "InvalidRange"
    assert "parameter '%s'" % name in str(e.value)
    assert "outside the range of 0-1" in str(e.value)


def test_nan_passes_range_checks_as_in_the_reference(ts):
    # f32 comparisons with NaN are false, so the reference accepts NaN; the
    # build can then only fail for want of a device
    b = ts.Session.builder().add_example(_img()).cauchy_dispersion(float("nan"))
    try:
        b.build()
    except ts.Error as e:
        assert e.kind != "InvalidRange", e


def test_zero_random_sample_locations(ts):
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().add_example(_img()).random_sample_locations(0).build()
    assert e.value.kind == "InvalidRange" and "m-rand" in str(e.value)


def test_zero_max_thread_count(ts):
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().add_example(_img()).max_thread_count(0).build()
    assert e.value.kind == "InvalidRange" and "max-thread-count" in str(e.value)


def test_no_examples(ts):
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().build()
    assert e.value.kind == "NoExamples"
    ex = ts.Example(_img()).set_sample_method(ts.SampleMethod.IGNORE)
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().add_example(ex).build()
    assert e.value.kind == "NoExamples"


def test_example_guide_mismatch(ts):
    b = ts.Session.builder().add_example(ts.Example(_img()).with_guide(_img())).add_example(_img())
    with pytest.raises(ts.Error) as e:
        b.build()
    assert e.value.kind == "ExampleGuideMismatch"
    assert "2 examples were provided, but only 1 guides were" in str(e.value)


def test_limits_enforced(ts):
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().add_example(_img()).nearest_neighbors(257).build()
    assert e.value.kind == "Limit"
    with pytest.raises(ts.Error) as e:
        ts.Session.builder().add_example(_img()).random_sample_locations(1025).build()
    assert e.value.kind == "Limit"


def test_style_transfer_without_example_guides_passes_validation(ts):
    # automatic guide maps are built for examples without a guide; the build
    # can then only fail for want of a device
    b = ts.Session.builder().add_example(_img()).load_target_guide(_img())
    try:
        b.build()
    except ts.Error as e:
        assert e.kind == "Cuda", e


def test_builder_is_consumed_by_build(ts):
    b = ts.Session.builder().random_sample_locations(0).add_example(_img())
    with pytest.raises(ts.Error):
        b.build()
    with pytest.raises(ts.Error) as e:
        b.seed(3)
    assert e.value.kind == "State"


def test_bad_image_arguments(ts):
    lib = ts.lib()
    h = lib.ts_builder_new()
    try:
        d = ts._ExampleDesc()
        d.rgba = None
        d.width, d.height = 4, 4
        assert lib.ts_builder_add_example(h, C.byref(d)) == 6  # TS_ERR_IMAGE
        assert lib.ts_builder_load_target_guide(h, None, 4, 4) == 6
        assert lib.ts_builder_inpaint_example_channel(h, 7, C.byref(d), 4, 4) == 1
    finally:
        lib.ts_builder_free(h)


def test_empty_batch_is_refused(ts):
    lib = ts.lib()
    b = lib.ts_batch_new(0)
    try:
        out = (C.c_void_p * 1)()
        assert lib.ts_batch_run(b, out) == 11  # TS_ERR_STATE
        assert b"empty batch" in lib.ts_batch_last_error(b)
        assert lib.ts_batch_size(b) == 0
        assert lib.ts_batch_add(b, None) == 14  # TS_ERR_NULL
    finally:
        lib.ts_batch_free(b)


def test_server_handles(ts):
    lib = ts.lib()
    lib.ts_server_free(None)
    h = lib.ts_server_new(0, 0, 4)  # NULL without a usable device
    if h:
        assert lib.ts_server_done(h, 12345) == -1
        lib.ts_server_free(h)
    out = C.c_void_p()
    assert lib.ts_server_wait(None, 1, C.byref(out), None) == 14  # TS_ERR_NULL
