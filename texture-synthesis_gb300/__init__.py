"""GB300-native texture synthesis: Python mirror of the reference's session API.

The reference (EmbarkStudios/texture-synthesis, Rust) is used as

    let session = Session::builder()
        .add_example(&"imgs/1.jpg")
        .seed(10)
        .build()?;
    let generated = session.run(None);

and this package keeps that shape over the C ABI in include/tsgpu.h:

    import importlib
    ts = importlib.import_module("texture-synthesis_gb300")
    session = ts.Session.builder().add_example(rgba).seed(10).build()
    generated = session.run()
    image = generated.into_image()          # H x W x 4 uint8

Images are numpy RGBA8 arrays (H x W x 4); decoding files is the caller's
job.  Every call runs on one CUDA device through libtsgpu.so; there is no
CPU fallback, and the package refuses to load when the library is missing.
"""
import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libtsgpu.so")
_lib = None

# ts_status (tsgpu.h); the first five mirror texture_synthesis::Error
STATUS = {
    0: "Ok", 1: "InvalidRange", 2: "SizeMismatch", 3: "ExampleGuideMismatch", 4: "NoExamples",
    5: "MapsCountMismatch", 6: "Image", 7: "Unsupported", 8: "NoValidSample", 9: "Index", 10: "Cuda",
    11: "State", 12: "Limit", 13: "OutOfMemory", 14: "Null",
}


class Error(Exception):
    """texture_synthesis::Error (lib/src/errors.rs:37-57) plus this library's
    own statuses; `kind` names the variant, `status` is the C status code."""

    def __init__(self, status, message):
        self.status = status
        self.kind = STATUS.get(status, "Unknown")
        super().__init__("%s: %s" % (self.kind, message))


class _ExampleDesc(C.Structure):
    _fields_ = [
        ("rgba", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
        ("guide_rgba", C.c_void_p), ("guide_width", C.c_uint32), ("guide_height", C.c_uint32),
        ("sample_method", C.c_int32),
        ("mask_rgba", C.c_void_p), ("mask_width", C.c_uint32), ("mask_height", C.c_uint32),
    ]


class _Limits(C.Structure):
    _fields_ = [("max_nearest_neighbors", C.c_uint32), ("max_random_sample_locations", C.c_uint32),
                ("max_examples", C.c_uint32), ("max_image_side", C.c_uint32)]


class _Progress(C.Structure):
    _fields_ = [("image", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("total_current", C.c_uint64), ("total_total", C.c_uint64),
                ("stage_current", C.c_uint64), ("stage_total", C.c_uint64)]


BATCH_PHASES = ("level_switch", "random_candidates", "knn_walk", "knn_exhaustive", "mean", "resolve",
                "resolve_team", "resolve_team_full", "commit")
KERNEL_KINDS = ("random_candidates", "knn_walk", "knn_exhaustive", "resolve", "commit", "level_switch", "mean",
                "knn_wait")


class RunStats(C.Structure):
    _fields_ = [("resolves", C.c_uint64), ("cost_evals", C.c_uint64), ("batches", C.c_uint64),
                ("stages", C.c_uint64), ("kernel_launches", C.c_uint64), ("gpu_ms", C.c_double),
                ("wall_ms", C.c_double), ("kernel_count", C.c_uint64 * 8), ("kernel_ms", C.c_double * 8),
                ("host_plan_ms", C.c_double), ("host_alloc_ms", C.c_double), ("host_enqueue_ms", C.c_double),
                ("host_wait_ms", C.c_double), ("host_finish_ms", C.c_double), ("upload_ms", C.c_double),
                ("readback_ms", C.c_double), ("host_pick_ms", C.c_double), ("host_launch_ms", C.c_double),
                ("knn_chunks", C.c_uint64)]

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("kernel_") or f == "kernel_launches"}
        d["kernels"] = {name: {"launches": int(self.kernel_count[i]), "ms": float(self.kernel_ms[i])}
                        for i, name in enumerate(KERNEL_KINDS)}
        return d


class _BatchStats(C.Structure):
    _fields_ = [("sessions", C.c_uint64), ("steps", C.c_uint64), ("launches", C.c_uint64),
                ("output_pixels", C.c_uint64), ("resolves", C.c_uint64), ("cost_evals", C.c_uint64),
                ("gpu_ms", C.c_double), ("wall_ms", C.c_double), ("plan_ms", C.c_double),
                ("phase_launches", C.c_uint64 * 9), ("phase_ms", C.c_double * 9), ("upload_ms", C.c_double),
                ("readback_ms", C.c_double)]


class _ImageDesc(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32)]


class _RequestTimes(C.Structure):
    _fields_ = [("submit_ms", C.c_double), ("admit_ms", C.c_double), ("done_ms", C.c_double)]


class _ServerStats(C.Structure):
    _fields_ = [(f, C.c_uint64) for f in ("submitted", "admitted", "completed", "failed", "ticks", "launches",
                                          "peak_active", "peak_bytes", "budget_bytes", "output_pixels",
                                          "cost_evals", "driver_tick_us", "driver_ring_wait_us",
                                          "driver_pick_wait_us", "driver_launch_us")]


class _LaunchRecord(C.Structure):
    _fields_ = [("kind", C.c_int32), ("stage", C.c_int32), ("batch_items", C.c_uint32), ("ms", C.c_float)]


class Tuning(C.Structure):
    """Launch-shape thresholds (ts_tuning): a CTA per item in steps of at
    most team_max_items items (every candidate scored up to
    team_full_max_items), and, on the plain path, a walk bitmap window in
    steps of at most walk_window_max_items.  Results never depend on them."""

    _fields_ = [("team_max_items", C.c_uint32), ("team_full_max_items", C.c_uint32),
                ("walk_window_max_items", C.c_uint32), ("trials", C.c_uint32), ("gpu_ms", C.c_double),
                ("default_gpu_ms", C.c_double)]

    @staticmethod
    def default():
        t = Tuning()
        lib().ts_tuning_default(C.byref(t))
        return t

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_PROGRESS_FN = C.CFUNCTYPE(None, C.POINTER(_Progress), C.c_void_p)
_BUILDER_FACTORY = C.CFUNCTYPE(C.c_void_p, C.c_void_p)
_BATCH_FILLER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p)

class _GatherPeak(C.Structure):
    _fields_ = [("patch_gbs", C.c_double), ("random_gbs", C.c_double), ("table_bytes", C.c_double),
                ("threads", C.c_uint32), ("patch_ms", C.c_float), ("random_ms", C.c_float),
                ("patch_ilp", C.c_int32), ("random_ilp", C.c_int32)]


# every function tsgpu.h declares: name -> (restype, argtypes)
SIGNATURES = {
    "ts_status_str": (C.c_char_p, [C.c_int]),
    "ts_get_limits": (None, [C.POINTER(_Limits)]),
    "ts_image_pyramid": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p, C.c_int32]),
    "ts_guide_map": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                               C.c_int32]),
    "ts_image_pyramid_noalloc": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p,
                                           C.c_void_p]),
    "ts_builder_new": (C.c_void_p, []),
    "ts_builder_free": (None, [C.c_void_p]),
    "ts_builder_last_error": (C.c_char_p, [C.c_void_p]),
    "ts_builder_add_example": (C.c_int, [C.c_void_p, C.POINTER(_ExampleDesc)]),
    "ts_builder_inpaint_example": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                             C.POINTER(_ExampleDesc), C.c_uint32, C.c_uint32]),
    "ts_builder_inpaint_example_channel": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(_ExampleDesc),
                                                     C.c_uint32, C.c_uint32]),
    "ts_builder_load_target_guide": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_builder_resize_input": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_builder_seed": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ts_builder_tiling_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "ts_builder_nearest_neighbors": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ts_builder_random_sample_locations": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ts_builder_random_init": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ts_builder_cauchy_dispersion": (C.c_int, [C.c_void_p, C.c_float]),
    "ts_builder_guide_alpha": (C.c_int, [C.c_void_p, C.c_float]),
    "ts_builder_backtrack_percent": (C.c_int, [C.c_void_p, C.c_float]),
    "ts_builder_backtrack_stages": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ts_builder_output_size": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_builder_max_thread_count": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ts_builder_batch_schedule": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_builder_device": (C.c_int, [C.c_void_p, C.c_int32]),
    "ts_builder_profile_kernels": (C.c_int, [C.c_void_p, C.c_int32]),
    "ts_builder_resolve_team": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_builder_build": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "ts_session_run": (C.c_int, [C.c_void_p, _PROGRESS_FN, C.c_void_p, C.POINTER(C.c_void_p)]),
    "ts_session_free": (None, [C.c_void_p]),
    "ts_session_last_error": (C.c_char_p, [C.c_void_p]),
    "ts_generated_dims": (None, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "ts_generated_image": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ts_generated_coord_map": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ts_generated_id_map": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ts_generated_resolved_count": (C.c_uint64, [C.c_void_p]),
    "ts_generated_resolved": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "ts_generated_stats": (None, [C.c_void_p, C.POINTER(RunStats)]),
    "ts_generated_free": (None, [C.c_void_p]),
    "ts_generated_launch_count": (C.c_uint64, [C.c_void_p]),
    "ts_generated_launches": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ts_batch_new": (C.c_void_p, [C.c_int32]),
    "ts_batch_free": (None, [C.c_void_p]),
    "ts_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "ts_batch_add": (C.c_int, [C.c_void_p, C.c_void_p]),
    "ts_batch_size": (C.c_uint64, [C.c_void_p]),
    "ts_batch_use_graph": (C.c_int, [C.c_void_p, C.c_int32]),
    "ts_batch_run": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "ts_batch_profile": (C.c_int, [C.c_void_p, C.c_int32]),
    "ts_batch_plan_threads": (C.c_int, [C.c_void_p, C.c_uint32]),
    "ts_batch_resolve_team": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_batch_stats_get": (None, [C.c_void_p, C.POINTER(_BatchStats)]),
    "ts_generated_debug_maps": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]),
    "ts_generated_coord_transform": (C.c_void_p, [C.c_void_p]),
    "ts_transform_free": (None, [C.c_void_p]),
    "ts_transform_dims": (None, [C.c_void_p, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "ts_transform_map_dims": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "ts_transform_write": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "ts_transform_read": (C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(C.c_void_p)]),
    "ts_transform_apply": (C.c_int, [C.c_void_p, C.POINTER(_ImageDesc), C.c_uint32, C.c_void_p, C.c_int32]),
    "ts_server_new": (C.c_void_p, [C.c_int32, C.c_uint64, C.c_uint32]),
    "ts_server_free": (None, [C.c_void_p]),
    "ts_server_last_error": (C.c_char_p, [C.c_void_p]),
    "ts_server_resolve_team": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "ts_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "ts_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p), C.POINTER(_RequestTimes)]),
    "ts_server_done": (C.c_int, [C.c_void_p, C.c_uint64]),
    "ts_server_stats_get": (None, [C.c_void_p, C.POINTER(_ServerStats)]),
    "ts_tuning_default": (None, [C.POINTER(Tuning)]),
    "ts_autotune_session": (C.c_int, [_BUILDER_FACTORY, C.c_void_p, C.c_uint32, C.POINTER(Tuning)]),
    "ts_autotune_batch": (C.c_int, [C.c_int32, _BATCH_FILLER, C.c_void_p, C.c_uint32, C.POINTER(Tuning)]),
    "ts_builder_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ts_batch_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ts_server_tuning": (C.c_int, [C.c_void_p, C.POINTER(Tuning)]),
    "ts_measure_gather_peak": (C.c_int, [C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int32,
                                         C.POINTER(_GatherPeak)]),
}


def library_path():
    return _LIB_PATH


def lib():
    """The loaded libtsgpu.so.  Raises if it has not been built: there is no
    other implementation to fall back to."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise RuntimeError("libtsgpu.so is not built (%s); run __graft_entry__.build() or "
                               "python texture-synthesis_gb300/build.py" % _LIB_PATH)
        L = C.CDLL(_LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def limits():
    out = _Limits()
    lib().ts_get_limits(C.byref(out))
    return {f: getattr(out, f) for f, _ in out._fields_}


def image_pyramid(image, levels, device=0):
    """ImagePyramid::new(image, Some(levels)) on the device: an array of
    max(levels, 1) x H x W x 4, coarsest level first."""
    img = _rgba(image)
    h, w = img.shape[:2]
    out = np.empty((max(1, levels), h, w, 4), np.uint8)
    rc = lib().ts_image_pyramid(img.ctypes.data, w, h, levels, out.ctypes.data, device)
    if rc:
        raise Error(rc, "ts_image_pyramid")
    return out


def gather_peak(width, height, k, reps=5, device=0):
    """ts_measure_gather_peak: GB/s of 32-bit gathers the GPU serves from a
    width x height texel table, in the cost loop's patch shape (k nearest
    offsets around a random centre) and fully random."""
    out = _GatherPeak()
    rc = lib().ts_measure_gather_peak(device, width, height, k, reps, C.byref(out))
    if rc:
        raise Error(rc, "ts_measure_gather_peak")
    return {f: getattr(out, f) for f, _ in out._fields_}


def guide_map(image, target, device=0):
    """The automatic guide of an example for a target guide
    (transform_to_guide_map + match_histograms, utils.rs:101-183)."""
    img = _rgba(image)
    tgt = _rgba(target)
    out = np.empty_like(img)
    rc = lib().ts_guide_map(img.ctypes.data, img.shape[1], img.shape[0], tgt.ctypes.data, tgt.shape[1],
                            tgt.shape[0], out.ctypes.data, device)
    if rc:
        raise Error(rc, "ts_guide_map")
    return out


@dataclass(frozen=True)
class Dims:
    """Dims (lib.rs:141-158)."""
    width: int
    height: int

    @staticmethod
    def square(size):
        return Dims(size, size)


class ChannelMask:
    """ChannelMask (utils.rs:46-53)."""
    R, G, B, A = 0, 1, 2, 3


class SampleMethod:
    """SampleMethod (lib.rs:458-484): ALL, IGNORE, or Image(mask)."""
    ALL = "all"
    IGNORE = "ignore"

    class Image:
        def __init__(self, mask):
            self.mask = _rgba(mask)


def _rgba(a):
    a = np.ascontiguousarray(a, dtype=np.uint8)
    if a.ndim != 3 or a.shape[2] != 4:
        raise ValueError("images are H x W x 4 RGBA8 arrays")
    return a


class Example:
    """Example / ExampleBuilder (lib.rs:486-623)."""

    def __init__(self, image):
        self.image = _rgba(image)
        self.guide = None
        self.sample_method = SampleMethod.ALL

    @staticmethod
    def builder(image):
        return Example(image)

    def with_guide(self, guide):
        self.guide = _rgba(guide)
        return self

    def set_sample_method(self, method):
        if isinstance(method, np.ndarray):
            method = SampleMethod.Image(method)
        self.sample_method = method
        return self

    def _desc(self, keep):
        d = _ExampleDesc()
        keep.append(self.image)
        d.rgba = self.image.ctypes.data
        d.height, d.width = self.image.shape[:2]
        if self.guide is not None:
            keep.append(self.guide)
            d.guide_rgba = self.guide.ctypes.data
            d.guide_height, d.guide_width = self.guide.shape[:2]
        sm = self.sample_method
        if isinstance(sm, SampleMethod.Image):
            d.sample_method = 2
            keep.append(sm.mask)
            d.mask_rgba = sm.mask.ctypes.data
            d.mask_height, d.mask_width = sm.mask.shape[:2]
        elif sm == SampleMethod.IGNORE:
            d.sample_method = 1
        else:
            d.sample_method = 0
        return d


def _as_example(e):
    return e if isinstance(e, Example) else Example(e)


class SessionBuilder:
    """SessionBuilder (session.rs:69-448).  Setters return self."""

    def __init__(self):
        self._h = lib().ts_builder_new()
        if not self._h:
            raise MemoryError("ts_builder_new")

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_builder_free(self._h)
            self._h = None

    def _check(self, rc):
        if rc:
            msg = lib().ts_builder_last_error(self._h)
            raise Error(rc, msg.decode() if msg else "")
        return self

    def add_example(self, example):
        keep = []
        d = _as_example(example)._desc(keep)
        return self._check(lib().ts_builder_add_example(self._h, C.byref(d)))

    def add_examples(self, examples):
        for e in examples:
            self.add_example(e)
        return self

    def inpaint_example(self, inpaint_mask, example, size):
        keep = []
        m = _rgba(inpaint_mask)
        d = _as_example(example)._desc(keep)
        return self._check(lib().ts_builder_inpaint_example(self._h, m.ctypes.data, m.shape[1], m.shape[0],
                                                            C.byref(d), size.width, size.height))

    def inpaint_example_channel(self, mask, example, size):
        keep = []
        d = _as_example(example)._desc(keep)
        return self._check(lib().ts_builder_inpaint_example_channel(self._h, int(mask), C.byref(d),
                                                                    size.width, size.height))

    def load_target_guide(self, guide):
        g = _rgba(guide)
        return self._check(lib().ts_builder_load_target_guide(self._h, g.ctypes.data, g.shape[1], g.shape[0]))

    def resize_input(self, dims):
        return self._check(lib().ts_builder_resize_input(self._h, dims.width, dims.height))

    def seed(self, value):
        return self._check(lib().ts_builder_seed(self._h, int(value)))

    def tiling_mode(self, is_tiling):
        return self._check(lib().ts_builder_tiling_mode(self._h, 1 if is_tiling else 0))

    def nearest_neighbors(self, count):
        return self._check(lib().ts_builder_nearest_neighbors(self._h, int(count)))

    def random_sample_locations(self, count):
        return self._check(lib().ts_builder_random_sample_locations(self._h, int(count)))

    def random_init(self, count):
        return self._check(lib().ts_builder_random_init(self._h, int(count)))

    def cauchy_dispersion(self, value):
        return self._check(lib().ts_builder_cauchy_dispersion(self._h, float(value)))

    def guide_alpha(self, value):
        return self._check(lib().ts_builder_guide_alpha(self._h, float(value)))

    def backtrack_percent(self, value):
        return self._check(lib().ts_builder_backtrack_percent(self._h, float(value)))

    def backtrack_stages(self, stages):
        return self._check(lib().ts_builder_backtrack_stages(self._h, int(stages)))

    def output_size(self, dims):
        return self._check(lib().ts_builder_output_size(self._h, dims.width, dims.height))

    def max_thread_count(self, count):
        return self._check(lib().ts_builder_max_thread_count(self._h, int(count)))

    def batch_schedule(self, divisor, max_batch=0):
        """Batch-snapshot schedule: max(1, R // divisor) items per batch step
        (R = resolved count at the step), capped at max_batch; divisor 0 means
        one item per step (the reference's single-thread semantics)."""
        return self._check(lib().ts_builder_batch_schedule(self._h, int(divisor), int(max_batch)))

    def device(self, ordinal):
        return self._check(lib().ts_builder_device(self._h, int(ordinal)))

    def resolve_team(self, max_batch, full_max_batch=256):
        """Resolve kernel forms by batch size (identical results): up to
        full_max_batch items, one CTA scores every candidate of an item; up to
        max_batch, one CTA per item with early exit; above, a warp per item."""
        return self._check(lib().ts_builder_resolve_team(self._h, int(max_batch), int(full_max_batch)))

    def tuning(self, tuning):
        """Launch-shape thresholds (a Tuning from autotune_session, or
        Tuning.default()); the results do not depend on them."""
        return self._check(lib().ts_builder_tuning(self._h, C.byref(tuning)))

    def profile_kernels(self, on=True):
        """Time every kernel launch with CUDA events (measurement runs)."""
        return self._check(lib().ts_builder_profile_kernels(self._h, 1 if on else 0))

    def build(self):
        out = C.c_void_p()
        rc = lib().ts_builder_build(self._h, C.byref(out))
        self._check(rc)
        return Session(out.value)


class Session:
    """Session (session.rs:22-66)."""

    def __init__(self, handle):
        self._h = handle

    @staticmethod
    def builder():
        return SessionBuilder()

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_session_free(self._h)
            self._h = None

    def run(self, progress=None):
        """Session::run: consumes the session.  progress(dict) is called once
        per stage with the current image and counters."""
        def _cb(p, _user):
            u = p.contents
            img = np.ctypeslib.as_array(C.cast(u.image, C.POINTER(C.c_uint8)),
                                        shape=(u.height, u.width, 4)).copy()
            progress({"image": img, "total": (u.total_current, u.total_total),
                      "stage": (u.stage_current, u.stage_total)})

        cb = _PROGRESS_FN(_cb) if progress else _PROGRESS_FN()
        out = C.c_void_p()
        rc = lib().ts_session_run(self._h, cb, None, C.byref(out))
        if rc:
            msg = lib().ts_session_last_error(self._h)
            raise Error(rc, msg.decode() if msg else "")
        return GeneratedImage(out.value)


class GeneratedImage:
    """GeneratedImage (lib.rs:378-455) with the generator's maps."""

    def __init__(self, handle):
        self._h = handle
        w, h = C.c_uint32(), C.c_uint32()
        lib().ts_generated_dims(self._h, C.byref(w), C.byref(h))
        self.width, self.height = w.value, h.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_generated_free(self._h)
            self._h = None

    def into_image(self):
        out = np.empty((self.height, self.width, 4), np.uint8)
        lib().ts_generated_image(self._h, out.ctypes.data)
        return out

    def coord_map(self):
        """(x, y, map) source coordinate of every pixel (the coordinate
        transform's buffer, ms.rs:655-684)."""
        out = np.empty((self.height, self.width, 3), np.uint32)
        lib().ts_generated_coord_map(self._h, out.ctypes.data)
        return out

    def id_map(self):
        """(patch id, map id) of every pixel (ms.rs:605-636)."""
        out = np.empty((self.height, self.width, 2), np.uint32)
        lib().ts_generated_id_map(self._h, out.ctypes.data)
        return out

    def resolved(self):
        """The resolved list (flat pixel index) and first-resolve scores."""
        n = lib().ts_generated_resolved_count(self._h)
        flat = np.empty(n, np.uint32)
        score = np.empty(n, np.float32)
        lib().ts_generated_resolved(self._h, flat.ctypes.data, score.ctypes.data)
        return flat, score

    def stats(self):
        st = RunStats()
        lib().ts_generated_stats(self._h, C.byref(st))
        return st.as_dict()

    def debug_maps(self, device=0):
        """save_debug's maps (lib.rs:404-419), computed on the device:
        (patch_id, map_id, uncertainty), each H x W x 4 uint8."""
        outs = [np.empty((self.height, self.width, 4), np.uint8) for _ in range(3)]
        rc = lib().ts_generated_debug_maps(self._h, outs[0].ctypes.data, outs[1].ctypes.data,
                                           outs[2].ctypes.data, device)
        if rc:
            raise Error(rc, "ts_generated_debug_maps")
        return tuple(outs)

    def coordinate_transform(self):
        """get_coordinate_transform (lib.rs:441-443)."""
        return CoordinateTransform(lib().ts_generated_coord_transform(self._h))

    def launches(self):
        """Per-launch timings of a profiled run: dicts of kernel, stage,
        batch_items, ms."""
        n = lib().ts_generated_launch_count(self._h)
        arr = (_LaunchRecord * max(1, n))()
        lib().ts_generated_launches(self._h, arr)
        return [{"kernel": KERNEL_KINDS[r.kind], "stage": r.stage, "batch_items": r.batch_items, "ms": r.ms}
                for r in arr[:n]]


class Batch:
    """The batched form: sessions added here run together, one launch per
    phase of each batch step carrying every session's step.  Each result is
    identical to Session.run on the same session."""

    def __init__(self, device=0, graph=False, profile=False, plan_threads=0, team=None, tuning=None):
        self._h = lib().ts_batch_new(device)
        if not self._h:
            raise Error(13, "ts_batch_new")
        if team is not None:
            lib().ts_batch_resolve_team(self._h, team[0], team[1])
        if tuning is not None:
            lib().ts_batch_tuning(self._h, C.byref(tuning))
        if graph:
            lib().ts_batch_use_graph(self._h, 1)
        if profile:
            lib().ts_batch_profile(self._h, 1)
        if plan_threads:
            lib().ts_batch_plan_threads(self._h, plan_threads)

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_batch_free(self._h)
            self._h = None

    def __len__(self):
        return int(lib().ts_batch_size(self._h))

    def _check(self, rc):
        if rc:
            msg = lib().ts_batch_last_error(self._h)
            raise Error(rc, msg.decode() if msg else "")

    def add(self, session):
        """Hands a built Session to the batch (the session is consumed)."""
        self._check(lib().ts_batch_add(self._h, session._h))
        return self

    def run(self):
        """Runs every added session; a list of GeneratedImage in add order."""
        n = len(self)
        out = (C.c_void_p * max(1, n))()
        self._check(lib().ts_batch_run(self._h, out))
        return [GeneratedImage(out[i]) for i in range(n)]

    def stats(self):
        st = _BatchStats()
        lib().ts_batch_stats_get(self._h, C.byref(st))
        d = {f: getattr(st, f) for f, _ in st._fields_ if not f.startswith("phase_")}
        d["phases"] = {name: {"launches": int(st.phase_launches[i]), "ms": float(st.phase_ms[i])}
                       for i, name in enumerate(BATCH_PHASES)}
        return d


class Server:
    """The served form: continuous batching of requests (built sessions).
    submit() queues a session and returns a ticket; wait(ticket) returns
    (GeneratedImage, times) with host timestamps in ms (submit, admit,
    done).  Results equal Session.run on the same session."""

    def __init__(self, device=0, hbm_budget=0, max_active=64, team=None, tuning=None):
        self._h = lib().ts_server_new(device, int(hbm_budget), int(max_active))
        if not self._h:
            raise Error(10, "ts_server_new: the device cannot be used")
        if team is not None:
            lib().ts_server_resolve_team(self._h, team[0], team[1])
        if tuning is not None:
            lib().ts_server_tuning(self._h, C.byref(tuning))

    def close(self):
        """Waits for every submitted request, then stops the server."""
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_server_free(self._h)
            self._h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _err(self, rc):
        msg = lib().ts_server_last_error(self._h)
        return Error(rc, msg.decode() if msg else "")

    def submit(self, session):
        ticket = C.c_uint64()
        rc = lib().ts_server_submit(self._h, session._h, C.byref(ticket))
        if rc:
            raise self._err(rc)
        return ticket.value

    def done(self, ticket):
        return lib().ts_server_done(self._h, ticket) == 1

    def wait(self, ticket):
        out = C.c_void_p()
        t = _RequestTimes()
        rc = lib().ts_server_wait(self._h, ticket, C.byref(out), C.byref(t))
        if rc:
            raise self._err(rc)
        return GeneratedImage(out.value), {"submit_ms": t.submit_ms, "admit_ms": t.admit_ms, "done_ms": t.done_ms}

    def stats(self):
        st = _ServerStats()
        lib().ts_server_stats_get(self._h, C.byref(st))
        return {f: getattr(st, f) for f, _ in st._fields_}


class CoordinateTransform:
    """CoordinateTransform (lib.rs:162-325): the source coordinate of every
    output pixel, written and read in the reference's binary format and
    applied to new sources on the device."""

    def __init__(self, handle):
        if not handle:
            raise Error(13, "coordinate transform")
        self._h = handle
        w, h, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
        lib().ts_transform_dims(self._h, C.byref(w), C.byref(h), C.byref(n))
        self.width, self.height, self.n_maps = w.value, h.value, n.value

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.ts_transform_free(self._h)
            self._h = None

    def original_maps(self):
        out = []
        for i in range(self.n_maps):
            w, h = C.c_uint32(), C.c_uint32()
            lib().ts_transform_map_dims(self._h, i, C.byref(w), C.byref(h))
            out.append(Dims(w.value, h.value))
        return out

    def write(self):
        """The serialised transform, as bytes."""
        n = C.c_size_t()
        rc = lib().ts_transform_write(self._h, None, 0, C.byref(n))
        if rc:
            raise Error(rc, "ts_transform_write")
        buf = (C.c_uint8 * n.value)()
        rc = lib().ts_transform_write(self._h, buf, n.value, C.byref(n))
        if rc:
            raise Error(rc, "ts_transform_write")
        return bytes(buf)

    @staticmethod
    def read(data):
        out = C.c_void_p()
        rc = lib().ts_transform_read(data, len(data), C.byref(out))
        if rc:
            raise Error(rc, "ts_transform_read: malformed transform")
        return CoordinateTransform(out.value)

    def apply(self, sources, device=0):
        """CoordinateTransform::apply: the output image (H x W x 4 uint8)."""
        imgs = [_rgba(im) for im in sources]
        descs = (_ImageDesc * max(1, len(imgs)))()
        for d, im in zip(descs, imgs):
            d.rgba, d.width, d.height = im.ctypes.data, im.shape[1], im.shape[0]
        out = np.empty((self.height, self.width, 4), np.uint8)
        rc = lib().ts_transform_apply(self._h, descs, len(imgs), out.ctypes.data, device)
        if rc:
            raise Error(rc, "ts_transform_apply")
        return out


def builder_from_spec(spec, batch_divisor=8, max_batch=0, device=0, profile=False, team_max_batch=None,
                      team_full_max_batch=256, tuning=None):
    """A SessionBuilder for a workload spec dict (see workloads.py)."""
    p = spec["params"]
    b = Session.builder()
    exs = spec["examples"]
    ip = spec.get("inpaint_mask")
    idx = spec.get("inpaint_index", -1)
    for i, e in enumerate(exs):
        ex = Example(e["image"])
        if e.get("guide") is not None:
            ex.with_guide(e["guide"])
        s = e.get("sample", "all")
        if s == "ignore":
            ex.set_sample_method(SampleMethod.IGNORE)
        elif s == "image":
            ex.set_sample_method(SampleMethod.Image(e["mask"]))
        if ip is not None and i == idx:
            b.inpaint_example(ip, ex, Dims(spec["out_w"], spec["out_h"]))
        else:
            b.add_example(ex)
    if spec.get("target_guide") is not None:
        b.load_target_guide(spec["target_guide"])
    b.output_size(Dims(spec["out_w"], spec["out_h"]))
    b.nearest_neighbors(p["nearest_neighbors"]).random_sample_locations(p["random_sample_locations"])
    b.cauchy_dispersion(p["cauchy_dispersion"]).backtrack_percent(p["backtrack_percent"])
    b.backtrack_stages(p["backtrack_stages"]).seed(p["seed"]).guide_alpha(p["guide_alpha"])
    b.tiling_mode(p["tiling_mode"])
    if p.get("random_init") is not None:
        b.random_init(p["random_init"])
    b.batch_schedule(batch_divisor, max_batch).device(device)
    if profile:
        b.profile_kernels(True)
    if team_max_batch is not None:
        b.resolve_team(team_max_batch, team_full_max_batch)
    if tuning is not None:
        b.tuning(tuning)
    return b


def autotune_session(make_builder, repeats=3):
    """The autotuner on the plain path (ts_autotune_session).  make_builder()
    returns a configured SessionBuilder for one run of the workload; it is
    called once per trial run.  Returns the fastest Tuning found."""
    errors = []

    @_BUILDER_FACTORY
    def factory(_user):
        try:
            sb = make_builder()
            h, sb._h = sb._h, None  # the tuner builds and frees it
            return h
        except Exception as e:  # reported after the tuner returns
            errors.append(e)
            return None

    t = Tuning()
    rc = lib().ts_autotune_session(factory, None, int(repeats), C.byref(t))
    if errors:
        raise errors[0]
    if rc:
        raise Error(rc, "ts_autotune_session")
    return t


def autotune_batch(make_sessions, device=0, repeats=2):
    """The autotuner on the batched form (ts_autotune_batch): make_sessions()
    returns the built Sessions of one batched run; it is called once per
    trial run.  Returns the fastest Tuning found (its team thresholds)."""
    errors = []

    @_BATCH_FILLER
    def fill(bh, _user):
        try:
            for s in make_sessions():
                rc = lib().ts_batch_add(bh, s._h)
                if rc:
                    return rc
            return 0
        except Exception as e:
            errors.append(e)
            return 11

    t = Tuning()
    rc = lib().ts_autotune_batch(int(device), fill, None, int(repeats), C.byref(t))
    if errors:
        raise errors[0]
    if rc:
        raise Error(rc, "ts_autotune_batch")
    return t


def run_spec(spec, batch_divisor=8, max_batch=0, device=0, team_max_batch=None, team_full_max_batch=256,
             tuning=None):
    """Build and run a workload spec; returns a dict shaped like the oracle's."""
    g = builder_from_spec(spec, batch_divisor, max_batch, device, team_max_batch=team_max_batch,
                          team_full_max_batch=team_full_max_batch, tuning=tuning).build().run()
    return generated_outputs(g)


def generated_outputs(g):
    """The outputs of a GeneratedImage as a dict shaped like the oracle's."""
    flat, score = g.resolved()
    st = g.stats()
    return {"image": g.into_image(), "coord": g.coord_map(), "id": g.id_map(), "resolved": flat,
            "scores": score, "evals": st["cost_evals"], "resolves": st["resolves"], "batches": st["batches"],
            "stats": st}
