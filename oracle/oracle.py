"""ctypes wrapper over the CPU oracle (test infrastructure only).

Used by tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline.  The product never imports this module.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class Example(C.Structure):
    _fields_ = [
        ("rgba", C.c_void_p),
        ("w", C.c_uint32),
        ("h", C.c_uint32),
        ("guide", C.c_void_p),
        ("gw", C.c_uint32),
        ("gh", C.c_uint32),
        ("sample_method", C.c_int32),
        ("mask", C.c_void_p),
    ]


class Params(C.Structure):
    _fields_ = [
        ("k", C.c_uint32),
        ("pad0", C.c_uint32),
        ("m", C.c_uint64),
        ("cauchy", C.c_float),
        ("p", C.c_float),
        ("stages", C.c_uint32),
        ("pad1", C.c_uint32),
        ("seed", C.c_uint64),
        ("alpha", C.c_float),
        ("tiling", C.c_int32),
        ("has_random_init", C.c_int32),
        ("pad2", C.c_uint32),
        ("random_init", C.c_uint64),
        ("out_w", C.c_uint32),
        ("out_h", C.c_uint32),
        ("batch_divisor", C.c_uint32),
        ("max_batch", C.c_uint32),
        ("nthreads", C.c_int32),
        ("pad3", C.c_uint32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("evals", C.c_uint64),
        ("resolves", C.c_uint64),
        ("batches", C.c_uint64),
        ("n_resolved", C.c_uint64),
    ]


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.tso_run.restype = C.c_int
        L.tso_run.argtypes = [
            C.POINTER(Params), C.c_uint32, C.POINTER(Example), C.c_void_p, C.c_void_p, C.c_int32,
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Stats),
        ]
        L.tso_resize.restype = C.c_int
        L.tso_resize.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int]
        L.tso_pyramid.restype = C.c_int
        L.tso_pyramid.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
        L.tso_pcg_seed.argtypes = [C.c_uint64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        L.tso_pcg_stream.argtypes = [C.c_uint64, C.c_uint32, C.c_void_p]
        L.tso_guide_map.restype = C.c_int
        L.tso_guide_map.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_uint32, C.c_uint32,
                                    C.c_void_p]
        L.tso_id_colour.restype = C.c_uint8
        L.tso_id_colour.argtypes = [C.c_uint64]
        L.tso_debug_maps.restype = None
        L.tso_debug_maps.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p,
                                     C.c_void_p, C.c_void_p]
        L.tso_gen_range_u32.restype = C.c_uint32
        L.tso_gen_range_u32.argtypes = [C.c_uint64, C.c_uint32]
        L.tso_gen_range_u64.restype = C.c_uint64
        L.tso_gen_range_u64.argtypes = [C.c_uint64, C.c_uint64]
        L.tso_exp_export.restype = C.c_double
        L.tso_exp_export.argtypes = [C.c_double]
        L.tso_knn.restype = C.c_size_t
        L.tso_knn.argtypes = [C.c_uint32, C.c_uint32, C.c_int, C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                              C.c_uint32, C.c_void_p]
        L.tso_exp_audit.restype = None
        L.tso_exp_audit.argtypes = [C.c_int]
        L.tso_exp_audit_counts.restype = None
        L.tso_exp_audit_counts.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
        _lib = L
    return _lib


def exp_audit(spec, **kw):
    """Runs spec with the exp audit on: (weights computed, weights whose f32
    value from the project exp differs from the C library's exp's)."""
    L = lib()
    L.tso_exp_audit(1)
    try:
        run(spec, **kw)
        n, d = C.c_uint64(), C.c_uint64()
        L.tso_exp_audit_counts(C.byref(n), C.byref(d))
    finally:
        L.tso_exp_audit(0)
    return n.value, d.value


class OracleError(RuntimeError):
    """A run the oracle refused; status is its TSO_ERR_* code (2 = no valid
    sample, 3 = index), numbered like the library's TS_ERR_NO_VALID_SAMPLE
    and TS_ERR_INDEX through NO_VALID_SAMPLE and INDEX below."""

    NO_VALID_SAMPLE = 2
    INDEX = 3

    def __init__(self, status):
        super().__init__("oracle run failed with status %d" % status)
        self.status = status


FILTERS = {"nearest": 0, "triangle": 1, "catmullrom": 2, "gaussian": 3}
SAMPLE = {"all": 0, "ignore": 1, "image": 2}


def _ptr(a):
    return None if a is None else a.ctypes.data


def resize(img, nw, nh, filt="catmullrom"):
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape[:2]
    out = np.zeros((nh, nw, 4), np.uint8)
    rc = lib().tso_resize(_ptr(img), w, h, _ptr(out), nw, nh, FILTERS[filt])
    if rc:
        raise RuntimeError("tso_resize failed: %d" % rc)
    return out


def pyramid(img, levels):
    img = np.ascontiguousarray(img, dtype=np.uint8)
    h, w = img.shape[:2]
    nl = max(1, levels)
    out = np.zeros((nl, h, w, 4), np.uint8)
    rc = lib().tso_pyramid(_ptr(img), w, h, levels, _ptr(out))
    if rc:
        raise RuntimeError("tso_pyramid failed: %d" % rc)
    return out


def run(spec, batch_divisor=8, max_batch=0, nthreads=1):
    """Run a session spec (see the package's workloads module for the dict
    layout) through the oracle.  Returns a dict of numpy outputs."""
    p = spec["params"]
    W, H = spec["out_w"], spec["out_h"]
    exs = spec["examples"]
    keep = []
    arr = (Example * len(exs))()
    for i, e in enumerate(exs):
        img = np.ascontiguousarray(e["image"], dtype=np.uint8)
        keep.append(img)
        arr[i].rgba = img.ctypes.data
        arr[i].h, arr[i].w = img.shape[:2]
        g = e.get("guide")
        if g is not None:
            g = np.ascontiguousarray(g, dtype=np.uint8)
            keep.append(g)
            arr[i].guide = g.ctypes.data
            arr[i].gh, arr[i].gw = g.shape[:2]
        arr[i].sample_method = SAMPLE[e.get("sample", "all")]
        mk = e.get("mask")
        if mk is not None:
            mk = np.ascontiguousarray(mk, dtype=np.uint8)
            keep.append(mk)
            arr[i].mask = mk.ctypes.data
    prm = Params()
    prm.k = p["nearest_neighbors"]
    prm.m = p["random_sample_locations"]
    prm.cauchy = p["cauchy_dispersion"]
    prm.p = p["backtrack_percent"]
    prm.stages = p["backtrack_stages"]
    prm.seed = p["seed"]
    prm.alpha = p["guide_alpha"]
    prm.tiling = 1 if p["tiling_mode"] else 0
    ri = p.get("random_init")
    prm.has_random_init = 0 if ri is None else 1
    prm.random_init = 0 if ri is None else ri
    prm.out_w, prm.out_h = W, H
    prm.batch_divisor = batch_divisor
    prm.max_batch = max_batch
    prm.nthreads = nthreads
    tg = spec.get("target_guide")
    if tg is not None:
        tg = np.ascontiguousarray(tg, dtype=np.uint8)
    ip = spec.get("inpaint_mask")
    if ip is not None:
        ip = np.ascontiguousarray(ip, dtype=np.uint8)
    N = W * H
    out = np.zeros((H, W, 4), np.uint8)
    coord = np.zeros((H, W, 3), np.uint32)
    ids = np.zeros((H, W, 2), np.uint32)
    resolved = np.zeros(N * 8, np.uint32)
    rscore = np.zeros(N * 8, np.float32)
    st = Stats()
    rc = lib().tso_run(C.byref(prm), len(exs), arr, _ptr(tg), _ptr(ip), spec.get("inpaint_index", -1),
                       _ptr(out), _ptr(coord), _ptr(ids), _ptr(resolved), _ptr(rscore), C.byref(st))
    if rc:
        raise OracleError(rc)
    n = st.n_resolved
    return {
        "image": out, "coord": coord, "id": ids,
        "resolved": resolved[:n].copy(), "scores": rscore[:n].copy(),
        "evals": st.evals, "resolves": st.resolves, "batches": st.batches,
    }


def knn(W, H, tiling, occ, mir, px, py, k):
    occ = np.ascontiguousarray(occ, dtype=np.uint8)
    mir = np.ascontiguousarray(mir, dtype=np.uint8)
    out = np.zeros((max(k, 1), 2), np.int32)
    n = lib().tso_knn(W, H, int(tiling), _ptr(occ), _ptr(mir), px, py, k, _ptr(out))
    return out[:n].copy()


def debug_maps(ids, flat, score):
    """get_id_maps and get_uncertainty_map (ms.rs:604-653) on the CPU: ids is
    H x W x 2 (patch, map), (flat, score) the resolved list."""
    ids = np.ascontiguousarray(ids, np.uint32)
    h, w = ids.shape[:2]
    flat = np.ascontiguousarray(flat, np.uint32)
    score = np.ascontiguousarray(score, np.float32)
    outs = [np.empty((h, w, 4), np.uint8) for _ in range(3)]
    lib().tso_debug_maps(ids.ctypes.data, h * w, flat.ctypes.data, score.ctypes.data, len(flat),
                         outs[0].ctypes.data, outs[1].ctypes.data, outs[2].ctypes.data)
    return tuple(outs)


def id_colour(seed):
    return int(lib().tso_id_colour(seed))


def guide_map(image, target):
    """transform_to_guide_map + match_histograms (utils.rs:101-183): the
    automatic guide of an example for a target guide, RGBA8."""
    img = np.ascontiguousarray(image, np.uint8)
    tgt = np.ascontiguousarray(target, np.uint8)
    out = np.empty_like(img)
    rc = lib().tso_guide_map(img.ctypes.data, img.shape[1], img.shape[0], tgt.ctypes.data, tgt.shape[1],
                             tgt.shape[0], out.ctypes.data)
    if rc:
        raise RuntimeError("tso_guide_map failed: %d" % rc)
    return out
