"""ts_image_pyramid_noalloc, the pyramid entry point that allocates no device
memory, against ts_image_pyramid: byte-identical pyramids, on calls made one
after another on one stream (the scratch array is reused), with the size
limits refused before any work is enqueued.

Device buffers come from torch (the caller owns them); the entry point is
called through the C ABI."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TS_OK, TS_ERR_IMAGE, TS_ERR_LIMIT, TS_ERR_NULL = 0, 6, 12, 14


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    t.cuda.set_device(0)
    return t


def _device_image(torch, img):
    return torch.from_numpy(np.ascontiguousarray(img)).to("cuda:0")


def _enqueue(ts, torch, d_in, w, h, levels, d_out, stream):
    return ts.lib().ts_image_pyramid_noalloc(C.c_void_p(d_in.data_ptr()), w, h, levels,
                                             C.c_void_p(d_out.data_ptr()), C.c_void_p(stream.cuda_stream))


def _check(got, img, levels, ts):
    ref = ts.image_pyramid(img, levels)
    assert got.shape == ref.shape
    bad = np.argwhere(got != ref)
    assert len(bad) == 0, "pyramid differs at %d places, first %s" % (len(bad), bad[:3].tolist())


def test_two_calls_in_a_row_match_the_allocating_entry_point(ts, wl, torch):
    cases = [(200, 300, 5), (77, 129, 4)]
    imgs = [wl.texture(31 + i, h, w) for i, (h, w, _) in enumerate(cases)]
    d_in = [_device_image(torch, im) for im in imgs]
    d_out = [torch.empty((max(1, l), h, w, 4), dtype=torch.uint8, device="cuda:0") for h, w, l in cases]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        for (h, w, l), di, do in zip(cases, d_in, d_out):
            assert _enqueue(ts, torch, di, w, h, l, do, stream) == TS_OK
    stream.synchronize()
    for (h, w, l), im, do in zip(cases, imgs, d_out):
        _check(do.cpu().numpy(), im, l, ts)


def test_repeated_call_reuses_scratch_without_allocating(ts, wl, torch):
    h, w, levels = 160, 96, 4
    img = wl.texture(5, h, w)
    d_in = _device_image(torch, img)
    outs = [torch.zeros((levels, h, w, 4), dtype=torch.uint8, device="cuda:0") for _ in range(3)]
    stream = torch.cuda.current_stream()
    assert _enqueue(ts, torch, d_in, w, h, levels, outs[0], stream) == TS_OK
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    for o in outs[1:]:
        assert _enqueue(ts, torch, d_in, w, h, levels, o, stream) == TS_OK
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free_before
    first = outs[0].cpu().numpy()
    _check(first, img, levels, ts)
    for o in outs[1:]:
        assert (o.cpu().numpy() == first).all()


@pytest.mark.parametrize("h,w,levels", [(3, 5, 4), (64, 48, 1), (50, 70, 0), (1024, 1024, 3), (1, 4096, 2)])
def test_edge_sizes(ts, wl, torch, h, w, levels):
    img = wl.texture(h + 3 * w, h, w)
    d_in = _device_image(torch, img)
    d_out = torch.empty((max(1, levels), h, w, 4), dtype=torch.uint8, device="cuda:0")
    assert _enqueue(ts, torch, d_in, w, h, levels, d_out, torch.cuda.current_stream()) == TS_OK
    torch.cuda.synchronize()
    _check(d_out.cpu().numpy(), img, levels, ts)


@pytest.mark.parametrize("h,w,levels,status", [
    (1024, 1025, 1, TS_ERR_LIMIT),   # more than 1024 * 1024 pixels
    (1, 4097, 1, TS_ERR_LIMIT),      # a side above 4096
    (8, 8, 17, TS_ERR_LIMIT),        # more than 16 levels
    (0, 8, 2, TS_ERR_IMAGE),
])
def test_refusals(ts, torch, h, w, levels, status):
    # buffers sized for the request, so nothing could go out of bounds
    d_in = torch.zeros((max(1, h), w, 4), dtype=torch.uint8, device="cuda:0")
    d_out = torch.zeros((max(1, levels), max(1, h), w, 4), dtype=torch.uint8, device="cuda:0")
    assert _enqueue(ts, torch, d_in, w, h, levels, d_out, torch.cuda.current_stream()) == status
    torch.cuda.synchronize()
    assert int(d_out.sum().item()) == 0


def test_null_buffers(ts, torch):
    lib = ts.lib()
    d = torch.zeros((4, 4, 4), dtype=torch.uint8, device="cuda:0")
    assert lib.ts_image_pyramid_noalloc(None, 4, 4, 1, C.c_void_p(d.data_ptr()), None) == TS_ERR_NULL
    assert lib.ts_image_pyramid_noalloc(C.c_void_p(d.data_ptr()), 4, 4, 1, None, None) == TS_ERR_NULL
