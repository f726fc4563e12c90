"""CoordinateTransform's binary format (lib.rs:168, 214-325) through the C
ABI without a GPU: read of a reference-layout buffer, write back byte for
byte, and the errors of malformed data."""
import struct

import numpy as np
import pytest


def transform_bytes(w, h, maps, buf):
    out = struct.pack("<4I", 0x12340001, w, h, len(maps))
    for mw, mh in maps:
        out += struct.pack("<2I", mw, mh)
    return out + np.asarray(buf, "<u4").tobytes()


def test_read_write_round_trip(ts):
    rng = np.random.default_rng(3)
    w, h = 7, 5
    buf = np.stack([rng.integers(0, 30, w * h), rng.integers(0, 20, w * h), rng.integers(0, 2, w * h)], 1)
    data = transform_bytes(w, h, [(30, 20), (40, 25)], buf.ravel())
    t = ts.CoordinateTransform.read(data)
    assert (t.width, t.height, t.n_maps) == (w, h, 2)
    assert t.original_maps() == [ts.Dims(30, 20), ts.Dims(40, 25)]
    assert t.write() == data


@pytest.mark.parametrize("mutate", ["magic", "version", "short", "empty"])
def test_malformed(ts, mutate):
    data = bytearray(transform_bytes(2, 2, [(4, 4)], np.zeros(12)))
    if mutate == "magic":
        data[3] = 0x99
    elif mutate == "version":
        data[0] = 0x02
    elif mutate == "short":
        data = data[:-4]
    else:
        data = bytearray()
    with pytest.raises(ts.Error) as e:
        ts.CoordinateTransform.read(bytes(data) if data else b"\0")
    assert e.value.kind == "InvalidRange"
