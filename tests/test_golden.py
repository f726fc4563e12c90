"""The oracle reproduces the committed golden fixtures bit for bit
(tests/golden/make_golden.py made them; they pin the oracle across changes
and machines -- the Rust reference cannot be run here to pin it)."""
import glob
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)


def test_fixtures_exist():
    assert len(FIXTURES) >= 6


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_matches_golden(oracle, path):
    d = np.load(path)
    spec, divisor = mg.unpack(d)
    r = oracle.run(spec, batch_divisor=divisor, nthreads=2)
    for k in ("image", "coord", "id", "resolved"):
        assert (r[k] == d["out_" + k]).all(), k
    assert (r["scores"].view(np.uint32) == d["out_scores"].view(np.uint32)).all()
    assert r["evals"] == int(d["out_evals"])
