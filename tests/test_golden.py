"""The oracle reproduces its committed golden vectors (tests/golden/, made by
tests/golden/make_golden.py): integer and index data exactly, floating point
to 1e-12 relative (the sample stream goes through libm's log, which may
differ by an ulp between machines)."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden", "oracle_golden.npz")


@pytest.fixture(scope="module")
def fresh(oracle):
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.cases(oracle)


def test_golden_file_present():
    assert os.path.exists(GOLD)


def test_oracle_reproduces_golden(fresh):
    gold = np.load(GOLD)
    assert set(gold.files) == set(fresh)
    for k in gold.files:
        g, f = gold[k], fresh[k]
        assert g.shape == f.shape, k
        if g.dtype.kind in "iu":
            assert np.array_equal(g, f), k
        else:
            scale = max(1.0, float(np.max(np.abs(g)))) if g.size else 1.0
            assert np.max(np.abs(g - f)) <= 1e-12 * scale, k
