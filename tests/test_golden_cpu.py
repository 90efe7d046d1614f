"""The committed golden fixtures (tests/golden/path_cases.npz, written by
tests/golden/make_golden.py from the pinned oracle) are reproduced by the
oracle: integer outputs exactly, floating-point ones to 1e-13 relative (the
host libm may differ in the last bit between machines)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

FIX = os.path.join(HERE, "golden", "path_cases.npz")


def test_oracle_reproduces_the_golden_fixtures():
    want = np.load(FIX)
    got = make_golden.cases()
    assert sorted(got) == sorted(want.files)
    for k in want.files:
        a, b = np.asarray(got[k]), want[k]
        assert a.shape == b.shape, k
        if np.issubdtype(b.dtype, np.integer):
            assert np.array_equal(a, b), k
        else:
            both_nan = np.isnan(a) & np.isnan(b)
            d = np.abs(a - b)[~both_nan]
            den = np.maximum(np.abs(b), 1e-300)[~both_nan]
            assert (np.isnan(a) == np.isnan(b)).all(), k
            assert d.size == 0 or np.max(d / den) <= 1e-13, k
