"""The FP64 re-solve kernels' table-driven exp(-x) against the host libm.

Tolerance: at most 2 units in the last place of the host value for
0 <= x < 708 (the method's error is about 1 ulp, the host's at most 1 ulp);
exactly 0 for x >= 708, where exp(-x) < 3.3e-308.
"""
import numpy as np
import pytest

import gs_workload as W

pytestmark = pytest.mark.gpu


def _dev_expneg(x):
    return W.probe_expneg(x)


def test_expneg_within_two_ulp():
    rng = np.random.default_rng(3)
    ln2_128 = np.log(2.0) / 128
    x = np.concatenate([
        [0.0, 5e-324, 1e-300, 1e-17, 1e-9, ln2_128, 2 * ln2_128, 3 * ln2_128, 0.5, 1.0,
         np.log(2.0), 700.0, 707.99],
        np.linspace(0.0, 1e-3, 10_001),
        rng.uniform(0.0, 1.0, 200_000),
        rng.uniform(0.0, 50.0, 200_000),
        rng.uniform(0.0, 708.0, 200_000),
        np.arange(1, 64 * 1100) * ln2_128 * 2,  # table boundaries
    ])
    x = x[x < 708.0]
    got = _dev_expneg(x)
    ref = np.exp(-x)
    ulp = np.abs(got - ref) / np.spacing(ref)
    assert np.all(np.isfinite(got))
    assert ulp.max() <= 2.0, f"max {ulp.max():.2f} ulp at x = {x[np.argmax(ulp)]!r}"


def test_expneg_underflows_to_zero():
    x = np.array([708.0, 710.0, 745.0, 1e4, 1e300])
    assert (_dev_expneg(x) == 0.0).all()
