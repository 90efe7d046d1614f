"""CvResult's summary measures (validation.rs:21-117) on hand-computed cases."""
import numpy as np

import geostat_rs as G


def test_cv_measures():
    o = np.array([1.0, 2.0, 3.0, 4.0])
    p = np.array([1.5, 1.5, 3.5, 3.0])
    v = np.array([0.25, 0.0, 1.0, 4.0])
    cv = G.CvResult(o, p, v)
    r = p - o
    assert cv.mean_error() == r.mean()
    assert cv.mae() == np.abs(r).mean()
    assert abs(cv.rmse() - np.sqrt((r * r).mean())) < 1e-15
    m = o.mean()
    assert abs(cv.rme() - (-r.mean() / m * 100)) < 1e-12
    assert abs(cv.vecv() - (1 - (r * r).sum() / ((o - m) ** 2).sum()) * 100) < 1e-12
    assert abs(cv.e1() - (1 - np.abs(r).sum() / np.abs(o - m).sum()) * 100) < 1e-12
    ok = v > 1e-12
    assert abs(cv.msdr() - (r[ok] ** 2 / v[ok]).mean()) < 1e-12
    z = G.CvResult(np.array([1.0, -1.0]), np.array([0.0, 0.0]), np.zeros(2))
    assert np.isnan(z.rme()) and np.isnan(z.msdr())
    flat = G.CvResult(np.ones(3), np.ones(3), np.ones(3))
    assert np.isnan(flat.vecv()) and np.isnan(flat.e1())
