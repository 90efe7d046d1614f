"""Cross-validation (validation.rs, tuning.rs) on the GPU against the oracle.

The oracle side follows the reference literally: for leave-one-out it builds a
predictor on the data without point i and predicts point i; for k-fold it
assigns folds by the reference's seeded shuffle and predicts each fold from the
others.  Tolerance: the parity bar of tests/gpu_common.py (1e-9 relative with
the usual floors); the GPU side keeps the full data's drift normalisation,
which changes results only by rounding.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, sph200_model, smooth_values, uniform_points

pytestmark = pytest.mark.gpu


def oracle_loo(c, v, model, okw, drift=None):
    n = len(c)
    pred, var = np.empty(n), np.empty(n)
    for i in range(n):
        keep = np.arange(n) != i
        kw = dict(okw)
        if drift is not None:
            kw.update(drift=drift[keep], target_drift=drift[i:i + 1])
        r = O.krige(c[keep], v[keep], model, c[i:i + 1], **kw)
        assert r["status"][0] == 0
        pred[i], var[i] = r["value"][0], r["variance"][0]
    return pred, var


def folds(n, k, seed):
    order = np.arange(n)
    u = O.rng_u64(seed, n)
    for idx, i in enumerate(range(n - 1, 0, -1)):
        j = int(u[idx] % np.uint64(i + 1))
        order[i], order[j] = order[j], order[i]
    fold_of = np.empty(n, dtype=int)
    fold_of[order] = np.arange(n) % k
    return fold_of


def check(cv, pred, var, v, sill):
    assert_close(cv.predicted, pred, float(np.mean(np.abs(v))), 1e-9, "predicted")
    assert_close(cv.variance, var, 1e-3 * sill, 1e-9, "variance")


@pytest.mark.parametrize("case", ["knn", "octant_uk", "global", "radius"])
def test_leave_one_out_matches_oracle(case):
    n = 60 if case == "global" else 400
    c = uniform_points(n, 2, 71, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    cfg = {"knn": G.KrigingConfig(max_neighbors=16),
           "octant_uk": G.KrigingConfig("universal", degree=1, max_per_octant=5),
           "global": G.KrigingConfig(),
           "radius": G.KrigingConfig(max_neighbors=24, search_radius=250.0, min_neighbors=3)}[case]
    okw = dict(method=cfg.method, degree=cfg.degree, max_neighbors=cfg.max_neighbors,
               max_per_octant=cfg.max_per_octant, radius=cfg.search_radius,
               min_neighbors=cfg.min_neighbors)
    pred, var = oracle_loo(c, v, m, okw)
    for prec in ("mixed", "fp64"):
        cv = G.leave_one_out(G.PointSet(c, v), m, cfg, precision=prec)
        assert np.array_equal(cv.observed, v)
        check(cv, pred, var, v, m.total_sill())


def test_leave_one_out_with_drift_matches_oracle():
    c = uniform_points(300, 2, 72, [1000.0, 1000.0])
    cov = O.rng_uniform(73, 300)
    v = smooth_values(c) + 2.0 * cov
    m = sph200_model()
    cfg = G.KrigingConfig("external_drift", n_vars=1, max_neighbors=20)
    pred, var = oracle_loo(c, v, m, dict(method="external_drift", max_neighbors=20),
                           drift=cov.reshape(-1, 1))
    cv = G.leave_one_out_with_drift(G.PointSet(c, v), cov.reshape(-1, 1), m, cfg)
    check(cv, pred, var, v, m.total_sill())


@pytest.mark.parametrize("k,seed", [(5, 11), (2, 3), (400, 7)])
def test_k_fold_matches_oracle(k, seed):
    n = 400
    c = uniform_points(n, 2, 74, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    fold_of = folds(n, k, seed)
    pred, var = np.empty(n), np.empty(n)
    for f in range(k):
        tr, te = fold_of != f, fold_of == f
        if not te.any():
            continue
        r = O.krige(c[tr], v[tr], m, c[te], max_neighbors=16)
        pred[te], var[te] = r["value"], r["variance"]
    cv = G.k_fold(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=16), k, seed)
    check(cv, pred, var, v, m.total_sill())


def test_cross_validation_3d_and_errors():
    c = uniform_points(300, 3, 75, [500.0, 500.0, 100.0])
    v = smooth_values(c)
    m = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 200.0, 30.0, 10.0, 0.0,
                                                      0.5, 0.3)])
    pred, var = oracle_loo(c, v, m, dict(max_neighbors=24))
    cv = G.leave_one_out(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=24))
    check(cv, pred, var, v, m.total_sill())
    small = G.PointSet(c[:2], v[:2])
    with pytest.raises(G.InsufficientData):
        G.leave_one_out(small, m)
    with pytest.raises(G.InvalidParameter):
        G.k_fold(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=8), 1, 0)
    with pytest.raises(G.InvalidParameter):
        G.k_fold(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=8), 301, 0)
    # min_neighbors above what a held-out point can have: the call fails
    far = np.vstack([c, [[5000.0, 5000.0, 0.0]]])
    with pytest.raises(G.NoNeighbors):
        G.leave_one_out(G.PointSet(far, np.append(v, 1.0)), m,
                        G.KrigingConfig(max_neighbors=8, search_radius=300.0, min_neighbors=2))


def test_tune_kriging_neighbors_matches_oracle_trace():
    c = uniform_points(250, 2, 76, [1000.0, 1000.0])
    v = smooth_values(c)
    m = sph200_model()
    cands = [4, 8, 16, 32]
    res = G.tune_kriging_neighbors(G.PointSet(c, v), m, "ordinary", cands)
    for (nb, vecv), k in zip(res.trace, cands):
        pred, _ = oracle_loo(c, v, m, dict(max_neighbors=k))
        ref = G.CvResult(v, pred, np.ones_like(v)).vecv()
        assert nb == k and abs(vecv - ref) <= 1e-9 * abs(ref)
    assert res.best_vecv == max(t[1] for t in res.trace)
