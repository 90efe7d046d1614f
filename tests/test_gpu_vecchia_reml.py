"""Vecchia REML and the grouped MLE on the GPU against the oracle.

REML log-likelihoods (polynomial trends of degree 0-2, external-drift bases
including a UTM-scale covariate; ungrouped and Guinness-grouped) agree with
the oracle within 1e-9 relative; the full-conditioning REML equals the exact
restricted likelihood; the fits reproduce the reference's REML tests
(vecchia.rs:2504-2645) and match the oracle's Nelder-Mead on the same starts.
"""
import math

import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Structure, VariogramModel
from gpu_common import uniform_points

pytestmark = pytest.mark.gpu


def _models():
    return [VariogramModel(0.05, [Structure("exponential", 1.0, 0.1)]),
            VariogramModel(0.02, [Structure("matern25", 1.0, 0.05)]),
            VariogramModel(0.1, [Structure("spherical", 0.7, 0.3), Structure("gaussian", 0.3, 0.2)])]


@pytest.fixture(scope="module", params=[2, 3])
def field(request):
    dim = request.param
    c = uniform_points(3000, dim, 201 + dim, [1.0] * dim)
    v = 2.0 + 3.0 * c[:, 0] - c[:, 1] + W.rff_field(c, _models()[1], 512, 202)
    return c, v


@pytest.mark.parametrize("deg,g,m", [(0, 1, 15), (1, 1, 15), (2, 1, 10), (1, 4, 15), (2, 8, 10)])
def test_reml_loglik_poly_matches_oracle(field, deg, g, m):
    c, v = field
    plan = G.VecchiaPlan(G.PointSet(c, v), m)
    order, nb, cnt = plan.arrays()
    ll, st = plan.reml_loglik(_models(), drift_degree=deg, group_size=g)
    assert (st == 0).all()
    f = O.poly_basis(c, deg)
    for i, mdl in enumerate(_models()):
        ref = O.vecchia_reml_loglik(c, v, mdl, order, nb, cnt, f, g)
        assert abs(ll[i] - ref) <= 1e-9 * abs(ref), (i, ll[i], ref)


@pytest.mark.parametrize("g", [1, 4])
def test_reml_loglik_drift_matches_oracle(field, g):
    c, v = field
    plan = G.VecchiaPlan(G.PointSet(c, v), 12)
    order, nb, cnt = plan.arrays()
    cov = np.stack([600_000.0 + 1e4 * np.exp(-((c[:, 0] - 0.5) ** 2) / 0.05),
                    np.sin(7.0 * c[:, 1])], 1)
    ll, st = plan.reml_loglik(_models(), drift=cov, group_size=g)
    assert (st == 0).all()
    f = O.drift_basis(cov)
    for i, mdl in enumerate(_models()):
        ref = O.vecchia_reml_loglik(c, v, mdl, order, nb, cnt, f, g)
        assert abs(ll[i] - ref) <= 1e-9 * abs(ref), (i, ll[i], ref)


def _cov_matrix(c, m):
    sill = m.nugget + sum(s.sill for s in m.structures)
    n = len(c)
    return np.array([[sill if a == b else sill - O.gamma_dh(m, c[a] - c[b]) for b in range(n)]
                     for a in range(n)])


def test_reml_full_conditioning_equals_exact_on_device():
    # vecchia.rs:2466-2481
    c, v = O.test_field_2d(16, 4)
    m = VariogramModel(0.05, [Structure("exponential", 1.0, 35.0)])
    f = O.poly_basis(c, 1)
    s = _cov_matrix(c, m)
    siz, sif = np.linalg.solve(s, v), np.linalg.solve(s, f)
    amat, cvec = f.T @ sif, f.T @ siz
    beta = np.linalg.solve(amat, cvec)
    exact = -0.5 * ((16 - 3) * math.log(2 * math.pi) + np.linalg.slogdet(s)[1]
                    + np.linalg.slogdet(amat)[1] + v @ siz - cvec @ beta)
    plan = G.VecchiaPlan(G.PointSet(c, v), 15)
    for g in (1, 2, 5):
        ll, st = plan.reml_loglik([m], drift_degree=1, group_size=g)
        assert st[0] == 0 and abs(ll[0] - exact) < 1e-7


def _gp_field(seed, n):
    u, eps = O.rng_draw(seed, 2 * n, n)
    c = u.reshape(n, 2) * 60.0
    truth = VariogramModel(0.05, [Structure("exponential", 1.0, 10.0)])
    return c, np.linalg.cholesky(_cov_matrix(c, truth)) @ eps


def test_reml_fit_tames_the_range_and_matches_oracle():
    # vecchia.rs:2504-2545, and the oracle's Nelder-Mead from the same starts
    c, gp = _gp_field(20, 90)
    v = 0.3 * c[:, 0] - 0.2 * c[:, 1] + gp
    ps = G.PointSet(c, v)
    ml_model, _, _, _ = G.vecchia_mle_fit(ps, "exponential", 8)
    model, ll, x, _ = G.vecchia_reml_fit(ps, "exponential", 8, drift_degree=1)
    reml_r = model.structures[0].range
    assert reml_r < ml_model.structures[0].range and reml_r < 40.0
    starts, _ = O.vecchia_mle_setup(c, v)
    xr, fr, _ = O.vecchia_fit_nm(c, v, "exponential", 8, starts, basis=O.poly_basis(c, 1))
    assert abs(-ll - fr) <= 1e-7 * abs(fr)
    assert np.max(np.abs(x[1:] - xr[1:])) < 1e-3
    # the Python binding's form (lib.rs:370-392)
    m2 = G.vecchia_reml(c[:, 0], c[:, 1], v, "exponential", 8, 1)
    assert abs(m2.structures[0].range - reml_r) < 1e-9 * reml_r


@pytest.mark.parametrize("utm", [False, True])
def test_reml_drift_fit_recovers_range(utm):
    # vecchia.rs:2548-2588, 2590-2638
    c, gp = _gp_field(21, 90)
    cov = np.exp(-((c[:, 0] - 30.0) ** 2 + (c[:, 1] - 30.0) ** 2) / 200.0)
    v = 8.0 * cov + gp
    drift = (600_000.0 + 1e4 * cov) if utm else cov
    model, ll, x, _ = G.vecchia_reml_drift_fit(G.PointSet(c, v), drift.reshape(-1, 1),
                                               "exponential", 8)
    assert model.structures[0].range < 40.0
    starts, _ = O.vecchia_mle_setup(c, v)
    xr, fr, _ = O.vecchia_fit_nm(c, v, "exponential", 8, starts,
                                 basis=O.drift_basis(drift.reshape(-1, 1)))
    assert abs(-ll - fr) <= 1e-7 * abs(fr)


def test_reml_drift_rejects_bad_covariates():
    # vecchia.rs:2641-2648
    c, v = O.test_field_2d(20, 1)
    ps = G.PointSet(c, v)
    with pytest.raises(G.DimensionMismatch):
        G.vecchia_reml_drift_fit(ps, [[1.0]], "exponential", 5)
    with pytest.raises(G.InvalidParameter):
        G.vecchia_reml_drift_fit(ps, [[] for _ in range(20)], "exponential", 5)
    with pytest.raises(G.InsufficientData):
        G.vecchia_reml_fit(G.PointSet(c[:4], v[:4]), "exponential", 3, drift_degree=1)


def test_grouped_mle_matches_ungrouped_under_full_conditioning():
    # vecchia.rs:2110-2128
    c, v = O.test_field_2d(16, 21)
    ps = G.PointSet(c, v)
    mu, llu, _, _ = G.vecchia_mle_fit(ps, "exponential", 15)
    mg, llg, _, _ = G.vecchia_mle_grouped_fit(ps, "exponential", 15, group_size=4)
    assert abs(llu - llg) < 1e-6
    assert abs(mu.nugget - mg.nugget) < 1e-4
    assert abs(mu.structures[0].sill - mg.structures[0].sill) < 1e-3
    assert abs(mu.structures[0].range - mg.structures[0].range) < 1e-2
    # and the oracle's grouped Nelder-Mead from the same starts
    starts, _ = O.vecchia_mle_setup(c, v)
    xr, fr, _ = O.vecchia_fit_nm(c, v, "exponential", 15, starts, group_size=4)
    assert abs(-llg - fr) <= 1e-8 * abs(fr)


def test_reml_large_sets_and_sorted_order_blocks():
    """m = 40 (beyond the mixed warp kernel: the FP64 block kernel for every
    point) and a coordinate-sorted order, whose consecutive points share
    neighbours so that Guinness blocks have many members."""
    c = uniform_points(2500, 2, 211, [1.0, 1.0])
    v = 1.0 + 2.0 * c[:, 1] + W.rff_field(c, _models()[0], 512, 212)
    plan = G.VecchiaPlan(G.PointSet(c, v), 40)
    order, nb, cnt = plan.arrays()
    ll, st = plan.reml_loglik(_models(), drift_degree=1)
    assert (st == 0).all()
    f = O.poly_basis(c, 1)
    for i, mdl in enumerate(_models()):
        ref = O.vecchia_reml_loglik(c, v, mdl, order, nb, cnt, f, 1)
        assert abs(ll[i] - ref) <= 1e-9 * abs(ref), (i, ll[i], ref)
    srt = np.lexsort((c[:, 1], np.floor(c[:, 0] * 20)))
    plan = G.VecchiaPlan(G.PointSet(c, v), 12, srt)
    order, nb, cnt = plan.arrays()
    for g in (4, 8):
        llg, stg = plan.loglik_grouped(_models(), g)
        llr, str_ = plan.reml_loglik(_models(), drift_degree=1, group_size=g)
        assert (stg == 0).all() and (str_ == 0).all()
        for i, mdl in enumerate(_models()):
            ref = O.vecchia_loglik_grouped(c, v, mdl, order, nb, cnt, g)
            assert abs(llg[i] - ref) <= 1e-9 * abs(ref), (g, i, llg[i], ref)
            ref = O.vecchia_reml_loglik(c, v, mdl, order, nb, cnt, f, g)
            assert abs(llr[i] - ref) <= 1e-9 * abs(ref), (g, i, llr[i], ref)


@pytest.mark.parametrize("seed,nug", [(31, 0.2), (51, 0.0)])
def test_param_se_matches_oracle(seed, nug):
    """vecchia_param_se (vecchia.rs:1666-1935): the batched GPU gradients
    give the oracle's semi-analytical standard errors (finite differences of
    the gradient: agreement at 1e-6 relative)."""
    truth = VariogramModel(nug, [Structure("exponential", 1.0, 12.0)])
    u, eps = O.rng_draw(seed, 280, 140)
    c = u.reshape(140, 2) * 60.0
    v = np.linalg.cholesky(_cov_matrix(c, truth)) @ eps
    # away from the optimum for the interior case; at the truth on the
    # boundary, where the restricted (sill, range) information is positive
    # definite (vecchia.rs:2686-2725)
    sill, rng_ = (1.1, 13.0) if nug > 0 else (1.0, 12.0)
    model = VariogramModel(nug, [Structure("exponential", sill, rng_)])
    got = G.vecchia_param_se_fit(G.PointSet(c, v), model, 12)
    ref = O.vecchia_param_se(c, v, "exponential", nug, sill, rng_, 12)
    for a, b in zip(got, ref):
        if np.isnan(b):
            assert np.isnan(a)
        else:
            assert abs(a - b) <= 1e-6 * abs(b), (got, ref)
    if nug == 0.0:
        assert np.isnan(got[0]) and got[1] > 0 and got[2] > 0
    got2 = G.vecchia_param_se(c[:, 0], c[:, 1], v, model, 12)
    assert np.allclose(got2, got, equal_nan=True)


def test_loo_cv_binding_forms():
    """lib.rs:695-745 loo_cv: leave-one-out, k-fold and block forms."""
    c = uniform_points(300, 2, 221, [100.0, 100.0])
    v = np.sin(c[:, 0] / 20.0) + np.cos(c[:, 1] / 20.0)
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 50.0)])
    loo = G.loo_cv(c[:, 0], c[:, 1], v, m, max_neighbors=16)
    kf = G.loo_cv(c[:, 0], c[:, 1], v, m, max_neighbors=16, folds=5, seed=3)
    bl = G.loo_cv(c[:, 0], c[:, 1], v, m, max_neighbors=16, blocks=(3, 3))
    for d in (loo, kf, bl):
        assert set(d) >= {"me", "mae", "rmse", "msdr", "vecv", "e1", "observed", "predicted",
                          "variance"}
        assert np.isfinite(d["predicted"]).all()
    assert bl["rmse"] >= loo["rmse"]
    with pytest.raises(G.InvalidParameter):
        G.loo_cv(c[:, 0], c[:, 1], v, m, folds=5, blocks=(2, 2))
