"""GPU parity of the Vecchia plan, log-likelihood and MLE against the oracle."""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Structure, VariogramModel
from gpu_common import assert_close, uniform_points

pytestmark = pytest.mark.gpu


def matern25(nug=0.02, sill=1.0, rng=0.05):
    return VariogramModel(nug, [Structure("matern25", sill, rng)])


@pytest.mark.parametrize("dim,n,m", [(2, 3000, 30), (3, 2500, 20), (2, 60, 100), (2, 5000, 8)])
def test_plan_matches_reference_plan_exactly(dim, n, m):
    if dim == 2:
        c, v = O.test_field_2d(n, 100 + n)
    else:
        c, v = O.test_field_3d(n, 100 + n)
    plan = G.VecchiaPlan(G.PointSet(c, v), m)
    order, nb, cnt = plan.arrays()
    o_ref, nb_ref, cnt_ref = O.vecchia_plan(c, m)
    assert order.tolist() == o_ref.tolist()
    assert (cnt == cnt_ref).all()
    mm = nb.shape[1]
    assert (nb == nb_ref[:, :mm]).all()


def test_plan_with_given_order():
    c, v = O.test_field_2d(2000, 7)
    order = np.arange(2000)[::-1].copy()
    plan = G.VecchiaPlan(G.PointSet(c, v), 15, order)
    o, nb, cnt = plan.arrays()
    o_ref, nb_ref, cnt_ref = O.vecchia_plan(c, 15, order)
    assert o.tolist() == o_ref.tolist() and (nb == nb_ref).all() and (cnt == cnt_ref).all()


def test_loglik_batch_matches_oracle_and_is_batch_invariant():
    c = uniform_points(20000, 2, 3, [1.0, 1.0])
    v = 0.5 + W.rff_field(c, matern25(), 1024, 5)
    ps = G.PointSet(c, v)
    plan = G.VecchiaPlan(ps, 30)
    order, nb, cnt = plan.arrays()
    models = [matern25(), matern25(0.05, 0.8, 0.08), matern25(0.001, 1.5, 0.02),
              VariogramModel(0.02, [Structure("exponential", 1.0, 0.05)]),
              VariogramModel(0.02, [Structure.with_anisotropy("spherical", 0.7, 0.2, 30.0, 0.5),
                                    Structure("matern15", 0.3, 0.05)])]
    ll, st = plan.loglik(models)
    assert (st == 0).all()
    for i, mdl in enumerate(models):
        ref = O.vecchia_loglik_plan(c, v, mdl, order, nb, cnt)
        assert_close([ll[i]], [ref], 1.0, 1e-9, f"candidate {i}")
        one, _ = plan.loglik([mdl])
        assert one[0] == ll[i]
    ll64, st64 = plan.loglik(models, precision="fp64")
    assert (st64 == 0).all()
    for i, mdl in enumerate(models):
        ref = O.vecchia_loglik_plan(c, v, mdl, order, nb, cnt)
        assert_close([ll64[i]], [ref], 1.0, 1e-11, f"fp64 candidate {i}")


def test_full_conditioning_equals_exact_likelihood():
    # vecchia.rs:1998-2010
    c, v = O.test_field_2d(14, 3)
    m = VariogramModel(0.05, [Structure("exponential", 1.0, 40.0)])
    got = G.vecchia_loglik(c[:, 0], c[:, 1], v, m, 13)
    assert abs(got - O.exact_loglik(c, v, m)) < 1e-9


def test_vecchia_loglik_entry_point_3d():
    c, v = O.test_field_3d(3000, 17)
    m = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 40.0, 20.0, 10.0, 5.0,
                                                      0.6, 0.4)])
    plan = G.VecchiaPlan(G.PointSet(c, v), 25)
    ll, st = plan.loglik([m])
    ref = O.vecchia_loglik(c, v, m, 25)
    assert st[0] == 0
    assert_close(ll, [ref], 1.0, 1e-9, "3-D loglik")


def test_rejected_models():
    c, v = O.test_field_2d(50, 1)
    plan = G.VecchiaPlan(G.PointSet(c, v), 5)
    ll, st = plan.loglik([VariogramModel(0.0, [Structure("power", 1.0, 1.0, param=1.0)])])
    assert st[0] == G.InvalidParameter.code and np.isnan(ll[0])
    with pytest.raises(G.InvalidParameter):
        G.VecchiaPlan(G.PointSet(c, v), 0)
    with pytest.raises(G.InsufficientData):
        G.VecchiaPlan(G.PointSet(c[:1], v[:1]), 3)


def test_mle_objective_parity_and_batched_nelder_mead():
    c, v = O.test_field_2d(400, 21)
    ps = G.PointSet(c, v)
    starts, rmax = O.vecchia_mle_setup(c, v)
    model, ll, x, nev = G.vecchia_mle_nm_fit(ps, "exponential", 12, starts=starts, max_iter=400)
    xr, fr, nr = O.vecchia_mle_nm(c, v, "exponential", 12, starts, max_iter=400)
    # same algorithm, same objective to ~1e-12: the optimum agrees closely
    assert abs(-ll - fr) <= 1e-7 * abs(fr)
    # x = (sqrt nugget, ln psill, ln range): the objective is even in x[0], so
    # simplices that part ways on ~1e-12 objective differences may end on
    # mirror images; the fitted model (nugget = x0^2) is what must agree
    assert abs(x[0] ** 2 - xr[0] ** 2) < 1e-3 * max(xr[0] ** 2, 1e-3)
    assert np.max(np.abs(x[1:] - xr[1:])) < 1e-3
    o, nb, cnt = O.vecchia_plan(c, 12)
    fx = O.vecchia_mle_objective(c, v, "exponential", 12, o, nb, cnt, rmax, x)
    assert abs(fx[0] + ll) <= 1e-9 * abs(fx[0])
    assert model.nugget >= 0 and model.structures[0].range > 0


# ------------------------------------------------------- joint prediction --
@pytest.mark.parametrize("dim,n,nt,m", [(2, 3000, 800, 30), (2, 2000, 600, 8), (3, 2000, 500, 20),
                                        (2, 1200, 300, 40)])
def test_vecchia_predict_matches_oracle(dim, n, nt, m):
    """vecchia.rs:748-866: targets appended after the data in max-min order,
    each conditioning on its m nearest earlier store points; m > 32 runs the
    FP64 Cholesky path for every target."""
    if dim == 2:
        c, v = O.test_field_2d(n, 300 + n)
        t = uniform_points(nt, 2, 301, [100.0, 100.0])
        mdl = VariogramModel(0.05, [Structure("exponential", 0.95, 25.0)])
    else:
        c, v = O.test_field_3d(n, 302)
        t = uniform_points(nt, 3, 303, [100.0, 100.0, 100.0])
        mdl = VariogramModel(0.05, [Structure.with_rotation("spherical", 0.9, 40.0, 20.0, 10.0, 5.0,
                                                            0.6, 0.4)])
    gv, gvar = G.vecchia_predict(c, v, mdl, t, m)
    rv, rvar = O.vecchia_predict(c, v, mdl, t, m)
    assert_close(gv, rv, float(np.mean(np.abs(v))), 1e-9, "value")
    assert_close(gvar, rvar, mdl.total_sill(), 1e-9, "variance")


def test_vecchia_predict_full_conditioning_equals_simple_kriging():
    # vecchia.rs:2131-2167: m >= n + targets gives global simple kriging
    c, v = O.test_field_2d(60, 5)
    mdl = VariogramModel(0.1, [Structure("exponential", 0.9, 30.0)])
    t = np.array([[12.0, 33.0], [55.0, 71.0], [80.0, 20.0], [40.0, 40.0]])
    gv, gvar = G.vecchia_predict(c, v, mdl, t, 1000)
    sk = O.krige(c, v, mdl, t, method="simple", mean=float(np.sum(v) / len(v)))
    assert np.max(np.abs(gv - sk["value"])) < 1e-8
    assert np.max(np.abs(gvar - sk["variance"])) < 1e-8


def test_vecchia_predict_deterministic_and_edge_cases():
    # vecchia.rs:2203-2240: bit-identical on repeat
    c, v = O.test_field_2d(150, 11)
    mdl = VariogramModel(0.05, [Structure("exponential", 0.95, 25.0)])
    t = np.array([[1.7 * i + 3.0, 96.0 - 1.6 * i] for i in range(60)])
    a = G.vecchia_predict(c, v, mdl, t, 8)
    b = G.vecchia_predict(c, v, mdl, t, 8)
    assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()
    r = O.vecchia_predict(c, v, mdl, t, 8)
    assert_close(a[0], r[0], float(np.mean(np.abs(v))), 1e-9, "value")
    assert_close(a[1], r[1], 1.0, 1e-9, "variance")
    # a target on a data point, and a single target
    t1 = np.array([c[17]])
    g1 = G.vecchia_predict(c, v, mdl, t1, 12)
    r1 = O.vecchia_predict(c, v, mdl, t1, 12)
    assert_close(g1[0], r1[0], 1.0, 1e-9, "value at a datum")
    assert_close(g1[1], r1[1], 1.0, 1e-9, "variance at a datum")
    # empty target set, and the reference's rejections
    e = G.vecchia_predict(c, v, mdl, np.zeros((0, 2)), 8)
    assert len(e[0]) == 0 and len(e[1]) == 0
    with pytest.raises(G.InvalidParameter):
        G.vecchia_predict(c, v, mdl, t, 0)
    with pytest.raises(G.InvalidParameter):
        G.vecchia_predict(c, v, VariogramModel(0.0, [Structure("power", 1.0, 1.0, param=1.0)]), t, 8)
    dup = np.vstack([c, c[:1]])
    with pytest.raises(G.DuplicatePoints):
        G.vecchia_predict(dup, np.append(v, 1.0), mdl, t, 8)


# ---------------------------------------------- gradient and BFGS fit (a19, a21) --
@pytest.mark.parametrize("kind", ["spherical", "exponential", "gaussian", "matern15", "matern25"])
def test_loglik_gradient_matches_oracle(kind):
    """loglik_grad_with_plan (vecchia.rs:416-530) for a batch of candidates."""
    c = uniform_points(6000, 2, 31, [1.0, 1.0])
    v = 0.5 + W.rff_field(c, matern25(), 1024, 7)
    plan = G.VecchiaPlan(G.PointSet(c, v), 20)
    order, nb, cnt = plan.arrays()
    cands = [VariogramModel(0.02, [Structure(kind, 1.0, 0.08)]),
             VariogramModel(0.2, [Structure(kind, 0.6, 0.03)]),
             VariogramModel(0.0004, [Structure(kind, 1.3, 0.15)])]
    for prec, tol in (("mixed", 1e-9), ("fp64", 1e-11)):
        ll, g, st = plan.loglik_grad(cands, prec)
        assert (st == 0).all()
        for i, mdl in enumerate(cands):
            s0 = mdl.structures[0]
            rl, rg = O.vecchia_loglik_grad(c, v, kind, mdl.nugget, s0.sill, s0.range, order, nb, cnt)
            assert_close([ll[i]], [rl], 1.0, tol, f"{prec} {kind} loglik {i}")
            # gradient components: relative to max(|component|, n * 1e-4)
            assert_close(g[i], rg, len(c) * 1e-4, tol, f"{prec} {kind} gradient {i}")


def test_gradient_rejects_models_without_closed_form():
    c = uniform_points(500, 2, 32, [1.0, 1.0])
    plan = G.VecchiaPlan(G.PointSet(c, c[:, 0] + c[:, 1]), 10)
    bad = [VariogramModel(0.1, [Structure("exponential", 0.5, 0.2), Structure("spherical", 0.4, 0.1)]),
           VariogramModel(0.1, [Structure.with_anisotropy("exponential", 0.5, 0.2, 30.0, 0.5)]),
           VariogramModel(0.1, [Structure("circular", 0.5, 0.2)])]
    ll, g, st = plan.loglik_grad(bad + [matern25()])
    assert (st[:3] == G.InvalidParameter.code).all() and st[3] == 0


def test_mle_bfgs_matches_oracle():
    """vecchia_mle (vecchia.rs:921-1081): the reference's three starts and
    analytical-gradient BFGS, with the starts advanced in lock-step."""
    for kind, n, m in (("exponential", 400, 12), ("matern25", 300, 10)):
        c, v = O.test_field_2d(n, 40 + n)
        model, ll, x, nev = G.vecchia_mle_fit(G.PointSet(c, v), kind, m)
        xr, fr, nr = O.vecchia_mle_bfgs(c, v, kind, m)
        assert abs(-ll - fr) <= 1e-7 * abs(fr), (kind, -ll, fr)
        assert abs(x[0] ** 2 - xr[0] ** 2) < 1e-3 * max(xr[0] ** 2, 1e-3), (kind, x, xr)
        assert np.max(np.abs(x[1:] - xr[1:])) < 1e-3, (kind, x, xr)
        assert nev < 1000  # BFGS: tens to hundreds of evaluations, not thousands
