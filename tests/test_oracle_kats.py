"""Pins the FP64 CPU oracle to the reference's own known answers.

Each test restates a test of geostat-rs (file:line given) against the oracle:
gstat golden values where the reference has them, otherwise the reference's
exactness / brute-force / closed-form identities.  These run on the CPU.
"""
import math

import numpy as np
import pytest

import pyoracle as O
from geostat_rs.model import Anisotropy, Structure, VariogramModel


def sph_model():
    # kriging.rs:852-854 `model()`
    return VariogramModel(0.05, [Structure("spherical", 0.95, 2.0)])


def sample_data():
    # kriging.rs:844-850 `sample_data()`
    c = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.4, 0.6]])
    v = np.array([1.0, 2.0, 1.5, 2.5, 1.7])
    return c, v


# ---------------------------------------------------------------- model.rs --
def test_rotation_3d_matches_gstat_setrot():
    # variogram/model.rs:906-952: gstat variogramLine with anis=c(30,20,40,.5,.3)
    m = VariogramModel(0.0, [Structure.with_rotation("spherical", 1.0, 100.0, 30.0, 20.0, 40.0,
                                                     0.5, 0.3)])
    cases = [
        ([1.0, 0.0, 0.0], 0.605458280770632),
        ([0.0, 1.0, 0.0], 0.577390658041395),
        ([0.0, 0.0, 1.0], 0.732990706603906),
        ([0.577350269190, 0.577350269190, 0.577350269190], 0.432164835884142),
        ([0.666666666667, -0.666666666667, 0.333333333333], 0.810043758779196),
        ([-0.534522483825, 0.267261241912, 0.801783725737], 0.575462768274161),
    ]
    for d, expected in cases:
        got = O.gamma_dh(m, [d[0] * 20.0, d[1] * 20.0, d[2] * 20.0])
        assert abs(got - expected) < 1e-9, (d, got, expected)


def test_gamma_boundary_and_closed_forms():
    # model.rs gamma_boundary_behavior + the closed forms of ModelKind::g
    m = VariogramModel(0.1, [Structure("spherical", 0.9, 100.0)])
    assert O.gamma_dh(m, [0.0, 0.0]) == 0.0
    assert O.gamma_dh(m, [1e-9, 0.0]) >= 0.1
    assert O.gamma_dh(m, [100.0, 0.0]) == pytest.approx(1.0, abs=1e-15)
    assert O.gamma_dh(m, [250.0, 0.0]) == pytest.approx(1.0, abs=1e-15)
    for kind, fn in [
        ("exponential", lambda d: 1 - math.exp(-d)),
        ("gaussian", lambda d: 1 - math.exp(-d * d)),
        ("matern15", lambda d: 1 - (1 + math.sqrt(3) * d) * math.exp(-math.sqrt(3) * d)),
        ("matern25", lambda d: 1 - (1 + math.sqrt(5) * d + 5 * d * d / 3) * math.exp(-math.sqrt(5) * d)),
    ]:
        mm = VariogramModel(0.0, [Structure(kind, 1.0, 10.0)])
        for h in (0.5, 3.0, 10.0, 40.0):
            assert O.gamma_dh(mm, [h, 0.0]) == pytest.approx(fn(h / 10.0), rel=1e-14, abs=1e-15)


def test_azimuth_mirror_symmetry_2d():
    # model.rs:870-903: azimuth 90 with ratio 0.5 equals the rotated frame
    m = VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 100.0, 90.0, 0.5)])
    # along azimuth 90 (x axis) the range is 100; along y it is 50
    assert O.gamma_dh(m, [100.0, 0.0]) == pytest.approx(1.0, abs=1e-12)
    assert O.gamma_dh(m, [0.0, 50.0]) == pytest.approx(1.0, abs=1e-12)
    assert O.gamma_dh(m, [0.0, 25.0]) == pytest.approx(O.gamma_dh(m, [50.0, 0.0]), abs=1e-12)


# --------------------------------------------------------------- linalg.rs --
def test_lu_known_system_and_singular():
    # linalg.rs:225-245
    a = np.array([[2.0, 1.0, -1.0], [-3.0, -1.0, 2.0], [-2.0, 1.0, 2.0]])
    x = O.lu_solve(a, [8.0, -11.0, -3.0])
    assert np.max(np.abs(x - [2.0, 3.0, -1.0])) < 1e-12
    with pytest.raises(O.OracleError) as e:
        O.lu_solve([[1.0, 2.0], [2.0, 4.0]], [1.0, 2.0])
    assert e.value.code == O.SINGULAR_SYSTEM


def test_cholesky_matches_lu_and_rejects_non_pd():
    # linalg.rs:248-268
    a = np.array([4.0, 1.0, 0.5, 1.0, 3.0, 0.2, 0.5, 0.2, 2.0]).reshape(3, 3)
    b = [1.0, 2.0, 3.0]
    assert np.max(np.abs(O.cholesky_solve(a, b) - O.lu_solve(a, b))) < 1e-12
    with pytest.raises(O.OracleError):
        O.cholesky_solve([[1.0, 2.0], [2.0, 4.0]], [1.0, 2.0])


def test_indefinite_kriging_like_system():
    # linalg.rs:270-283
    a = np.array([[1.0, 0.3, 1.0], [0.3, 1.0, 1.0], [1.0, 1.0, 0.0]])
    b = np.array([0.7, 0.5, 1.0])
    x = O.lu_solve(a, b)
    assert np.max(np.abs(a @ x - b)) < 1e-12
    assert abs(x[0] + x[1] - 1.0) < 1e-12


# --------------------------------------------------------------- search.rs --
def _random_points(n, seed):
    u = O.rng_uniform(seed, 2 * n)
    return (u * 100.0).reshape(n, 2)


def test_kdtree_matches_brute_force():
    # search.rs:364-377
    pts = _random_points(500, 5)
    u = O.rng_uniform(6, 400)
    for t in range(200):
        target = [u[2 * t] * 120.0 - 10.0, u[2 * t + 1] * 120.0 - 10.0]
        for k, r in [(1, None), (8, None), (16, 15.0), (1000, 5.0)]:
            assert O.kdtree_knn(pts, target, k, r) == O.knn_brute(pts, target, k, r)


def test_bucket_grid_matches_brute_force_incrementally():
    # search.rs:379-396
    pts = _random_points(400, 9)
    u = O.rng_uniform(10, 400)
    after = [i for i in range(400) if i % 37 == 0]
    targets = np.array([[u[2 * q] * 100.0, u[2 * q + 1] * 100.0] for q in range(len(after))])
    for k, r in [(4, None), (16, 20.0)]:
        res, _ = O.bucketgrid_queries(pts, [0, 0], [100, 100], 400, after, targets, k, r)
        for q, i in enumerate(after):
            assert res[q] == O.knn_brute(pts[:i + 1], targets[q], k, r)


def test_bucket_grid_degenerate_axes():
    # search.rs:410-445
    pts = np.array([[i * 10.0, 5.0] for i in range(50)])
    res, dims = O.bucketgrid_queries(pts, [0, 5], [500, 5], 50, [49], [[123.0, 5.0]], 5)
    assert dims == [50, 1]
    assert res[0] == O.knn_brute(pts, [123.0, 5.0], 5)
    _, dims3 = O.bucketgrid_queries(np.zeros((1, 3)), [0, 0, 5], [500, 500, 5], 100, [], [], 1)
    assert dims3[2] == 1 and dims3[0] * dims3[1] * dims3[2] <= 400
    _, dims1 = O.bucketgrid_queries(np.zeros((1, 2)), [3, 3], [3, 3], 10, [], [], 1)
    assert dims1 == [1, 1]


def test_empty_and_single_point_search():
    # search.rs:398-407
    assert O.kdtree_knn(np.array([[1.0, 1.0]]), [0.0, 0.0], 5) == [0]
    assert O.kdtree_knn(np.array([[1.0, 1.0]]), [0.0, 0.0], 5, 0.5) == []


# ----------------------------------------------------------------- data.rs --
def test_duplicate_pair_detection():
    # data.rs:201-213
    assert O.duplicate_pair(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])) is None
    assert O.duplicate_pair(np.array([[0, 0], [1, 2], [1, 2], [3, 3]], float)) == (1, 2)
    assert O.duplicate_pair(np.array([[0.0, 1.0], [-0.0, 1.0]])) == (0, 1)


def test_grid_centers_order():
    # grid.rs:99-109
    c = O.grid_centers([0, 0], [4, 2], [4, 2])
    assert c.shape == (8, 2)
    assert c[0].tolist() == [0.5, 0.5] and c[1].tolist() == [1.5, 0.5]
    assert c[4].tolist() == [0.5, 1.5] and c[7].tolist() == [3.5, 1.5]


# ------------------------------------------------------------------ rng.rs --
def _py_xoshiro(seed, count):
    M = (1 << 64) - 1

    def sm(st):
        st = (st + 0x9E3779B97F4A7C15) & M
        z = st
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
        return st, z ^ (z >> 31)

    st, s = seed, []
    for _ in range(4):
        st, v = sm(st)
        s.append(v)
    rotl = lambda x, k: ((x << k) | (x >> (64 - k))) & M
    out = []
    for _ in range(count):
        out.append((rotl((s[0] + s[3]) & M, 23) + s[0]) & M)
        t = (s[1] << 17) & M
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t
        s[3] = rotl(s[3], 45)
    return out


def test_rng_stream_matches_published_algorithm():
    # rng.rs:7-48; splitmix64(0) first output is the published 0xE220A8397B1DCDAF
    assert _py_xoshiro(0, 1)  # exercise
    st = 0
    st = (st + 0x9E3779B97F4A7C15) & ((1 << 64) - 1)
    assert O.rng_u64(42, 100).tolist() == _py_xoshiro(42, 100)
    assert O.rng_u64(0, 5).tolist() == _py_xoshiro(0, 5)
    u = O.rng_uniform(1, 10000)
    assert (u >= 0).all() and (u < 1).all()
    z = O.rng_normal(7, 100000)
    assert abs(z.mean()) < 0.02 and abs(z.var() - 1) < 0.05


# -------------------------------------------------------------- kriging.rs --
def test_ordinary_kriging_exact_at_data():
    # kriging.rs:1205-1220
    c, v = sample_data()
    r = O.krige(c, v, sph_model(), c)
    assert np.max(np.abs(r["value"] - v)) < 1e-8
    assert np.max(r["variance"]) < 1e-8


def test_power_model_matches_gstat_ordinary_kriging():
    # kriging.rs:1222-1268 (gstat krige with vgm(2.0,"Pow",1.2))
    c = np.array([[0, 0], [10, 0], [0, 10], [10, 10], [5, 5]], float)
    v = np.array([1.0, 2.0, 1.5, 2.5, 1.8])
    m = VariogramModel(0.0, [Structure("power", 2.0, 1.0, param=1.2)])
    r = O.krige(c, v, m, np.array([[3.0, 4.0], [7.0, 8.0], [5.0, 5.0]]))
    assert abs(r["value"][0] - 1.5252052569) < 1e-6
    assert abs(r["variance"][0] - 6.4437897810) < 1e-5
    assert abs(r["value"][1] - 2.1366210000) < 1e-6
    assert abs(r["variance"][1] - 7.7780140000) < 1e-5
    assert abs(r["value"][2] - 1.8) < 1e-6 and r["variance"][2] < 1e-6


def test_far_field_simple_and_ordinary():
    # kriging.rs:1360-1383
    c, v = sample_data()
    m = sph_model()
    ok = O.krige(c, v, m, np.array([[1e6, 1e6]]))
    assert ok["variance"][0] >= 0.99 * m.total_sill() and np.isfinite(ok["value"][0])
    sk = O.krige(c, v, m, np.array([[1e6, 1e6]]), method="simple", mean=1.74)
    assert abs(sk["value"][0] - 1.74) < 1e-9
    assert abs(sk["variance"][0] - m.total_sill()) < 1e-9
    assert np.isnan(sk["lagrange"][0]) and np.isfinite(ok["lagrange"][0])


def test_universal_kriging_reproduces_exact_drift():
    # kriging.rs:1385-1413
    c = np.array([[i, j] for i in range(4) for j in range(4)], float)
    v = 2.0 + 3.0 * c[:, 0] - c[:, 1]
    t = np.array([[1.5, 1.5], [5.0, 2.0]])
    r = O.krige(c, v, sph_model(), t, method="universal", degree=1)
    assert np.max(np.abs(r["value"] - (2 + 3 * t[:, 0] - t[:, 1]))) < 1e-7


def test_external_drift_reproduces_linear_relation():
    # kriging.rs:1415-1445
    xs = [(i * 10.0, j * 10.0) for i in range(5) for j in range(5)]
    c = np.array(xs)
    d = np.sin(c[:, 0] * 0.13 + c[:, 1] * 0.07)
    v = 2.0 + 3.0 * d
    t = np.array([[12.0, 33.0], [45.0, 5.0]])
    td = np.array([[0.4], [-0.7]])
    r = O.krige(c, v, sph_model(), t, method="external_drift", drift=d.reshape(-1, 1),
                target_drift=td)
    assert np.max(np.abs(r["value"] - (2 + 3 * td[:, 0]))) < 1e-7


def test_octant_search_balances_clustered_neighbors():
    # kriging.rs:960-1011
    c = np.array([[1.0, 0.1], [1.1, -0.1], [1.2, 0.2], [1.3, -0.2], [1.4, 0.05],
                  [-2.0, 0.5], [-2.0, -0.5], [0.5, -2.0], [0.5, 2.0]])
    v = np.array([10.0] * 5 + [0.0] * 4)
    t = np.array([[0.0, 0.0]])
    near = O.krige(c, v, sph_model(), t, max_neighbors=4)["value"][0]
    octn = O.krige(c, v, sph_model(), t, max_neighbors=4, max_per_octant=1)["value"][0]
    assert near > 9.0 and octn < near - 2.0


def test_min_neighbors_and_invalid_configs():
    # kriging.rs:913-958
    c, v = sample_data()
    r = O.krige(c, v, sph_model(), np.array([[0.5, 0.5], [1.5, 1.5]]), radius=0.75,
                min_neighbors=3)
    assert r["status"][0] == 0 and r["status"][1] == O.NO_NEIGHBORS
    assert np.isnan(r["value"][1])
    with pytest.raises(O.OracleError):
        O.krige(c, v, sph_model(), c, min_neighbors=0)
    with pytest.raises(O.OracleError):
        O.krige(c, v, sph_model(), c, max_neighbors=2, min_neighbors=3)


def test_duplicate_points_rejected_up_front():
    # kriging.rs:1191-1203
    c = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    with pytest.raises(O.OracleError) as e:
        O.krige(c, np.array([1.0, 2.0, 2.1, 1.5]), sph_model(), c)
    assert e.value.code == O.DUPLICATE_POINTS and "1 and 2" in str(e.value)


def test_kdtree_neighborhood_matches_global_at_full_k():
    # kriging.rs:1570-1592
    c, v = sample_data()
    t = np.array([[0.3, 0.3], [0.9, 0.1], [2.0, 2.0]])
    g = O.krige(c, v, sph_model(), t)
    loc = O.krige(c, v, sph_model(), t, max_neighbors=len(c))
    assert np.max(np.abs(g["value"] - loc["value"])) < 1e-12
    assert np.max(np.abs(g["variance"] - loc["variance"])) < 1e-12


def test_measurement_error_smooths():
    # kriging.rs:856-911
    c, v = sample_data()
    ex = O.krige(c, v, sph_model(), c)
    nz = O.krige(c, v, sph_model(), c, measurement_error=np.full(5, 0.5))
    assert np.max(np.abs(ex["value"] - v)) < 1e-8
    assert np.min(np.abs(nz["value"] - v)) > 1e-3 and np.min(nz["variance"]) > 1e-3
    z = O.krige(c, v, sph_model(), np.array([[0.3, 0.7]]), measurement_error=np.zeros(5))
    e2 = O.krige(c, v, sph_model(), np.array([[0.3, 0.7]]))
    assert abs(z["value"][0] - e2["value"][0]) < 1e-14


def test_anisotropic_search_prefers_major_axis():
    # kriging.rs:1013-1066 (shape of the test: the ellipse admits the far
    # major-axis point over a nearer minor-axis one)
    c = np.array([[3.0, 0.0], [0.0, 2.0], [10.0, 10.0], [-10.0, 10.0]])
    v = np.array([5.0, -5.0, 0.0, 0.0])
    t = np.array([[0.0, 0.0]])
    eu = O.krige(c, v, sph_model(), t, max_neighbors=1, kcap=1)
    an = O.krige(c, v, sph_model(), t, max_neighbors=1, kcap=1,
                 anisotropic_search=Anisotropy(90.0, 0.25))
    assert eu["neighbors"][0, 0] == 1 and an["neighbors"][0, 0] == 0


def test_kriging_3d_exact_and_far_field():
    # tests/three_d.rs:48-76
    c, v = O.test_field_3d(150, 5)
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 40.0)])
    idx = list(range(0, 150, 30))
    r = O.krige(c, v, m, c[idx])
    assert np.max(np.abs(r["value"] - v[idx])) < 1e-7 and np.max(r["variance"]) < 1e-7
    far = O.krige(c, v, m, np.array([[1e5, 1e5, 1e5]]))
    assert far["variance"][0] >= 0.99 * m.total_sill()


# -------------------------------------------------------------- vecchia.rs --
def exp_model(nug, sill, rng_):
    return VariogramModel(nug, [Structure("exponential", sill, rng_)])


def test_vecchia_full_conditioning_equals_exact():
    # vecchia.rs:1998-2010
    c, v = O.test_field_2d(14, 3)
    m = exp_model(0.05, 1.0, 40.0)
    assert abs(O.vecchia_loglik(c, v, m, 13) - O.exact_loglik(c, v, m)) < 1e-9


def test_vecchia_approximation_is_close_with_maxmin():
    # vecchia.rs:2012-2026
    c, v = O.test_field_2d(90, 11)
    m = exp_model(0.05, 1.0, 30.0)
    ex = O.exact_loglik(c, v, m)
    assert abs(O.vecchia_loglik(c, v, m, 12) - ex) / abs(ex) < 0.02


def test_vecchia_predict_full_conditioning_equals_simple_kriging():
    # vecchia.rs:2131-2167
    c, v = O.test_field_2d(60, 5)
    m = exp_model(0.1, 0.9, 30.0)
    t = np.array([[12.0, 33.0], [55.0, 71.0], [80.0, 20.0], [40.0, 40.0]])
    pv, pvar = O.vecchia_predict(c, v, m, t, 1000)
    sk = O.krige(c, v, m, t, method="simple", mean=float(np.sum(v) / len(v)))
    assert np.max(np.abs(pv - sk["value"])) < 1e-8
    assert np.max(np.abs(pvar - sk["variance"])) < 1e-8


def test_vecchia_predict_small_m_tracks_and_is_deterministic():
    # vecchia.rs:2169-2240
    c, v = O.test_field_2d(150, 9)
    m = exp_model(0.05, 0.95, 25.0)
    t = np.array([[2.5 * i + 1.0, 97.0 - 2.3 * i] for i in range(40)])
    pv, pvar = O.vecchia_predict(c, v, m, t, 25)
    sk = O.krige(c, v, m, t, method="simple", mean=float(np.mean(v)))
    assert np.max(np.abs(pv - sk["value"])) < 0.02
    assert np.max(np.abs(pvar - sk["variance"])) < 0.02
    c2, v2 = O.test_field_2d(150, 11)
    t2 = np.array([[1.7 * i + 3.0, 96.0 - 1.6 * i] for i in range(60)])
    a = O.vecchia_predict(c2, v2, m, t2, 8)
    b = O.vecchia_predict(c2, v2, m, t2, 8)
    assert a[0].tobytes() == b[0].tobytes() and a[1].tobytes() == b[1].tobytes()


def test_lazy_maxmin_matches_exact_traversal():
    # vecchia.rs:2276-2289
    for seed in (3, 11, 29):
        c, _ = O.test_field_2d(400, seed)
        assert O.maxmin_order(c).tolist() == O.maxmin_order_brute(c).tolist()
    c, _ = O.test_field_2d(50, 7)
    assert sorted(O.maxmin_order(c).tolist()) == list(range(50))


def test_incremental_predecessors_match_brute_force():
    # vecchia.rs:2290-2310
    c, _ = O.test_field_2d(300, 13)
    m = 8
    order, nb, cnt = O.vecchia_plan(c, m)
    for k in range(len(c)):
        t = order[k]
        prev = sorted(((float(np.sum((c[t] - c[j]) ** 2)), j) for j in order[:k]))[:m]
        assert sorted(j for _, j in prev) == sorted(nb[k, :cnt[k]].tolist())


def test_vecchia_rejects_bad_args():
    # vecchia.rs:2312-2319
    c, v = O.test_field_2d(10, 1)
    m = VariogramModel(0.1, [Structure("spherical", 1.0, 20.0)])
    with pytest.raises(O.OracleError):
        O.vecchia_loglik(c, v, m, 0)
    with pytest.raises(O.OracleError):
        O.vecchia_loglik(c, v, VariogramModel(0.0, [Structure("power", 1.0, 1.0, param=1.0)]), 5)


# ---------------------------------------------------------------- optim.rs --
def test_nelder_mead_rosenbrock_and_multistart():
    # optim.rs:294-324
    rosen = lambda x: (1 - x[0]) ** 2 + 100 * (x[1] - x[0] ** 2) ** 2
    x, fx = O.nelder_mead_multistart(rosen, [[-1.2, 1.0]], 0.1, 5000)
    assert abs(x[0] - 1) < 1e-3 and abs(x[1] - 1) < 1e-3 and fx < 1e-6
    wells = lambda x: -2 * math.exp(-0.5 * (x[0] + 3) ** 2) - 3 * math.exp(-0.5 * (x[0] - 3) ** 2)
    _, single = O.nelder_mead_multistart(wells, [[-3.0]], 0.1, 500)
    assert single > -2.5
    x, fx = O.nelder_mead_multistart(wells, [[-3.0], [3.0], [0.0]], 0.1, 500)
    assert abs(x[0] - 3.0) < 1e-2 and fx < -2.9


# ------------------------------------------------ gradient / BFGS (a19, a21) --
def test_g_and_dg_matches_finite_differences():
    # vecchia.rs:2846-2875
    h = 1e-6
    unit = lambda kind: VariogramModel(0.0, [Structure(kind, 1.0, 1.0)])
    for kind in ("spherical", "exponential", "gaussian", "matern15", "matern25"):
        for d in (0.1, 0.3, 0.7, 1.5, 2.5):
            g, dg = O.g_and_dg(kind, d)
            gam = lambda x: O.gamma_dh(unit(kind), [x, 0.0])
            assert abs(g - gam(d)) < 1e-12, (kind, d)
            fd = (gam(d + h) - gam(d - h)) / (2 * h)
            assert abs(dg - fd) < 1e-5, (kind, d, dg, fd)
    for kind in ("circular", "hole", "wave"):
        assert O.g_and_dg(kind, 0.5) is None


def test_loglik_gradient_matches_finite_differences():
    # vecchia.rs:2878-2935
    c, v = O.test_field_2d(60, 11)
    order, nb, cnt = O.vecchia_plan(c, 8)
    for kind in ("spherical", "exponential", "gaussian", "matern15", "matern25"):
        nug, ps, rg = 0.05, 0.9, 22.0
        ll, g = O.vecchia_loglik_grad(c, v, kind, nug, ps, rg, order, nb, cnt)
        at = lambda a, b, r: O.vecchia_loglik_plan(
            c, v, VariogramModel(a, [Structure(kind, b, r)]), order, nb, cnt)
        assert abs(ll - at(nug, ps, rg)) < 1e-9, kind
        fd = [(at(nug * (1 + 1e-4), ps, rg) - at(nug * (1 - 1e-4), ps, rg)) / (2e-4 * nug),
              (at(nug, ps * (1 + 1e-4), rg) - at(nug, ps * (1 - 1e-4), rg)) / (2e-4 * ps),
              (at(nug, ps, rg * (1 + 1e-4)) - at(nug, ps, rg * (1 - 1e-4))) / (2e-4 * rg)]
        for q in range(3):
            assert abs(g[q] - fd[q]) < 1e-2 * max(abs(fd[q]), 1.0), (kind, q, g[q], fd[q])


def test_gradient_is_zero_for_a_clamped_variance():
    # vecchia.rs:2937-2990
    c = np.array([[0.0, 0.0], [1e-13, 0.0]])
    v = np.array([0.3, -0.7])
    ll, g = O.vecchia_loglik_grad(c, v, "spherical", 0.0, 1.0, 10.0, [0, 1],
                                  np.array([[-1], [0]]), np.array([0, 1]))
    z0 = 0.5
    assert abs(g[1] - (-0.5 / 1.0 + 0.5 * z0 * z0 / 1.0)) < 1e-9


def test_bfgs_reference_known_answers():
    # optim.rs tests: Rosenbrock, two-well multistart, quadratic
    f = lambda x: (1 - x[0]) ** 2 + 100 * (x[1] - x[0] ** 2) ** 2
    gr = lambda x: [-2 * (1 - x[0]) - 400 * x[0] * (x[1] - x[0] ** 2), 200 * (x[1] - x[0] ** 2)]
    x, fx = O.bfgs_multistart(f, gr, [[-1.2, 1.0]], 200)
    assert abs(x[0] - 1) < 1e-4 and abs(x[1] - 1) < 1e-4 and fx < 1e-8
    w = lambda x: -2 * np.exp(-0.5 * (x[0] + 3) ** 2) - 3 * np.exp(-0.5 * (x[0] - 3) ** 2)
    wg = lambda x: [2 * (x[0] + 3) * np.exp(-0.5 * (x[0] + 3) ** 2)
                    + 3 * (x[0] - 3) * np.exp(-0.5 * (x[0] - 3) ** 2)]
    _, single = O.bfgs_multistart(w, wg, [[-3.0]], 100)
    assert single > -2.5
    x, fx = O.bfgs_multistart(w, wg, [[-3.0], [3.0], [0.0]], 100)
    assert abs(x[0] - 3) < 1e-3 and fx < -2.9
    ctr = np.array([2.0, -1.0, 0.5])
    x, fx = O.bfgs_multistart(lambda x: float(np.sum((x - ctr) ** 2)),
                              lambda x: list(2 * (x - ctr)), [[0.0, 0.0, 0.0]], 100)
    assert np.max(np.abs(x - ctr)) < 1e-6 and fx < 1e-10
    # never worse than the best point visited (wrong-signed gradient)
    x, fx = O.bfgs_multistart(lambda x: x[0] ** 2, lambda x: [-2 * x[0]], [[1.0]], 50)
    assert fx <= 1.0 + 1e-13


def test_vecchia_mle_bfgs_path_improves_on_the_starts():
    c, v = O.test_field_2d(300, 21)
    x, f, ne = O.vecchia_mle_bfgs(c, v, "exponential", 10)
    starts, rmax = O.vecchia_mle_setup(c, v)
    o, nb, cnt = O.vecchia_plan(c, 10)
    f0 = O.vecchia_mle_objective(c, v, "exponential", 10, o, nb, cnt, rmax, starts)
    assert f < np.min(f0) and np.isfinite(f) and ne > 3


# ----------------------------------------- grouped Vecchia (Guinness 2018) --
def _exp_model(nug, rng_):
    return VariogramModel(nug, [Structure("exponential", 1.0, rng_)])


def test_grouped_matches_ungrouped_at_group_size_one():
    # vecchia.rs:2050-2063
    c, v = O.test_field_2d(90, 11)
    m = _exp_model(0.05, 30.0)
    order = O.maxmin_order(c)
    o, nb, cnt = O.vecchia_plan(c, 12, order)
    ungrouped = O.vecchia_loglik_plan(c, v, m, o, nb, cnt)
    assert abs(O.vecchia_loglik_grouped(c, v, m, o, nb, cnt, 1) - ungrouped) < 1e-12


def test_grouped_full_conditioning_equals_exact():
    # vecchia.rs:2066-2085
    c, v = O.test_field_2d(20, 4)
    m = _exp_model(0.05, 40.0)
    exact = O.exact_loglik(c, v, m)
    o, nb, cnt = O.vecchia_plan(c, len(c) - 1, O.maxmin_order(c))
    for g in (2, 3, 5, 8):
        assert abs(O.vecchia_loglik_grouped(c, v, m, o, nb, cnt, g) - exact) < 1e-8


def test_grouped_at_least_as_close_as_ungrouped():
    # vecchia.rs:2088-2107
    c, v = O.test_field_2d(90, 11)
    m = _exp_model(0.05, 30.0)
    exact = O.exact_loglik(c, v, m)
    o, nb, cnt = O.vecchia_plan(c, 12, O.maxmin_order(c))
    err0 = abs(O.vecchia_loglik_plan(c, v, m, o, nb, cnt) - exact)
    for g in (2, 4, 6):
        assert abs(O.vecchia_loglik_grouped(c, v, m, o, nb, cnt, g) - exact) <= err0 + 1e-9


# ------------------------------------------------------- Vecchia REML --------
def _cov_matrix(c, m):
    sill = m.nugget + sum(s.sill for s in m.structures)
    n = len(c)
    out = np.empty((n, n))
    for a in range(n):
        for b in range(n):
            out[a, b] = sill if a == b else sill - O.gamma_dh(m, c[a] - c[b])
    return out


def _exact_reml(c, v, m, f):
    # vecchia.rs:2431-2463 exact_reml: the full restricted likelihood
    n, p = f.shape
    s = _cov_matrix(c, m)
    siz = np.linalg.solve(s, v)
    sif = np.linalg.solve(s, f)
    amat = f.T @ sif
    cvec = f.T @ siz
    beta = np.linalg.solve(amat, cvec)
    resid = v @ siz - cvec @ beta
    return -0.5 * ((n - p) * math.log(2 * math.pi) + np.linalg.slogdet(s)[1]
                   + np.linalg.slogdet(amat)[1] + resid)


def test_poly_and_drift_bases():
    # vecchia.rs:1181-1272: p = C(degree + dim, dim); centred, unit-variance columns
    c, _ = O.test_field_3d(40, 3)
    for deg, p in ((0, 1), (1, 4), (2, 10)):
        f = O.poly_basis(c, deg)
        assert f.shape == (40, p)
        np.testing.assert_array_equal(f[:, 0], 1.0)
    f = O.poly_basis(c[:, :2], 1)
    # exponent order (0,0), (0,1), (1,0): the last dimension varies fastest
    np.testing.assert_allclose(f[:, 1], (c[:, 1] - c[:, 1].mean()) / c[:, 1].std(), atol=1e-12)
    np.testing.assert_allclose(f[:, 2], (c[:, 0] - c[:, 0].mean()) / c[:, 0].std(), atol=1e-12)
    d = O.drift_basis(np.stack([c[:, 0] * 1e4 + 6e5, c[:, 2]], 1))
    np.testing.assert_array_equal(d[:, 0], 1.0)
    np.testing.assert_allclose(d[:, 1:].mean(0), 0.0, atol=1e-12)
    np.testing.assert_allclose(d[:, 1:].std(0), 1.0, atol=1e-12)


def test_reml_full_conditioning_equals_exact():
    # vecchia.rs:2466-2481 (ungrouped), and every group size on the same plan
    c, v = O.test_field_2d(16, 4)
    m = _exp_model(0.05, 35.0)
    f = O.poly_basis(c, 1)
    exact = _exact_reml(c, v, m, f)
    o, nb, cnt = O.vecchia_plan(c, len(c) - 1)
    for g in (1, 2, 3, 5, 16):
        assert abs(O.vecchia_reml_loglik(c, v, m, o, nb, cnt, f, g) - exact) < 1e-7
    fq = O.poly_basis(c, 2)
    assert abs(O.vecchia_reml_loglik(c, v, m, o, nb, cnt, fq, 4) - _exact_reml(c, v, m, fq)) < 1e-7


def _gp_field(seed, n, truth):
    # the reference tests' draw: 2n uniforms (x, y in [0, 60)), then n normals
    # from one stream; values = L eps with L the Cholesky factor of Sigma
    u, eps = O.rng_draw(seed, 2 * n, n)
    c = u.reshape(n, 2) * 60.0
    l = np.linalg.cholesky(_cov_matrix(c, truth))
    return c, l @ eps


def _reml_fit(c, v, kind, m, f, g=1):
    starts, _ = O.vecchia_mle_setup(c, v)
    x, fx, _ = O.vecchia_fit_nm(c, v, kind, m, starts, basis=f, group_size=g)
    return math.exp(x[2]), -fx


def test_reml_tames_the_range_under_a_trend():
    # vecchia.rs:2504-2545
    c, gp = _gp_field(20, 90, _exp_model(0.05, 10.0))
    v = 0.3 * c[:, 0] - 0.2 * c[:, 1] + gp
    x, _, _ = O.vecchia_mle_bfgs(c, v, "exponential", 8)
    ml_r = math.exp(x[2])
    reml_r, _ = _reml_fit(c, v, "exponential", 8, O.poly_basis(c, 1))
    assert reml_r < ml_r and reml_r < 40.0


@pytest.mark.parametrize("utm", [False, True])
def test_reml_drift_recovers_range_with_a_covariate(utm):
    # vecchia.rs:2548-2588 and 2590-2638 (UTM-scale covariate)
    c, gp = _gp_field(21, 90, _exp_model(0.05, 10.0))
    cov = np.exp(-((c[:, 0] - 30.0) ** 2 + (c[:, 1] - 30.0) ** 2) / 200.0)
    v = 8.0 * cov + gp
    drift = 600_000.0 + 1e4 * cov if utm else cov
    r, _ = _reml_fit(c, v, "exponential", 8, O.drift_basis(drift.reshape(-1, 1)))
    assert r < 40.0


def test_vecchia_mle_grouped_matches_ungrouped_under_full_conditioning():
    # vecchia.rs:2110-2128
    c, v = O.test_field_2d(16, 21)
    m = len(c) - 1
    xu, fu, _ = O.vecchia_mle_bfgs(c, v, "exponential", m)
    starts, _ = O.vecchia_mle_setup(c, v)
    xg, fg, _ = O.vecchia_fit_nm(c, v, "exponential", m, starts, group_size=4)
    assert abs(fu - fg) < 1e-6
    assert abs(xu[0] ** 2 - xg[0] ** 2) < 1e-4
    assert abs(math.exp(xu[1]) - math.exp(xg[1])) < 1e-3
    assert abs(math.exp(xu[2]) - math.exp(xg[2])) < 1e-2


# ------------------------------------------------------- block kriging -------
def _block_offsets(size, n):
    # kriging.rs:815-838 block_offsets
    return np.array([[((ix + 0.5) / n[0] - 0.5) * size[0], ((iy + 0.5) / n[1] - 0.5) * size[1]]
                     for iy in range(n[1]) for ix in range(n[0])])


def test_block_kriging_averages_point_predictions():
    # kriging.rs:1525-1567: with a global neighbourhood the block BLUP is the
    # mean of the point BLUPs, and the block variance is below the point's
    c, v = sample_data()
    m = sph_model()
    ctr = np.array([[0.6, 0.4]])
    off = _block_offsets([0.4, 0.4], [4, 4])
    blk = O.krige_block(c, v, m, ctr, off)
    assert blk["status"][0] == 0
    pts = O.krige(c, v, m, ctr + off)
    assert abs(blk["value"][0] - pts["value"].mean()) < 1e-10
    assert blk["variance"][0] < O.krige(c, v, m, ctr)["variance"][0]
    with pytest.raises(O.OracleError):
        O.krige_block(c, v, m, ctr, off, method="universal")


def test_power_model_rejects_block_kriging():
    # kriging.rs:1314-1322
    c, v = sample_data()
    m = VariogramModel(0.0, [Structure("power", 1.0, 1.0, param=1.0)])
    with pytest.raises(O.OracleError):
        O.krige_block(c, v, m, [[0.5, 0.5]], [[0.0, 0.0], [0.1, 0.0], [0.0, 0.1], [0.1, 0.1]])


def _smooth_field(n, seed, period=20.0):
    # validation.rs:991-1002 smooth_field
    u, _ = O.rng_draw(seed, 2 * n, 0)
    c = u.reshape(n, 2) * 100.0
    return c, np.sin(c[:, 0] / period) + np.cos(c[:, 1] / period)


def _oracle_fold_cv(c, v, m, fold_of):
    # cv_with_folds (validation.rs:219-265): a predictor per fold on the rest
    pred, var = np.empty(len(c)), np.empty(len(c))
    for f in np.unique(fold_of):
        tr, te = fold_of != f, fold_of == f
        r = O.krige(c[tr], v[tr], m, c[te])
        assert (r["status"] == 0).all()
        pred[te], var[te] = r["value"], r["variance"]
    return pred, var


def test_spatial_block_assignment():
    # validation.rs:298-328: dimension 0 fastest, the maxima in the last block
    c = np.array([[0.0, 0.0], [10.0, 0.0], [0.0, 10.0], [10.0, 10.0], [4.9, 5.1], [2.6, 7.4]])
    f = O.spatial_block_assignment(c, [2, 2])
    assert list(f) == [0, 1, 2, 3, 2, 2]
    f = O.spatial_block_assignment(c, [4, 1])
    assert list(f) == [0, 3, 0, 3, 1, 1]


def test_block_cv_covers_every_point_and_has_skill():
    # validation.rs:1052-1067
    from geostat_rs.api import CvResult
    c, v = _smooth_field(120, 7)
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 50.0)])
    pred, var = _oracle_fold_cv(c, v, m, O.spatial_block_assignment(c, [4, 4]))
    assert np.isfinite(pred).all() and (np.isfinite(var) & (var >= 0)).all()
    assert CvResult(v, pred, var).vecv() > 0.0


def test_block_cv_is_harsher_than_random_k_fold():
    # validation.rs:1070-1097
    from geostat_rs.api import CvResult
    c, v = _smooth_field(150, 3, period=200.0)
    v = np.sin(c[:, 0] / 200.0) + np.cos(c[:, 1] / 200.0)
    m = VariogramModel(0.0, [Structure("spherical", 1.0, 300.0)])
    order = np.arange(150)
    u = O.rng_u64(1, 150)
    for idx, i in enumerate(range(149, 0, -1)):
        j = int(u[idx] % np.uint64(i + 1))
        order[i], order[j] = order[j], order[i]
    kf = np.empty(150, dtype=int)
    kf[order] = np.arange(150) % 10
    rnd = CvResult(v, *_oracle_fold_cv(c, v, m, kf))
    blk = CvResult(v, *_oracle_fold_cv(c, v, m, O.spatial_block_assignment(c, [5, 5])))
    assert blk.rmse() >= rnd.rmse()


# ------------------------------------------------ Vecchia parameter SEs ------
def _gp_draw(seed, n, truth):
    u, eps = O.rng_draw(seed, 2 * n, n)
    c = u.reshape(n, 2) * 60.0
    return c, np.linalg.cholesky(_cov_matrix(c, truth)) @ eps


def test_param_se_are_finite_and_informative():
    # vecchia.rs:2651-2683
    c, v = _gp_draw(31, 140, _exp_model(0.2, 12.0))
    x, _, _ = O.vecchia_mle_bfgs(c, v, "exponential", 12)
    rng_ = math.exp(x[2])
    se = O.vecchia_param_se(c, v, "exponential", x[0] ** 2, math.exp(x[1]), rng_, 12)
    assert np.isfinite(se[1]) and se[1] > 0
    assert np.isfinite(se[2]) and 0 < se[2] < rng_


def test_param_se_at_the_zero_nugget_boundary():
    # vecchia.rs:2686-2725
    c, v = _gp_draw(51, 140, _exp_model(0.0, 12.0))
    se = O.vecchia_param_se(c, v, "exponential", 0.0, 1.0, 12.0, 12)
    assert np.isnan(se[0])
    assert np.isfinite(se[1]) and se[1] > 0 and np.isfinite(se[2]) and se[2] > 0


# ------------------------------------------- anisotropic search and limits ---
def test_anisotropic_search_radius_is_the_major_axis_radius():
    # kriging.rs:1068-1100: the radius is the ellipse's major-axis radius
    c = np.array([[0.0, 5.0], [5.0, 0.0]])
    v = np.array([100.0, 999.0])
    r = O.krige(c, v, sph_model(), np.array([[0.0, 0.0]]), radius=5.0,
                anisotropic_search=Anisotropy(0.0, 0.5))
    assert r["status"][0] == 0 and abs(r["value"][0] - 100.0) < 1e-6


def test_anisotropic_search_octants_follow_the_rotated_frame():
    # kriging.rs:1102-1150
    c = [[0.1, 1.0], [-0.1, 1.1], [0.2, 1.2], [-0.2, 1.3], [0.05, 1.4],
         [0.5, -2.0], [-0.5, -2.0], [-2.0, 0.5], [2.0, 0.5]]
    v = [10.0] * 5 + [0.0] * 4
    t = np.array([[0.0, 0.0]])
    nearest = O.krige(c, v, sph_model(), t, max_neighbors=4)["value"][0]
    octant = O.krige(c, v, sph_model(), t, max_neighbors=4, max_per_octant=1,
                     anisotropic_search=Anisotropy(90.0, 1.0))["value"][0]
    assert nearest > 9.0 and octant < nearest - 2.0


def test_anisotropic_search_works_in_3d_with_dip():
    # kriging.rs:1152-1178: azimuth 0, dip 90 points the major axis along +z
    c = np.array([[0.0, 0.0, 4.0], [4.0, 0.0, 0.0]])
    v = np.array([100.0, 0.0])
    r = O.krige(c, v, sph_model(), np.array([[0.0, 0.0, 0.0]]), max_neighbors=1,
                anisotropic_search=Anisotropy(0.0, 0.2, 1.0, 90.0, 0.0))
    assert abs(r["value"][0] - 100.0) < 1e-6


def test_anisotropic_model_weights_by_direction():
    # kriging.rs:1380-1402
    c = np.array([[0.0, 30.0], [30.0, 0.0], [-25.0, -25.0]])
    v = np.array([10.0, 0.0, 5.0])
    m = VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 100.0, 0.0, 0.25)])
    assert O.krige(c, v, m, np.array([[0.0, 0.0]]))["value"][0] > 5.0


def test_neighborhood_limits_apply():
    # kriging.rs:1404-1420: nothing within the radius is NoNeighbors; a datum
    # is reproduced
    c, v = sample_data()
    r = O.krige(c, v, sph_model(), np.array([[0.5, 0.2], c[0]]), max_neighbors=3, radius=0.001)
    assert r["status"][0] == 5 and np.isnan(r["value"][0])
    assert r["status"][1] == 0 and abs(r["value"][1] - v[0]) < 1e-8


# ---------------------------------------------- more Vecchia known answers ---
def test_guinness_blocks_partition_the_order_within_group_size():
    # vecchia.rs:2031-2048
    c, _ = O.test_field_2d(4000, 42)
    o, nb, cnt = O.vecchia_plan(c, 30)
    for g in (2, 4, 8, 16):
        covered = 0
        for k0, k1 in O.guinness_blocks(o, nb, cnt, g):
            assert k0 == covered and 0 < k1 - k0 <= g
            covered = k1
        assert covered == len(c)


def test_mle_full_conditioning_is_exact_optimum():
    # vecchia.rs:2228-2259
    c, v = O.test_field_2d(28, 5)
    full = len(c) - 1
    x, f, _ = O.vecchia_mle_bfgs(c, v, "exponential", full)
    nug, sill, rng_ = x[0] ** 2, math.exp(x[1]), math.exp(x[2])
    assert sill > 0 and rng_ > 0 and nug >= 0
    for fn_, fp, fr in ((1.0, 0.7, 1.0), (1.0, 1.4, 1.0), (1.0, 1.0, 0.7), (1.0, 1.0, 1.4),
                        (3.0, 1.0, 1.0)):
        pert = VariogramModel(max(nug * fn_, 1e-9), [Structure("exponential", sill * fp, rng_ * fr)])
        assert -f >= O.vecchia_loglik(c, v, pert, full) - 1e-6


def test_mle_beats_a_wrong_model():
    # vecchia.rs:2261-2270
    c, v = O.test_field_2d(60, 9)
    _, f, _ = O.vecchia_mle_bfgs(c, v, "exponential", 12)
    wrong = VariogramModel(0.5, [Structure("exponential", 0.1, 5.0)])
    assert -f > O.vecchia_loglik(c, v, wrong, 15)


def test_semi_analytical_se_matches_the_full_finite_difference_reference():
    # vecchia.rs:2727-2755 (with nll_hessian_se_reference, :2739-2799)
    c, v = O.test_field_2d(80, 17)
    o, nb, cnt = O.vecchia_plan(c, 10)
    theta = [0.08, 0.9, 18.0]

    def nll(p):
        if p[1] <= 0 or p[2] <= 0 or p[0] < 0:
            return math.inf
        mdl = VariogramModel(p[0], [Structure("matern15", p[1], p[2])])
        return -O.vecchia_loglik_plan(c, v, mdl, o, nb, cnt)

    h = [max(abs(t) * 1e-3, 1e-5) for t in theta]
    f0 = nll(theta)
    hess = np.zeros((3, 3))
    for i in range(3):
        tp, tm = list(theta), list(theta)
        tp[i] += h[i]
        tm[i] -= h[i]
        hess[i, i] = (nll(tp) - 2 * f0 + nll(tm)) / (h[i] * h[i])
        for j in range(i + 1, 3):
            q = []
            for si, sj in ((1, 1), (1, -1), (-1, 1), (-1, -1)):
                t = list(theta)
                t[i] += si * h[i]
                t[j] += sj * h[j]
                q.append(nll(t))
            hess[i, j] = hess[j, i] = (q[0] - q[1] - q[2] + q[3]) / (4 * h[i] * h[j])
    diag = [O.lu_solve(hess, np.eye(3)[i])[i] for i in range(3)]
    ref = [math.sqrt(d) if d > 0 else math.nan for d in diag]
    new = O.vecchia_param_se(c, v, "matern15", *theta, 10)
    for a, b in zip(new, ref):
        if math.isnan(b):
            assert math.isnan(a)
        else:
            assert abs(a - b) < 1e-3 * max(b, 1.0)


# --------------------------------------------------- tests/three_d.rs ---------
def test_universal_kriging_3d_reproduces_drift():
    # tests/three_d.rs:77-110
    c = np.array([[i * 10.0, j * 10.0, l * 5.0] for i in range(4) for j in range(4)
                  for l in range(3)])
    v = 1.0 + 0.2 * c[:, 0] - 0.1 * c[:, 1] + 0.5 * c[:, 2]
    m = VariogramModel(0.05, [Structure("exponential", 1.0, 30.0)])
    t = np.array([[15.0, 25.0, 7.5]])
    r = O.krige(c, v, m, t, method="universal", degree=1)
    assert abs(r["value"][0] - (1.0 + 0.2 * 15.0 - 0.1 * 25.0 + 0.5 * 7.5)) < 1e-7


def test_vertical_anisotropy_shortens_z_range():
    # tests/three_d.rs:112-134
    m = VariogramModel(0.0, [Structure("spherical", 1.0, 100.0, Anisotropy(0.0, 1.0, 0.25))])
    assert abs(O.gamma_dh(m, [0.0, 100.0, 0.0]) - 1.0) < 1e-12
    assert abs(O.gamma_dh(m, [0.0, 0.0, 25.0]) - 1.0) < 1e-12
    assert O.gamma_dh(m, [0.0, 0.0, 10.0]) > O.gamma_dh(m, [0.0, 10.0, 0.0])


def test_block_kriging_3d_uses_z_separation():
    # tests/three_d.rs:219-254
    c, v = O.test_field_3d(100, 13)
    m = VariogramModel(0.05, [Structure("spherical", 1.0, 30.0)])
    ctr = np.array([[42.0, 37.0, 18.0]])
    block = O.krige_block(c, v, m, ctr, [[0.0, 0.0, 0.0]])
    point = O.krige(c, v, m, ctr)
    assert abs(block["value"][0] - point["value"][0]) < 1e-10
    assert abs(block["variance"][0] - (point["variance"][0] - m.nugget)) < 1e-10
    deg = O.krige_block(c, v, m, ctr, [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]])
    ver = O.krige_block(c, v, m, ctr, [[0.0, 0.0, -5.0], [0.0, 0.0, 5.0]])
    assert abs(ver["value"][0] - deg["value"][0]) > 1e-6 and ver["variance"][0] >= 0.0


# ------------------------------------------- validation.rs / tuning.rs -------
def _fold_assignment(n, k, seed):
    # validation.rs:201-213 (rng.rs shuffle: Fisher-Yates from the end)
    order = np.arange(n)
    u = O.rng_u64(seed, n)
    for idx, i in enumerate(range(n - 1, 0, -1)):
        j = int(u[idx] % np.uint64(i + 1))
        order[i], order[j] = order[j], order[i]
    fold_of = np.empty(n, dtype=int)
    fold_of[order] = np.arange(n) % k
    return fold_of


def test_k_equals_n_matches_leave_one_out_and_folds_are_balanced():
    # validation.rs:1005-1037
    from geostat_rs.api import CvResult
    m = VariogramModel(0.01, [Structure("spherical", 1.0, 50.0)])
    c, v = _smooth_field(40, 5)
    fo = _fold_assignment(40, 40, 123)
    assert sorted(fo) == list(range(40))
    kf = _oracle_fold_cv(c, v, m, fo)
    loo = _oracle_fold_cv(c, v, m, np.arange(40))
    assert np.max(np.abs(kf[0] - loo[0])) < 1e-12 and np.max(np.abs(kf[1] - loo[1])) < 1e-12
    c, v = _smooth_field(53, 8)
    fo = _fold_assignment(53, 5, 42)
    assert np.array_equal(fo, _fold_assignment(53, 5, 42))
    sizes = np.bincount(fo)
    assert sizes.sum() == 53 and sizes.max() - sizes.min() <= 1
    assert CvResult(v, *_oracle_fold_cv(c, v, m, fo)).vecv() > 50.0


def test_tunes_kriging_neighbors():
    # tuning.rs:172-188 with tuning.rs:97-125 (the best leave-one-out VEcv)
    from geostat_rs.api import CvResult
    # tuning.rs:133-144 field(120, 9) draws the same stream as vecchia.rs's
    # field (x, y uniform, then a normal, per point); only the signal differs
    c, v = O.test_field_2d(120, 9)
    noise = v - np.sin(c[:, 0] / 25.0) - np.cos(c[:, 1] / 30.0)
    v = np.sin(c[:, 0] / 20.0) + np.cos(c[:, 1] / 25.0) + noise
    m = VariogramModel(0.02, [Structure("spherical", 1.0, 40.0)])
    trace = []
    for k in (4, 8, 16, 32):
        pred = np.empty(120)
        var = np.empty(120)
        for i in range(120):
            keep = np.arange(120) != i
            r = O.krige(c[keep], v[keep], m, c[i:i + 1], max_neighbors=k)
            pred[i], var[i] = r["value"][0], r["variance"][0]
        trace.append((k, CvResult(v, pred, var).vecv()))
    best = max(trace, key=lambda kv: kv[1])
    assert best[0] in (4, 8, 16, 32) and np.isfinite(best[1])


# ------------------------------------------------------ variogram/model.rs ---
_GPU_KINDS = ("spherical", "exponential", "gaussian", "matern15", "matern25")


def test_path_models_bounded_and_monotone_to_sill():
    # variogram/model.rs all_models_bounded_and_monotone_to_sill (the kinds
    # of the path)
    for kind in _GPU_KINDS:
        m = VariogramModel(0.0, [Structure(kind, 2.0, 50.0)])
        prev = 0.0
        for i in range(1, 101):
            g = O.gamma_dh(m, [i * 5.0, 0.0])
            assert prev - 1e-12 <= g <= 2.0 + 1e-12, kind
            prev = g
        assert O.gamma_dh(m, [5000.0, 0.0]) > 1.99, kind


def test_anisotropy_stretches_minor_axis_and_zonal_ratio():
    # variogram/model.rs anisotropy_stretches_minor_axis,
    # zonal_anisotropy_ratio_above_one
    m = VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 100.0, 0.0, 0.5)])
    assert abs(O.gamma_dh(m, [0.0, 100.0]) - 1.0) < 1e-12
    assert O.gamma_dh(m, [0.0, 50.0]) < 1.0 - 1e-6
    assert abs(O.gamma_dh(m, [50.0, 0.0]) - 1.0) < 1e-12
    assert O.gamma_dh(m, [30.0, 0.0]) > O.gamma_dh(m, [0.0, 30.0])
    iso = VariogramModel(0.1, [Structure("exponential", 0.9, 40.0)])
    assert abs(O.gamma_dh(iso, [3.0, 4.0]) - O.gamma_dh(iso, [5.0, 0.0])) < 1e-12
    z = VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 50.0, 0.0, 2.0)])
    assert abs(O.gamma_dh(z, [0.0, 50.0]) - 1.0) < 1e-12
    assert abs(O.gamma_dh(z, [100.0, 0.0]) - 1.0) < 1e-12
    assert O.gamma_dh(z, [50.0, 0.0]) < 1.0 - 1e-6
    assert O.gamma_dh(z, [30.0, 0.0]) < O.gamma_dh(z, [0.0, 30.0])
    mir = VariogramModel(0.0, [Structure.with_anisotropy("spherical", 1.0, 100.0, 90.0, 0.5)])
    for dh in ([10.0, 20.0], [-35.0, 12.0], [60.0, -5.0]):
        assert abs(O.gamma_dh(z, dh) - O.gamma_dh(mir, dh)) < 1e-12


def test_rotation_3d_reduces_to_2d_style_when_dip_and_rake_are_zero():
    # variogram/model.rs rotation_3d_reduces_to_2d_style_when_dip_and_rake_are_zero
    full = VariogramModel(0.05, [Structure.with_rotation("exponential", 0.9, 80.0, 55.0, 0.0,
                                                         0.0, 0.4, 0.6)])
    az = math.radians(55.0)
    s, c = math.sin(az), math.cos(az)
    for x, y, zz in ((10.0, 20.0, 5.0), (-30.0, 15.0, -8.0), (40.0, -25.0, 0.0)):
        hm, hn, hz = x * s + y * c, (x * c - y * s) / 0.4, zz / 0.6
        old = 0.05 + 0.9 * (1.0 - math.exp(-math.sqrt(hm * hm + hn * hn + hz * hz) / 80.0))
        assert abs(old - O.gamma_dh(full, [x, y, zz])) < 1e-12
