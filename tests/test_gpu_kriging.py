"""GPU parity of moving-neighbourhood kriging against the FP64 oracle.

Every test calls the CUDA library through its C ABI (geostat_rs) and checks
neighbour sets bit-exactly and estimates/variances within the tolerance of
tests/gpu_common.py, for both the mixed-precision and the plain FP64 paths.
"""
import numpy as np
import pytest

import pyoracle as O
import geostat_rs as G
import gs_workload as W
from geostat_rs.model import Anisotropy, Structure, VariogramModel
from gpu_common import (assert_close, sph200_model, rotated_3d_model, clustered_matern_model, clustered_points,
                        max_rel, smooth_values, uniform_points)

pytestmark = pytest.mark.gpu


def run_both(coords, values, model, targets, cfg_kw, oracle_kw=None, kcap=None, drift=None,
             tdrift=None, errors=None, precisions=("mixed", "fp64")):
    ps = G.PointSet(coords, values)
    cfg = G.KrigingConfig(**cfg_kw)
    if drift is not None:
        k = G.Kriging.with_external_drift(ps, model, cfg, drift)
    elif errors is not None:
        k = G.Kriging.with_measurement_error(ps, model, cfg, errors)
    else:
        k = G.Kriging.new(ps, model, cfg)
    okw = dict(method=cfg.method, mean=cfg.mean, degree=cfg.degree,
               max_neighbors=cfg.max_neighbors, min_neighbors=cfg.min_neighbors,
               max_per_octant=cfg.max_per_octant, radius=cfg.search_radius,
               anisotropic_search=cfg.anisotropic_search, drift=drift, target_drift=tdrift,
               measurement_error=errors, kcap=kcap or 0)
    ref = O.krige(coords, values, model, targets, **okw)
    outs = {}
    for prec in precisions:
        if tdrift is not None:
            outs[prec] = k.predict_many_with_drift(targets, tdrift, prec, full=True)
        else:
            outs[prec] = k.predict_many(targets, prec, full=True)
    return k, ref, outs


def check(ref, out, values, sill, tol=1e-9):
    st = out.status & 0x3f
    assert (st == ref["status"].astype(np.uint8)).all()
    vscale = float(np.mean(np.abs(values)))
    rv = assert_close(out.value, ref["value"], vscale, tol, "value")
    rs = assert_close(out.variance, ref["variance"], 1e-3 * sill, tol, "variance")
    return rv, rs


# ------------------------------------------------------------ neighbours --
@pytest.mark.parametrize("dim,n,k", [(2, 2000, 32), (3, 5000, 64), (2, 300, 1), (2, 50, 80)])
def test_knn_neighbour_sets_bit_exact(dim, n, k):
    ext = [1000.0, 1000.0] if dim == 2 else [2000.0, 2000.0, 200.0]
    c = uniform_points(n, dim, 7 + dim, ext)
    v = smooth_values(c)
    t = uniform_points(1500, dim, 99, np.asarray(ext) * 1.1) - 0.05 * np.asarray(ext)
    ref = O.krige(c, v, sph200_model(), t, max_neighbors=k, kcap=min(k, n))
    assert ref["boundary_ties"] == 0
    k_ = G.Kriging.new(G.PointSet(c, v), sph200_model(), G.KrigingConfig(max_neighbors=k))
    idx, cnt = k_.neighbors(t, min(k, n))
    assert (cnt == ref["nb_count"]).all()
    assert (idx == ref["neighbors"]).all()


def _brute_d2(c, t):
    """Squared distances in the reference's operation order
    (((0 + dx0^2) + dx1^2) [+ dx2^2]), no fused multiply-adds."""
    d2 = np.zeros((len(t), len(c)))
    for d in range(c.shape[1]):
        dx = t[:, d:d + 1] - c[None, :, d]
        d2 = d2 + dx * dx
    return d2


def test_lattice_data_boundary_ties():
    """Lattice data points and lattice-aligned targets, where the k-th and
    (k+1)-th candidates often tie exactly.  The reference keeps, among
    candidates tied at the k-th distance, the first its kd-tree traversal met
    (search.rs:15-21 strict <; the traversal order comes from
    select_nth_unstable_by in build_rec, search.rs:102-113); the device
    search keeps the smaller indices.  Away from such ties the sets must be
    identical; at a tie both sets must hold the same squared distances, and
    the device's set must be the (squared distance, index) smallest.  The
    number of tie targets and of targets where the two rules pick different
    points is printed (and recorded in the design notes)."""
    g = np.arange(60) * 10.0
    yy, xx = np.meshgrid(g, g, indexing="ij")
    c = np.stack([xx.ravel(), yy.ravel()], 1)
    v = smooth_values(c)
    k = 16
    q = np.arange(40) * 14.5 + 5.0
    ty, tx = np.meshgrid(q, q, indexing="ij")
    t = np.concatenate([np.stack([tx.ravel(), ty.ravel()], 1),
                        uniform_points(400, 2, 321, [590.0, 590.0])])
    ref = O.krige(c, v, sph200_model(), t, max_neighbors=k, kcap=k)
    kr = G.Kriging.new(G.PointSet(c, v), sph200_model(), G.KrigingConfig(max_neighbors=k))
    idx, cnt = kr.neighbors(t, k)
    assert (cnt == k).all() and (ref["nb_count"] == k).all()
    d2 = _brute_d2(c, t)
    order = np.lexsort((np.broadcast_to(np.arange(len(c)), d2.shape), d2), axis=1)
    srt = np.take_along_axis(d2, order, axis=1)
    tie = srt[:, k - 1] == srt[:, k]
    assert tie.sum() > 100  # the lattice makes boundary ties routine
    assert (idx[~tie] == ref["neighbors"][~tie]).all()
    assert (idx == order[:, :k]).all()  # device: (squared distance, index) order
    gd = np.take_along_axis(d2, idx.astype(np.int64), axis=1)
    od = np.take_along_axis(d2, ref["neighbors"].astype(np.int64), axis=1)
    assert (gd == od).all()  # the same distance classes at every target
    differ = (idx != ref["neighbors"]).any(axis=1)
    print(f"lattice k={k}: {len(t)} targets, {int(tie.sum())} with a boundary tie, "
          f"{int(differ.sum())} where the traversal-order rule keeps other points")
    ok = ~differ & (ref["status"] == 0)
    out = kr.predict_many(t, "mixed", full=True)
    assert_close(out.value[ok], ref["value"][ok], float(np.mean(np.abs(v))), 1e-9, "lattice value")
    assert_close(out.variance[ok], ref["variance"][ok], 1e-3, 1e-9, "lattice variance")


def test_radius_and_octant_neighbour_sets_bit_exact():
    c = clustered_points(20000, 3, extent=10000.0, nblobs=40)
    v = smooth_values(c)
    t = uniform_points(800, 2, 5, [10000.0, 10000.0])
    cases = [dict(max_neighbors=16, search_radius=300.0),
             dict(max_neighbors=64, max_per_octant=16, min_neighbors=4),
             dict(max_per_octant=4),
             dict(max_neighbors=40, max_per_octant=16, search_radius=800.0)]
    for case in cases:
        cfg = G.KrigingConfig(**case)
        kcap = 64
        ref = O.krige(c, v, sph200_model(), t, max_neighbors=cfg.max_neighbors,
                      max_per_octant=cfg.max_per_octant, radius=cfg.search_radius,
                      min_neighbors=cfg.min_neighbors, kcap=kcap)
        kk = G.Kriging.new(G.PointSet(c, v), sph200_model(), cfg)
        idx, cnt = kk.neighbors(t, kcap)
        assert (cnt == ref["nb_count"]).all(), case
        assert (idx == ref["neighbors"]).all(), case


@pytest.mark.parametrize("dim", [2, 3])
def test_anisotropic_search_and_octants_bit_exact(dim):
    ext = [1000.0, 1000.0] if dim == 2 else [1000.0, 1000.0, 300.0]
    c = uniform_points(4000, dim, 21, ext)
    v = smooth_values(c)
    t = uniform_points(600, dim, 22, ext)
    an = Anisotropy(35.0, 0.4, 0.5, 12.0, 7.0)
    for case in (dict(max_neighbors=24, anisotropic_search=an),
                 dict(max_neighbors=32, max_per_octant=6, anisotropic_search=an),
                 dict(max_neighbors=20, search_radius=120.0, anisotropic_search=an)):
        cfg = G.KrigingConfig(**case)
        ref = O.krige(c, v, sph200_model(), t, max_neighbors=cfg.max_neighbors,
                      max_per_octant=cfg.max_per_octant, radius=cfg.search_radius,
                      anisotropic_search=an, kcap=32)
        kk = G.Kriging.new(G.PointSet(c, v), sph200_model(), cfg)
        idx, cnt = kk.neighbors(t, 32)
        assert (cnt == ref["nb_count"]).all(), case
        assert (idx == ref["neighbors"]).all(), case


# ---------------------------------------------------- estimates / variances --
def test_config1_ordinary_kriging_full_size():
    """2-D OK: n=2000 in [0,1000]^2, nugget 0.1 + Sph(1, 200), 100x100 grid, n_max=32."""
    c = uniform_points(2000, 2, 2024, [1000.0, 1000.0])
    m = sph200_model()
    v = 10.0 + W.rff_field(c, VariogramModel(0.1, [Structure("exponential", 1.0, 200.0 / 3)]),
                           2048, 11)
    t = O.grid_centers([0, 0], [1000, 1000], [100, 100])
    k, ref, outs = run_both(c, v, m, t, dict(max_neighbors=32))
    for prec, out in outs.items():
        check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-11)
    # grid entry point == explicit targets
    gv, gvar = k.predict_grid([0, 0], [1000, 1000], [100, 100])
    assert np.array_equal(gv, outs["mixed"].value)


@pytest.mark.parametrize("kind", ["spherical", "exponential", "gaussian", "matern15", "matern25"])
def test_kinds_2d(kind):
    c = uniform_points(1500, 2, 31, [100.0, 100.0])
    v = smooth_values(c)
    m = VariogramModel(0.05, [Structure(kind, 1.0, 25.0)])
    t = uniform_points(700, 2, 32, [100.0, 100.0])
    _, ref, outs = run_both(c, v, m, t, dict(max_neighbors=24))
    for prec, out in outs.items():
        check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-10)


def test_config2_shape_3d_nested_rotated():
    """3-D OK with nugget + rotated Sph(300/150/40, az 30, dip 10) + Exp(800), n_max=64."""
    c = uniform_points(20000, 3, 5, [2000.0, 2000.0, 200.0])
    m = rotated_3d_model()
    v = W.rff_field(c, m, 1024, 3)
    t = uniform_points(3000, 3, 6, [2000.0, 2000.0, 200.0])
    _, ref, outs = run_both(c, v, m, t, dict(max_neighbors=64))
    for prec, out in outs.items():
        check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-10)


def _ok_condition(c, model, nb, cnt):
    """2-norm condition number of each target's ordinary-kriging matrix
    [C 1; 1^T 0] (kriging.rs:527-567) over its neighbours, from the oracle's
    gamma_dh."""
    c0 = model.total_sill()
    out = np.empty(len(cnt))
    for t in range(len(cnt)):
        ids = nb[t, :cnt[t]]
        n = len(ids)
        a = np.zeros((n + 1, n + 1))
        for i in range(n):
            for j in range(i, n):
                g = O.gamma_dh(model, c[ids[i]] - c[ids[j]])
                a[i, j] = a[j, i] = c0 - g
        a[:n, n] = a[n, :n] = 1.0
        out[t] = np.linalg.cond(a)
    return out


def test_ill_conditioned_gaussian_goes_to_fp64():
    """Gaussian without nugget: cond(A) ~ 1e10 and beyond, out of reach of an
    FP32 factorisation.  The mixed kernel must hand such systems to the FP64
    tiers (status bit 0x40, statuses otherwise exact).  Two backward-stable
    FP64 solvers of the same system (the bordered LDL^T tier and the plain
    FP64 build's partial-pivoting LU) agree only to about cond(A) * 2^-53, and
    so do the FP64 build and the oracle (their exp differs in the last bit);
    the test therefore compares the mixed path with the FP64 build per target
    within max(1e-9, 8 cond(A) 2^-53) relative, and the FP64 build with the
    oracle within the same bound.  Measured on a GB300: mixed vs FP64 build
    2.3e-7 (values), 8e-11 (variances); FP64 build vs oracle 3.9e-7."""
    c = uniform_points(600, 2, 33, [100.0, 100.0])
    v = smooth_values(c)
    m = VariogramModel(0.0, [Structure("gaussian", 1.0, 25.0)])
    t = uniform_points(200, 2, 34, [100.0, 100.0])
    k, ref, outs = run_both(c, v, m, t, dict(max_neighbors=16))
    out, f64 = outs["mixed"], outs["fp64"]
    routed = (out.status & 0x40) != 0
    assert routed.sum() > 0
    assert ((out.status & 0x3f) == (f64.status & 0x3f)).all()
    assert ((out.status & 0x3f) == ref["status"].astype(np.uint8)).all()
    ok = ref["status"] == 0
    nb, cnt = k.neighbors(t, 16)
    cond = _ok_condition(c, m, nb, cnt)
    assert np.median(cond[routed]) > 1e8  # the routed systems are the ill-conditioned ones
    bound = np.maximum(1e-9, 8.0 * cond * 2.0 ** -53)
    vs = float(np.mean(np.abs(v)))
    for name, a, b, floor in (("value", out.value, f64.value, vs),
                              ("variance", out.variance, f64.variance, 1e-3),
                              ("value vs oracle", f64.value, ref["value"], vs),
                              ("variance vs oracle", f64.variance, ref["variance"], 1e-3)):
        rel = np.abs(a - b)[ok] / np.maximum(np.abs(b), floor)[ok]
        assert (rel <= bound[ok]).all(), f"{name}: worst {np.max(rel / bound[ok]):.2f} x bound"
    # well-conditioned targets (none routed) meet the 1e-9 bar outright
    well = ok & (cond < 1e6)
    if well.any():
        assert_close(out.value[well], f64.value[well], vs, 1e-9, "well-conditioned value")


@pytest.mark.parametrize("method,deg", [("simple", 1), ("universal", 1), ("universal", 2)])
def test_methods_2d_and_3d(method, deg):
    for dim in (2, 3):
        ext = [500.0] * dim
        c = uniform_points(3000, dim, 40 + dim, ext)
        v = smooth_values(c) + (0.01 * c[:, 0] if method == "universal" else 0.0)
        m = VariogramModel(0.02, [Structure("exponential", 0.8, 120.0),
                                  Structure("spherical", 0.2, 300.0)])
        t = uniform_points(500, dim, 50 + dim, ext)
        kw = dict(method=method, degree=deg, max_neighbors=30)
        if method == "simple":
            kw["mean"] = float(np.mean(v))
        _, ref, outs = run_both(c, v, m, t, kw)
        for prec, out in outs.items():
            check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-10)
        if method != "simple":
            assert_close(outs["mixed"].lagrange, ref["lagrange"], 1.0, 1e-9, "lagrange")


def test_external_drift_and_measurement_error():
    c = uniform_points(2500, 2, 61, [1000.0, 1000.0])
    cov = O.rng_uniform(62, 2500)
    v = smooth_values(c) + 2.0 * cov
    m = clustered_matern_model()
    t = uniform_points(400, 2, 63, [1000.0, 1000.0])
    tc = O.rng_uniform(64, 400).reshape(-1, 1)
    _, ref, outs = run_both(c, v, m, t, dict(method="external_drift", n_vars=1, max_neighbors=32),
                            drift=cov.reshape(-1, 1), tdrift=tc)
    for prec, out in outs.items():
        check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-10)
    err = 0.05 * O.rng_uniform(65, 2500)
    _, ref, outs = run_both(c, v, sph200_model(), t, dict(max_neighbors=20), errors=err)
    for prec, out in outs.items():
        check(ref, out, v, 1.1, 1e-9 if prec == "mixed" else 1e-10)


def test_octant_uneven_systems_clustered():
    """Octant search on clustered data: systems of 4..64 neighbours in one launch."""
    c = clustered_points(30000, 9, extent=10000.0, nblobs=60)
    m = clustered_matern_model()
    v = W.rff_field(c, m, 512, 4)
    t = uniform_points(1500, 2, 10, [10000.0, 10000.0])
    _, ref, outs = run_both(c, v, m, t, dict(max_neighbors=64, max_per_octant=16,
                                             min_neighbors=4))
    counts = ref["nb_count"]
    assert counts.min() < 64 <= counts.max()
    for prec, out in outs.items():
        check(ref, out, v, m.total_sill(), 1e-9 if prec == "mixed" else 1e-10)


# ---------------------------------------------- the reference's known answers --
def sample():
    c = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0], [0.4, 0.6]])
    v = np.array([1.0, 2.0, 1.5, 2.5, 1.7])
    return c, v, VariogramModel(0.05, [Structure("spherical", 0.95, 2.0)])


def test_reference_known_answers_on_gpu():
    c, v, m = sample()
    # kriging.rs:1205 exact at data (global neighbourhood)
    pv, pvar = G.Kriging.new(G.PointSet(c, v), m).predict_many(c)
    assert np.max(np.abs(pv - v)) < 1e-8 and np.max(pvar) < 1e-8
    # kriging.rs:1371 SK far field
    sk = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig("simple", mean=1.74))
    fv, fvar = sk.predict_many(np.array([[1e6, 1e6]]))
    assert abs(fv[0] - 1.74) < 1e-9 and abs(fvar[0] - m.total_sill()) < 1e-9
    # kriging.rs:1570 global == moving at k = n
    t = np.array([[0.3, 0.3], [0.9, 0.1], [2.0, 2.0]])
    g = G.Kriging.new(G.PointSet(c, v), m).predict_many(t)
    l = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(max_neighbors=5)).predict_many(t)
    assert np.max(np.abs(g[0] - l[0])) < 1e-12 and np.max(np.abs(g[1] - l[1])) < 1e-12
    # kriging.rs:1385 UK reproduces a linear drift
    cu = np.array([[i, j] for i in range(4) for j in range(4)], float)
    vu = 2.0 + 3.0 * cu[:, 0] - cu[:, 1]
    tu = np.array([[1.5, 1.5], [5.0, 2.0]])
    uv, _ = G.Kriging.new(G.PointSet(cu, vu), m, G.KrigingConfig("universal")).predict_many(tu)
    assert np.max(np.abs(uv - (2 + 3 * tu[:, 0] - tu[:, 1]))) < 1e-7
    # kriging.rs:960 octant balancing
    co = np.array([[1.0, 0.1], [1.1, -0.1], [1.2, 0.2], [1.3, -0.2], [1.4, 0.05],
                   [-2.0, 0.5], [-2.0, -0.5], [0.5, -2.0], [0.5, 2.0]])
    vo = np.array([10.0] * 5 + [0.0] * 4)
    near = G.Kriging.new(G.PointSet(co, vo), m, G.KrigingConfig(max_neighbors=4)).predict_many(
        np.zeros((1, 2)))[0][0]
    octn = G.Kriging.new(G.PointSet(co, vo), m, G.KrigingConfig(max_neighbors=4, max_per_octant=1)
                         ).predict_many(np.zeros((1, 2)))[0][0]
    assert near > 9.0 and octn < near - 2.0
    # kriging.rs:913 min_neighbors -> NaN + NoNeighbors status
    kr = G.Kriging.new(G.PointSet(c, v), m, G.KrigingConfig(search_radius=0.75, min_neighbors=3))
    r = kr.predict_many(np.array([[0.5, 0.5], [1.5, 1.5]]), full=True)
    assert r.status[0] == 0 and r.status[1] == 5 and np.isnan(r.value[1])


def test_construction_errors_match_reference():
    c, v, m = sample()
    ps = G.PointSet(c, v)
    with pytest.raises(G.InvalidParameter):
        G.Kriging.new(ps, m, G.KrigingConfig(min_neighbors=0))
    with pytest.raises(G.InvalidParameter):
        G.Kriging.new(ps, m, G.KrigingConfig(max_neighbors=2, min_neighbors=3))
    with pytest.raises(G.InsufficientData):
        G.Kriging.new(ps, m, G.KrigingConfig(min_neighbors=6))
    with pytest.raises(G.InvalidParameter):
        G.Kriging.new(ps, m, G.KrigingConfig(search_radius=-1.0))
    with pytest.raises(G.InvalidParameter):
        G.Kriging.new(ps, m, G.KrigingConfig("universal", degree=3))
    with pytest.raises(G.InvalidParameter):
        G.Kriging.new(ps, m, G.KrigingConfig("external_drift", n_vars=1))
    dup = G.PointSet(np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 0.0], [0.0, 1.0]]),
                     np.array([1.0, 2.0, 2.1, 1.5]))
    with pytest.raises(G.DuplicatePoints, match="1 and 2"):
        G.Kriging.new(dup, m)


def test_python_binding_mirror_matches_oracle():
    c = uniform_points(800, 2, 71, [100.0, 100.0])
    v = smooth_values(c)
    m = VariogramModel(0.05, [Structure("exponential", 0.95, 20.0)])
    tx, ty = np.linspace(1, 99, 50), np.linspace(99, 1, 50)
    pv, pvar = G.krige(c[:, 0], c[:, 1], v, m, tx, ty, max_neighbors=16, octant=4)
    ref = O.krige(c, v, m, np.stack([tx, ty], 1), max_neighbors=16, max_per_octant=4)
    assert_close(pv, ref["value"], 10.0, 1e-9, "krige")
    gv, gvar = G.krige_grid(c[:, 0], c[:, 1], v, m, (0.0, 0.0, 100.0, 50.0), 20, 10,
                            max_neighbors=12)
    gref = O.krige(c, v, m, O.grid_centers([0, 0], [100, 50], [20, 10]), max_neighbors=12)
    assert_close(gv, gref["value"], 10.0, 1e-9, "krige_grid")
    c3 = uniform_points(800, 3, 72, [100.0, 100.0, 30.0])
    v3 = smooth_values(c3)
    t3 = uniform_points(60, 3, 73, [100.0, 100.0, 30.0])
    pv3, _ = G.krige_3d(c3[:, 0], c3[:, 1], c3[:, 2], v3, m, t3[:, 0], t3[:, 1], t3[:, 2],
                        method="universal", max_neighbors=20)
    ref3 = O.krige(c3, v3, m, t3, method="universal", max_neighbors=20)
    assert_close(pv3, ref3["value"], 10.0, 1e-9, "krige_3d")


# ------------------------------------------------ consecutive grid targets --
# A block solves consecutive targets and keeps the matrix entries of the
# neighbours they share; grid targets (x fastest) exercise that reuse with
# neighbour sets that change by a few points per step, and octant / radius
# searches make the neighbour count vary from target to target.
@pytest.mark.parametrize("case", [
    dict(max_neighbors=64),
    dict(max_neighbors=24, method="universal", degree=1),
    dict(max_neighbors=48, method="universal", degree=2),
    dict(max_neighbors=64, max_per_octant=16, min_neighbors=4),
    dict(max_neighbors=40, search_radius=45.0, min_neighbors=2),
    dict(max_neighbors=30, method="simple", mean=10.0),
])
def test_grid_targets_reuse_shared_neighbours(case):
    c = uniform_points(6000, 2, 404, [1000.0, 1000.0])
    m = VariogramModel(0.05, [Structure.with_anisotropy("spherical", 0.7, 150.0, 30.0, 0.5),
                              Structure("exponential", 0.25, 400.0)])
    v = 10.0 + W.rff_field(c, m, 1024, 12)
    t = O.grid_centers([100, 100], [900, 900], [120, 40])
    k, ref, outs = run_both(c, v, m, t, case, precisions=("mixed",))
    check(ref, outs["mixed"], v, m.total_sill())


def test_grid_targets_reuse_3d_and_external_drift():
    c = uniform_points(8000, 3, 405, [600.0, 600.0, 60.0])
    m = rotated_3d_model()
    v = W.rff_field(c, m, 1024, 13)
    t = O.grid_centers([50, 50, 5], [550, 550, 55], [64, 8, 4])
    k, ref, outs = run_both(c, v, m, t, dict(max_neighbors=64), precisions=("mixed",))
    check(ref, outs["mixed"], v, m.total_sill())
    c2 = uniform_points(5000, 2, 406, [1000.0, 1000.0])
    m2 = sph200_model()
    drift = 0.01 * c2[:, 0:1] + O.rng_uniform(407, 5000).reshape(-1, 1)
    v2 = 3.0 * drift[:, 0] + smooth_values(c2)
    t2 = O.grid_centers([100, 100], [900, 900], [100, 20])
    tdrift = 0.01 * t2[:, 0:1] + 0.5
    k2, ref2, outs2 = run_both(c2, v2, m2, t2, dict(max_neighbors=32, method="external_drift",
                                                    n_vars=1),
                               drift=drift, tdrift=tdrift, precisions=("mixed",))
    check(ref2, outs2["mixed"], v2, m2.total_sill())
